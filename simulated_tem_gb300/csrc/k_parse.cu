// The Atoms block of a LAMMPS data file parsed on the GPU (src/Lib_XYZFiles.f90:1108-1117,
// input_lammps: for every atom a list-directed read of id, type, x, y, z; the rest of the
// line is ignored).
//
// The block's bytes are in device memory.  Line starts: each block of threads owns a
// 64 KB segment and counts its newlines (16-byte loads, coalesced); an exclusive scan over
// the segments gives each segment's first line number; each segment then writes the starts
// of its lines (the byte after each newline) in order, 4 KB per step with a block-wide scan
// of the threads' newline counts.  Then one thread per atom line reads five tokens:
// two integers and three reals, each correctly rounded (parse_number.cuh), separated by
// blanks or commas.  A line with fewer than five tokens, a malformed token or a number
// outside the exact parser's range records its line number (the smallest such line wins)
// and nothing is guessed.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "parse_number.cuh"

namespace stem {
namespace {

constexpr int kSeg = 65536;   // bytes per segment (one block)
constexpr int kChunk = 4096;  // bytes per block-wide step: 256 threads x 16 bytes

// newlines among the 16 bytes at t[i0, i0 + 16) (bytes at or past n are not newlines),
// as a bit mask (bit k: byte i0 + k)
__device__ __forceinline__ unsigned newline_mask(const char* __restrict__ t, int64_t n, int64_t i0) {
  unsigned m = 0;
  if (i0 + 16 <= n && ((uintptr_t)(t + i0) & 15) == 0) {  // a caller's buffer may start unaligned
    const uint4 v = *reinterpret_cast<const uint4*>(t + i0);
    const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (((w[k >> 2] >> (8 * (k & 3))) & 0xFFu) == (unsigned)'\n') m |= 1u << k;
  } else {  // the end of the text, or an unaligned buffer
    for (int k = 0; k < 16 && i0 + k < n; ++k)
      if (t[i0 + k] == '\n') m |= 1u << k;
  }
  return m;
}

__global__ void __launch_bounds__(256) k_count_lines(const char* __restrict__ t, int64_t n, int64_t nseg,
                                                     long long* __restrict__ seg_count) {
  __shared__ int part[8];
  for (int64_t sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    int c = 0;
    for (int ch = 0; ch < kSeg / kChunk; ++ch) {
      const int64_t i0 = sg * kSeg + (int64_t)ch * kChunk + 16 * threadIdx.x;
      if (i0 < n) c += __popc(newline_mask(t, n, i0));
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long s = 0;
      for (int w = 0; w < 8; ++w) s += part[w];
      seg_count[sg] = s;
    }
    __syncthreads();
  }
}

// exclusive scan of nseg counts in place (one block)
__global__ void __launch_bounds__(1024) k_scan_segments(long long* __restrict__ v, int64_t nseg) {
  __shared__ long long buf[1024];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t off = 0; off < nseg; off += 1024) {
    const int64_t i = off + threadIdx.x;
    const long long x = i < nseg ? v[i] : 0;
    buf[threadIdx.x] = x;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
      const long long a = threadIdx.x >= d ? buf[threadIdx.x - d] : 0;
      __syncthreads();
      buf[threadIdx.x] += a;
      __syncthreads();
    }
    if (i < nseg) v[i] = carry + buf[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}

// starts[k] = byte offset of line k (k < n_lines; the rest stay -1); line 0 starts at 0.
// Per 4 KB step every thread holds the newline mask of its 16 bytes; a block-wide scan of
// the counts gives each newline its line number.
__global__ void __launch_bounds__(256) k_line_starts(const char* __restrict__ t, int64_t n, int64_t nseg,
                                                     const long long* __restrict__ seg_base, int64_t n_lines,
                                                     long long* __restrict__ starts) {
  __shared__ int wsum[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    long long base = seg_base[sg];  // newlines before this step
    for (int ch = 0; ch < kSeg / kChunk; ++ch) {
      const int64_t c0 = sg * kSeg + (int64_t)ch * kChunk;
      if (c0 >= n) break;  // block-uniform
      const int64_t i0 = c0 + 16 * threadIdx.x;
      const unsigned m = i0 < n ? newline_mask(t, n, i0) : 0u;
      const int c = __popc(m);
      int incl = c;  // inclusive warp scan
      for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += a;
      }
      if (lane == 31) wsum[warp] = incl;
      __syncthreads();
      int woff = 0, total = 0;
      for (int w = 0; w < 8; ++w) {
        if (w < warp) woff += wsum[w];
        total += wsum[w];
      }
      long long k = base + woff + incl - c + 1;  // the line the first newline here starts
      for (unsigned mm = m; mm; mm &= mm - 1, ++k)
        if (k < n_lines) starts[k] = i0 + __ffs(mm);  // the byte after the newline
      base += total;
      __syncthreads();  // wsum is rewritten by the next step
    }
    if (sg == 0 && threadIdx.x == 0 && n_lines > 0) starts[0] = 0;
  }
}

__device__ __forceinline__ const char* skip_blanks(const char* p, const char* end) {
  while (p < end && pn::is_blank(*p)) ++p;
  return p;
}

__device__ __forceinline__ bool token_end(const char* p, const char* end) {
  return p >= end || pn::is_blank(*p) || *p == '\n';
}

__global__ void __launch_bounds__(256) k_parse_atoms(const char* __restrict__ t, int64_t n,
                                                     const long long* __restrict__ starts, int64_t n_atoms,
                                                     double* __restrict__ x, int64_t ldx, int* __restrict__ types,
                                                     unsigned long long* __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_atoms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const char* end = t + n;
    const long long st = starts[i];
    if (st < 0 || st > n) {  // the block has fewer lines than atoms
      atomicMin(bad, (unsigned long long)i);
      continue;
    }
    const char* p = t + st;
    bool ok = true;
    long long id = 0, ty = 0;
    double v[3] = {0.0, 0.0, 0.0};
    int used = 0;
    p = skip_blanks(p, end);
    ok = pn::parse_int(p, end, id, used) && token_end(p + used, end);
    p += used;
    if (ok) {
      p = skip_blanks(p, end);
      ok = pn::parse_int(p, end, ty, used) && token_end(p + used, end);
      p += used;
    }
    for (int c = 0; c < 3 && ok; ++c) {
      p = skip_blanks(p, end);
      ok = pn::parse_real(p, end, v[c], used) && token_end(p + used, end);
      p += used;
    }
    if (!ok) {
      atomicMin(bad, (unsigned long long)i);
      continue;
    }
    x[i * ldx + 0] = v[0];
    x[i * ldx + 1] = v[1];
    x[i * ldx + 2] = v[2];
    if (types) types[i] = (int)ty;
    (void)id;
  }
}

}  // namespace

int64_t parse_segments(int64_t n_bytes) { return (n_bytes + kSeg - 1) / kSeg; }

cudaError_t launch_parse_atoms(const char* d_text, int64_t n_bytes, int64_t n_atoms, long long* d_seg,
                               long long* d_starts, double* d_x, int64_t ldx, int* d_types,
                               unsigned long long* d_bad, cudaStream_t st) {
  const int64_t nseg = parse_segments(n_bytes);
  if (nseg <= 0 || n_atoms <= 0) return cudaSuccess;
  int grid = (int)(nseg < 8192 ? nseg : 8192);
  cudaMemsetAsync(d_starts, 0xFF, (size_t)n_atoms * sizeof(long long), st);  // -1: no such line
  cudaMemsetAsync(d_bad, 0xFF, sizeof(unsigned long long), st);
  k_count_lines<<<grid, 256, 0, st>>>(d_text, n_bytes, nseg, d_seg);
  k_scan_segments<<<1, 1024, 0, st>>>(d_seg, nseg);
  k_line_starts<<<grid, 256, 0, st>>>(d_text, n_bytes, nseg, d_seg, n_atoms, d_starts);
  const int64_t pb = (n_atoms + 255) / 256;
  k_parse_atoms<<<(int)(pb < 16384 ? pb : 16384), 256, 0, st>>>(d_text, n_bytes, d_starts, n_atoms, d_x, ldx,
                                                                 d_types, d_bad);
  return cudaGetLastError();
}

}  // namespace stem
