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

// The atom lines of an .xyz file (src/Lib_XYZFiles.f90:820-826, input0): `read(uu,*) atom,
// dat(1:nColumns)`.  The species is the token up to a blank, comma, slash or the end of the
// line; character(len=6) keeps its first 6 characters (blank padded): the key is those 6
// bytes.  Then ncols numbers, correctly rounded; the first ncopy go to x.
__global__ void __launch_bounds__(256) k_parse_xyz(const char* __restrict__ t, int64_t n,
                                                   const long long* __restrict__ starts, int64_t n_atoms, int ncols,
                                                   double* __restrict__ x, int64_t ldx, int ncopy,
                                                   unsigned long long* __restrict__ keys,
                                                   unsigned long long* __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_atoms;
       i += (int64_t)gridDim.x * blockDim.x) {
    const char* end = t + n;
    const long long st = starts[i];
    if (st < 0 || st > n) {
      atomicMin(bad, (unsigned long long)i);
      continue;
    }
    const char* p = skip_blanks(t + st, end);
    const char* q = p;
    while (q < end && !pn::is_blank(*q) && *q != '\n' && *q != '/') ++q;
    if (q == p || *p == '\'' || *p == '"') {  // no species (or a quoted one, not read here)
      atomicMin(bad, (unsigned long long)i);
      continue;
    }
    unsigned long long key = 0;
    for (int k = 0; k < 6; ++k) {
      const unsigned char ch = p + k < q ? (unsigned char)p[k] : (unsigned char)' ';
      key |= (unsigned long long)ch << (8 * k);
    }
    p = q;
    bool ok = true;
    for (int c = 0; c < ncols && ok; ++c) {
      p = skip_blanks(p, end);
      double v = 0.0;
      int used = 0;
      ok = pn::parse_real(p, end, v, used) && token_end(p + used, end);
      p += used;
      if (ok && c < ncopy) x[i * ldx + c] = v;
    }
    if (!ok) {
      atomicMin(bad, (unsigned long long)i);
      continue;
    }
    keys[i] = key;
  }
}

// Species numbers in order of first appearance (input0 :829-846).  Block b takes lines
// [b chunk, (b + 1) chunk) in order and records the keys it meets first (at most
// kSpeciesMax; one more marks an overflow); one thread merges the block tables in block
// order; then every line looks its key up (binary search over a sorted copy).
constexpr int kSpeciesMax = 1000;
constexpr int kSpeciesBlocks = 4 * 152;

__global__ void __launch_bounds__(256) k_species_block(const unsigned long long* __restrict__ keys, int64_t n,
                                                       int64_t chunk, unsigned long long* __restrict__ tables) {
  __shared__ unsigned long long sk[256];
  __shared__ unsigned long long tab[kSpeciesMax];
  __shared__ int cnt, last;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = lo + chunk < n ? lo + chunk : n;
  if (threadIdx.x == 0) cnt = 0, last = -1;
  __syncthreads();
  for (int64_t base = lo; base < hi; base += 256) {
    const int64_t i = base + threadIdx.x;
    const unsigned long long mine = i < hi ? keys[i] : 0ull;
    sk[threadIdx.x] = mine;
    // a step that only repeats the last species seen (one species, or atoms grouped by
    // species) adds nothing to the table
    const int lk = last;
    if (__syncthreads_and(lk >= 0 && (i >= hi || mine == tab[lk]))) continue;
    if (threadIdx.x == 0) {
      const int m = (int)(hi - base < 256 ? hi - base : 256);
      for (int k = 0; k < m && cnt <= kSpeciesMax; ++k) {
        const unsigned long long key = sk[k];
        if (last >= 0 && tab[last] == key) continue;  // runs of one species
        int f = -1;
        for (int j = 0; j < cnt; ++j)
          if (tab[j] == key) {
            f = j;
            break;
          }
        if (f < 0) {
          if (cnt == kSpeciesMax) {
            cnt = kSpeciesMax + 1;
            break;
          }
          f = cnt;
          tab[cnt++] = key;
        }
        last = f;
      }
    }
    __syncthreads();
  }
  unsigned long long* out = tables + (size_t)blockIdx.x * (kSpeciesMax + 1);
  const int c = cnt;
  for (int j = threadIdx.x; j < (c < kSpeciesMax ? c : kSpeciesMax); j += blockDim.x) out[1 + j] = tab[j];
  if (threadIdx.x == 0) out[0] = (unsigned long long)c;
}

// table: kSpeciesMax keys in order of first appearance, then the count; sorted keys and
// their numbers after it.  The block tables are staged in shared memory first (when they
// hold at most kStage - kSpeciesMax keys together), so that the serial merge reads no
// global memory.
constexpr int kStage = 4096;

__global__ void __launch_bounds__(1024) k_species_merge(const unsigned long long* __restrict__ tables, int n_blocks,
                                                        unsigned long long* __restrict__ table) {
  __shared__ int counts[kSpeciesBlocks], offs[kSpeciesBlocks + 1];
  __shared__ unsigned long long stage[kStage - kSpeciesMax];
  __shared__ unsigned long long gt[kSpeciesMax];
  for (int b = threadIdx.x; b < n_blocks; b += blockDim.x)
    counts[b] = (int)tables[(size_t)b * (kSpeciesMax + 1)];
  __syncthreads();
  if (threadIdx.x == 0) {
    int o = 0;
    for (int b = 0; b < n_blocks; ++b) {
      offs[b] = o;
      o += counts[b] > kSpeciesMax ? kSpeciesMax + 1 : counts[b];
    }
    offs[n_blocks] = o;
  }
  __syncthreads();
  const bool staged = offs[n_blocks] <= kStage - kSpeciesMax;
  if (staged)
    for (int b = 0; b < n_blocks; ++b) {
      const int cb = counts[b] > kSpeciesMax ? 0 : counts[b];
      for (int j = threadIdx.x; j < cb; j += blockDim.x)
        stage[offs[b] + j] = tables[(size_t)b * (kSpeciesMax + 1) + 1 + j];
    }
  __syncthreads();
  if (threadIdx.x != 0) return;
  unsigned long long* sorted = table + kSpeciesMax + 1;
  unsigned long long* ids = sorted + kSpeciesMax;
  int cnt = 0;
  for (int b = 0; b < n_blocks && cnt <= kSpeciesMax; ++b) {
    const int cb = counts[b];
    if (cb > kSpeciesMax) {
      cnt = kSpeciesMax + 1;
      break;
    }
    for (int j = 0; j < cb; ++j) {
      const unsigned long long key = staged ? stage[offs[b] + j] : tables[(size_t)b * (kSpeciesMax + 1) + 1 + j];
      bool seen = false;
      for (int k = cnt - 1; k >= 0 && !seen; --k) seen = gt[k] == key;
      if (seen) continue;
      if (cnt == kSpeciesMax) {
        cnt = kSpeciesMax + 1;
        break;
      }
      gt[cnt++] = key;
    }
  }
  for (int k = 0; k < cnt && k < kSpeciesMax; ++k) table[k] = gt[k];
  table[kSpeciesMax] = (unsigned long long)cnt;
  if (cnt > kSpeciesMax) return;
  for (int k = 0; k < cnt; ++k) {  // insertion sort of (key, number)
    const unsigned long long key = gt[k];
    int j = k;
    while (j > 0 && sorted[j - 1] > key) {
      sorted[j] = sorted[j - 1];
      ids[j] = ids[j - 1];
      --j;
    }
    sorted[j] = key;
    ids[j] = (unsigned long long)(k + 1);
  }
}

__global__ void __launch_bounds__(256) k_species_assign(const unsigned long long* __restrict__ keys, int64_t n,
                                                        const unsigned long long* __restrict__ table,
                                                        int* __restrict__ types) {
  __shared__ unsigned long long sk[kSpeciesMax];
  __shared__ int sid[kSpeciesMax];
  const int cnt = (int)table[kSpeciesMax];
  if (cnt > kSpeciesMax) return;  // block-uniform
  for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
    sk[j] = table[kSpeciesMax + 1 + j];
    sid[j] = (int)table[2 * kSpeciesMax + 1 + j];
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = keys[i];
    int a = 0, b = cnt - 1, id = 0;
    while (a <= b) {
      const int m = (a + b) >> 1;
      if (sk[m] == key) {
        id = sid[m];
        break;
      }
      if (sk[m] < key) a = m + 1;
      else b = m - 1;
    }
    types[i] = id;
  }
}

// the line starts of n_atoms lines (shared by both readers)
cudaError_t launch_line_starts(const char* d_text, int64_t n_bytes, int64_t n_atoms, long long* d_seg,
                               long long* d_starts, unsigned long long* d_bad, cudaStream_t st) {
  const int64_t nseg = (n_bytes + kSeg - 1) / kSeg;
  const int grid = (int)(nseg < 8192 ? nseg : 8192);
  cudaMemsetAsync(d_starts, 0xFF, (size_t)n_atoms * sizeof(long long), st);  // -1: no such line
  cudaMemsetAsync(d_bad, 0xFF, sizeof(unsigned long long), st);
  k_count_lines<<<grid, 256, 0, st>>>(d_text, n_bytes, nseg, d_seg);
  k_scan_segments<<<1, 1024, 0, st>>>(d_seg, nseg);
  k_line_starts<<<grid, 256, 0, st>>>(d_text, n_bytes, nseg, d_seg, n_atoms, d_starts);
  return cudaGetLastError();
}

}  // namespace

int64_t parse_segments(int64_t n_bytes) { return (n_bytes + kSeg - 1) / kSeg; }

int64_t species_scratch(int64_t n_atoms) {
  (void)n_atoms;
  return (int64_t)kSpeciesBlocks * (kSpeciesMax + 1) + 3 * kSpeciesMax + 1;
}

cudaError_t launch_parse_xyz(const char* d_text, int64_t n_bytes, int64_t n_atoms, int ncols, long long* d_seg,
                             long long* d_starts, double* d_x, int64_t ldx, unsigned long long* d_keys,
                             unsigned long long* d_bad, cudaStream_t st) {
  if (n_bytes <= 0 || n_atoms <= 0) return cudaSuccess;
  cudaError_t e = launch_line_starts(d_text, n_bytes, n_atoms, d_seg, d_starts, d_bad, st);
  if (e != cudaSuccess) return e;
  const int64_t pb = (n_atoms + 255) / 256;
  const int ncopy = (int)(ldx < ncols ? ldx : ncols);
  k_parse_xyz<<<(int)(pb < 16384 ? pb : 16384), 256, 0, st>>>(d_text, n_bytes, d_starts, n_atoms, ncols, d_x, ldx,
                                                              ncopy, d_keys, d_bad);
  return cudaGetLastError();
}

cudaError_t launch_species(const unsigned long long* d_keys, int64_t n, unsigned long long* d_scratch,
                           int32_t* d_types, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  unsigned long long* tables = d_scratch;
  unsigned long long* table = d_scratch + (size_t)kSpeciesBlocks * (kSpeciesMax + 1);
  const int64_t chunk0 = (n + kSpeciesBlocks - 1) / kSpeciesBlocks;
  const int64_t chunk = chunk0 < 256 ? 256 : chunk0;
  const int blocks = (int)((n + chunk - 1) / chunk);
  k_species_block<<<blocks, 256, 0, st>>>(d_keys, n, chunk, tables);
  k_species_merge<<<1, 1024, 0, st>>>(tables, blocks, table);
  if (d_types) {
    const int64_t pb = (n + 255) / 256;
    k_species_assign<<<(int)(pb < 4 * 152 ? pb : 4 * 152), 256, 0, st>>>(d_keys, n, table, d_types);
  }
  return cudaGetLastError();
}

int species_table_offset() { return kSpeciesBlocks * (kSpeciesMax + 1); }

cudaError_t launch_parse_atoms(const char* d_text, int64_t n_bytes, int64_t n_atoms, long long* d_seg,
                               long long* d_starts, double* d_x, int64_t ldx, int* d_types,
                               unsigned long long* d_bad, cudaStream_t st) {
  const int64_t nseg = parse_segments(n_bytes);
  if (nseg <= 0 || n_atoms <= 0) return cudaSuccess;
  cudaError_t e = launch_line_starts(d_text, n_bytes, n_atoms, d_seg, d_starts, d_bad, st);
  if (e != cudaSuccess) return e;
  const int64_t pb = (n_atoms + 255) / 256;
  k_parse_atoms<<<(int)(pb < 16384 ? pb : 16384), 256, 0, st>>>(d_text, n_bytes, d_starts, n_atoms, d_x, ldx,
                                                                 d_types, d_bad);
  return cudaGetLastError();
}

}  // namespace stem
