// K1: findGdotR + link-cell binning as a counting sort.
//
// Follows Lib_DynamicalTwoBeamImaging.f90:1160-1265 (findGdotR) and
// Lib_LinkCell3D.f90:691-748 (add0): for every periodic replica nn and atom jj
//   y = RU (x + Ruvw(nn)) + delta,  z = y - lc_delta,
// the atom is kept when floor(ia z) lies inside the link-cell box; it goes to
// cell floor(ia z) with fractional offset ia z - floor(ia z), and its phase is
// g . y.  The cell assignment is computed in FP64 with explicitly rounded
// operations in the reference's evaluation order, so it is bit-identical to
// the reference's.  An FP32 pass rejects candidates that are far outside the
// box first (the FP64 path only runs near and inside it).
//
// Instead of per-cell arrays grown by doubling, the kept atoms are counted per
// cell, the counts scanned, and the atoms scattered; a per-cell rank by
// candidate index (replica-major, atom order) then restores the reference's
// insertion order, so the result is deterministic.
#include <cuda_runtime.h>

#include "internal.h"

namespace stem {
namespace {

constexpr int kScanBlock = 1024;  // counts per scan block (256 threads x 4)
constexpr double kInv2Pi = 0.15915494309189533577;

// index of the job whose range [base(j), base(j+1)) holds v (bases ascending)
template <typename F>
__device__ __forceinline__ int find_job(int n_jobs, int64_t v, F base) {
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base(mid) <= v)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ double dot3_rn(double a0, double a1, double a2, double b0, double b1, double b2) {
  // (a0*b0 + a1*b1) + a2*b2 with every operation rounded separately
  return __dadd_rn(__dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1)), __dmul_rn(a2, b2));
}

// One thread per candidate (replica nn, atom jj) in the reference's insertion
// order t = nn * N + jj.  kExact: every kept candidate goes through the
// reference's rounded FP64 arithmetic (the FP64 imaging path needs its exact
// fractional offsets).  Otherwise the kept candidates use fused FP64
// multiply-adds, which agree with the reference to a few ulp, and fall back to
// the exact arithmetic whenever a cell coordinate lies within 1e-9 cells of a
// cell face: the cell assignment is bit-identical either way, the offsets and
// the phase agree to ~1e-14.
template <bool kExact>
__global__ void __launch_bounds__(256) k_bin_transform(const BinParams* __restrict__ jobs, int n_jobs,
                                                       int64_t total, int64_t cap, int* __restrict__ counts,
                                                       int* __restrict__ tmp_key, int* __restrict__ tmp_cell,
                                                       int* __restrict__ tmp_slot, double4_32a* __restrict__ tmp_f,
                                                       unsigned long long* __restrict__ counters) {
  const float margin = 2e-3f;  // cells; the FP32 position error is below 1e-4 cells
  for (int64_t tg = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; tg < total;
       tg += (int64_t)gridDim.x * blockDim.x) {
    const int job = n_jobs == 1 ? 0 : find_job(n_jobs, tg, [&](int k) { return jobs[k].cand_base; });
    const BinParams& p = jobs[job];
    const int64_t t = tg - p.cand_base;  // the reference's insertion order within the image
    const int nn = p.n_atoms <= 0x7fffffff && t <= 0x7fffffff ? (int)((unsigned)t / (unsigned)p.n_atoms)
                                                               : (int)(t / p.n_atoms);
    const int64_t jj = t - (int64_t)nn * p.n_atoms;
    const double* xa = p.x + jj * p.ldx;
    const double x0 = xa[0], x1 = xa[1], x2 = xa[2];

    // FP32 reject test
    const float yf0 = (float)x0 + p.Ruvwf[3 * nn + 0];
    const float yf1 = (float)x1 + p.Ruvwf[3 * nn + 1];
    const float yf2 = (float)x2 + p.Ruvwf[3 * nn + 2];
    const float zf0 = p.RUf[0] * yf0 + p.RUf[3] * yf1 + p.RUf[6] * yf2 + p.shiftf[0];
    const float zf1 = p.RUf[1] * yf0 + p.RUf[4] * yf1 + p.RUf[7] * yf2 + p.shiftf[1];
    const float zf2 = p.RUf[2] * yf0 + p.RUf[5] * yf1 + p.RUf[8] * yf2 + p.shiftf[2];
    const float cf0 = zf0 * p.iaf[0], cf1 = zf1 * p.iaf[1], cf2 = zf2 * p.iaf[2];
    bool keep = cf0 >= -margin && cf0 < p.Ex + margin && cf1 >= -margin && cf1 < p.Ey + margin &&
                cf2 >= -margin && cf2 < p.Ez + margin;
    double c0 = 0, c1 = 0, c2 = 0, y0 = 0, y1 = 0, y2 = 0;
    if (keep) {
      const double yy0 = __dadd_rn(x0, p.Ruvw[3 * nn + 0]);
      const double yy1 = __dadd_rn(x1, p.Ruvw[3 * nn + 1]);
      const double yy2 = __dadd_rn(x2, p.Ruvw[3 * nn + 2]);
      bool exact = kExact;
      if (!kExact) {
        y0 = fma(p.RU[6], yy2, fma(p.RU[3], yy1, p.RU[0] * yy0)) + p.delta[0];
        y1 = fma(p.RU[7], yy2, fma(p.RU[4], yy1, p.RU[1] * yy0)) + p.delta[1];
        y2 = fma(p.RU[8], yy2, fma(p.RU[5], yy1, p.RU[2] * yy0)) + p.delta[2];
        c0 = (y0 - p.lc_delta[0]) * p.ia[0];
        c1 = (y1 - p.lc_delta[1]) * p.ia[4];
        c2 = (y2 - p.lc_delta[2]) * p.ia[8];
        const double e = 1e-9;
        const double f0 = c0 - floor(c0), f1 = c1 - floor(c1), f2 = c2 - floor(c2);
        exact = f0 < e || f0 > 1.0 - e || f1 < e || f1 > 1.0 - e || f2 < e || f2 > 1.0 - e;
      }
      if (exact) {
        // the reference's order, every operation rounded separately
        y0 = __dadd_rn(dot3_rn(p.RU[0], p.RU[3], p.RU[6], yy0, yy1, yy2), p.delta[0]);
        y1 = __dadd_rn(dot3_rn(p.RU[1], p.RU[4], p.RU[7], yy0, yy1, yy2), p.delta[1]);
        y2 = __dadd_rn(dot3_rn(p.RU[2], p.RU[5], p.RU[8], yy0, yy1, yy2), p.delta[2]);
        const double z0 = __dsub_rn(y0, p.lc_delta[0]);
        const double z1 = __dsub_rn(y1, p.lc_delta[1]);
        const double z2 = __dsub_rn(y2, p.lc_delta[2]);
        c0 = dot3_rn(p.ia[0], p.ia[3], p.ia[6], z0, z1, z2);
        c1 = dot3_rn(p.ia[1], p.ia[4], p.ia[7], z0, z1, z2);
        c2 = dot3_rn(p.ia[2], p.ia[5], p.ia[8], z0, z1, z2);
      }
      // pointInSupercell: floor(c) in [0, N) on every axis
      keep = c0 >= 0.0 && c0 < (double)p.Ex && c1 >= 0.0 && c1 < (double)p.Ey && c2 >= 0.0 &&
             c2 < (double)p.Ez;
    }
    // warp-aggregated compaction slot
    const unsigned mask = __ballot_sync(__activemask(), keep);
    if (!keep) continue;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&counters[0], (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const int64_t idx = (int64_t)base + __popc(mask & ((1u << lane) - 1));

    const double fl0 = floor(c0), fl1 = floor(c1), fl2 = floor(c2);
    const int cx = (int)fl0, cy = (int)fl1, cz = (int)fl2;
    const int cell = (int)p.cell_base + cx + p.Ex * (cy + p.Ey * cz);
    // consecutive atoms often share a cell: one atomic per cell and warp
    const unsigned same = __match_any_sync(mask, cell);
    const int first = __ffs(same) - 1;
    int slot0 = 0;
    if (lane == first) slot0 = atomicAdd(&counts[cell], __popc(same));
    const int slot = __shfl_sync(same, slot0, first) + __popc(same & ((1u << lane) - 1));
    if (idx >= cap) continue;  // overflow: counted, not stored; the host grows the arrays and retries
    const double gdotr = kExact ? dot3_rn(p.g[0], p.g[1], p.g[2], y0, y1, y2)
                                : fma(p.g[2], y2, fma(p.g[1], y1, p.g[0] * y0));
    tmp_key[idx] = (int)t;
    tmp_cell[idx] = cell;
    tmp_slot[idx] = slot;
    tmp_f[idx] = make_double4_32a(__dsub_rn(c0, fl0), __dsub_rn(c1, fl1), __dsub_rn(c2, fl2), gdotr);
  }
}

// Exclusive scan of the per-cell counts in three passes.
__global__ void __launch_bounds__(256) k_scan_blocks(const int* __restrict__ counts, int64_t n,
                                                     int* __restrict__ block_sums,
                                                     unsigned long long* __restrict__ counters) {
  __shared__ int warp_sums[8];
  __shared__ int warp_max[8];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * 4;
  int s = 0, m = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int v = (base + i < n) ? counts[base + i] : 0;
    s += v;
    m = max(m, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  if ((threadIdx.x & 31) == 0) {
    warp_sums[threadIdx.x >> 5] = s;
    warp_max[threadIdx.x >> 5] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0, mm = 0;
    for (int w = 0; w < 8; ++w) {
      t += warp_sums[w];
      mm = max(mm, warp_max[w]);
    }
    block_sums[blockIdx.x] = t;
    atomicMax(&counters[1], (unsigned long long)mm);
  }
}

__global__ void __launch_bounds__(1024) k_scan_top(int* __restrict__ block_sums, int nb) {
  __shared__ int buf[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int off = 0; off < nb; off += 1024) {
    const int i = off + threadIdx.x;
    const int v = (i < nb) ? block_sums[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
      const int a = (threadIdx.x >= d) ? buf[threadIdx.x - d] : 0;
      __syncthreads();
      buf[threadIdx.x] += a;
      __syncthreads();
    }
    if (i < nb) block_sums[i] = carry + buf[threadIdx.x] - v;  // exclusive
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_scan_final(const int* __restrict__ counts, int64_t n,
                                                    const int* __restrict__ block_sums, int* __restrict__ start) {
  __shared__ int warp_sums[8];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * 4;
  int v[4], s = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[i] = (base + i < n) ? counts[base + i] : 0;
    s += v[i];
  }
  // inclusive warp scan of per-thread sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int a = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += a;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  int woff = 0;
  for (int w = 0; w < warp; ++w) woff += warp_sums[w];
  int run = block_sums[blockIdx.x] + woff + incl - s;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (base + i < n) start[base + i] = run;
    run += v[i];
    if (base + i == n - 1) start[n] = run;  // the owner of the last cell writes the total
  }
}

__global__ void __launch_bounds__(256) k_bin_place(const int* __restrict__ tmp_cell, const int* __restrict__ tmp_slot,
                                                   const int* __restrict__ start,
                                                   const unsigned long long* __restrict__ counters,
                                                   int64_t cap, int* __restrict__ perm) {
  const int64_t nkept = (int64_t)counters[0];
  if (nkept > cap) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nkept; i += (int64_t)gridDim.x * blockDim.x)
    perm[start[tmp_cell[i]] + tmp_slot[i]] = (int)i;
}

// Per cell: order the entries by candidate index (the reference's insertion
// order) and write the records.  Cells of up to kRankRegs entries rank in
// registers; larger cells rank from memory.
constexpr int kRankRegs = 24;

__device__ __forceinline__ void write_record(const BinnedAtoms& b, int dst, const double4_32a& f, int packed,
                                             double a11, double a22, double a33, int want_fp64) {
  b.p32[dst] = make_float4((float)(a11 * f.x), (float)(a22 * f.y), (float)(a33 * f.z), __int_as_float(packed));
  if (want_fp64) {
    double sn, cs;
    sincos(f.w, &sn, &cs);
    b.f64[dst] = make_double4_32a(f.x, f.y, f.z, 0.0);
    b.cs64[dst] = make_double2(cs, sn);
  } else {
    // g.y reduced modulo one cycle in FP64, the phasor in FP32
    double tcyc = f.w * kInv2Pi;
    tcyc = tcyc - rint(tcyc);
    float sf, cf;
    sincospif(2.0f * (float)tcyc, &sf, &cf);
    b.cs32[dst] = make_float2(cf, sf);
  }
}

__global__ void __launch_bounds__(128) k_bin_finalize(const BinParams* __restrict__ jobs, int n_jobs,
                                                      const int* __restrict__ start, const int* __restrict__ counts,
                                                      int64_t n_cells, const int* __restrict__ perm,
                                                      const int* __restrict__ tmp_key,
                                                      const double4_32a* __restrict__ tmp_f, int want_fp64,
                                                      BinnedAtoms b, const unsigned long long* __restrict__ counters,
                                                      int64_t cap) {
  if ((int64_t)counters[0] > cap) return;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (int64_t)gridDim.x * blockDim.x) {
    const int job = n_jobs == 1 ? 0 : find_job(n_jobs, c, [&](int k) { return jobs[k].cell_base; });
    const BinParams& p = jobs[job];
    const int Ex = p.Ex, Ey = p.Ey;
    const double a11 = p.a_col[0], a22 = p.a_col[1], a33 = p.a_col[2];
    const int64_t cl = c - p.cell_base;
    const int s = start[c], n = counts[c];
    const int cz = (int)(cl / ((int64_t)Ex * Ey));
    const int rem = (int)(cl - (int64_t)cz * Ex * Ey);
    const int cy = rem / Ex, cx = rem - cy * Ex;
    const int packed = pack_cell(cx, cy, cz);
    if (n <= kRankRegs) {
      int key[kRankRegs], ti[kRankRegs];
#pragma unroll
      for (int i = 0; i < kRankRegs; ++i) {
        ti[i] = (i < n) ? perm[s + i] : 0;
        key[i] = (i < n) ? tmp_key[ti[i]] : 0x7fffffff;
      }
#pragma unroll
      for (int i = 0; i < kRankRegs; ++i) {
        if (i >= n) break;
        int r = 0;
#pragma unroll
        for (int j = 0; j < kRankRegs; ++j) r += (key[j] < key[i]);
        write_record(b, s + r, tmp_f[ti[i]], packed, a11, a22, a33, want_fp64);
      }
    } else {
      for (int i = 0; i < n; ++i) {
        const int t = perm[s + i];
        const int ki = tmp_key[t];
        int r = 0;
        for (int j = 0; j < n; ++j) r += (tmp_key[perm[s + j]] < ki);
        write_record(b, s + r, tmp_f[t], packed, a11, a22, a33, want_fp64);
      }
    }
  }
}

int grid_for(int64_t n, int threads, int max_blocks) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

}  // namespace

cudaError_t launch_bin(const BinParams* d_jobs, int n_jobs, int64_t total_cand, int64_t total_cells, int64_t cap,
                       Scratch& s, BinnedAtoms& b, bool exact, cudaStream_t st) {
  cudaMemsetAsync(b.cell_count, 0, sizeof(int) * total_cells, st);
  cudaMemsetAsync(s.counters, 0, sizeof(unsigned long long) * 8, st);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = grid_for(total_cand, 256, sms * 16);
  if (exact)
    k_bin_transform<true><<<grid, 256, 0, st>>>(d_jobs, n_jobs, total_cand, cap, b.cell_count, s.tmp_key, s.tmp_cell,
                                                s.tmp_slot, s.tmp_f, s.counters);
  else
    k_bin_transform<false><<<grid, 256, 0, st>>>(d_jobs, n_jobs, total_cand, cap, b.cell_count, s.tmp_key,
                                                 s.tmp_cell, s.tmp_slot, s.tmp_f, s.counters);
  const int nb = (int)((total_cells + kScanBlock - 1) / kScanBlock);
  k_scan_blocks<<<nb, 256, 0, st>>>(b.cell_count, total_cells, s.block_sums, s.counters);
  k_scan_top<<<1, 1024, 0, st>>>(s.block_sums, nb);
  k_scan_final<<<nb, 256, 0, st>>>(b.cell_count, total_cells, s.block_sums, b.cell_start);
  k_bin_place<<<sms * 8, 256, 0, st>>>(s.tmp_cell, s.tmp_slot, b.cell_start, s.counters, cap, s.perm);
  return cudaGetLastError();
}

cudaError_t launch_bin_finalize(const BinParams* d_jobs, int n_jobs, int64_t total_cells, int64_t cap, Scratch& s,
                                BinnedAtoms& b, int want_fp64, cudaStream_t st) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_bin_finalize<<<grid_for(total_cells, 128, sms * 16), 128, 0, st>>>(d_jobs, n_jobs, b.cell_start, b.cell_count,
                                                                       total_cells, s.perm, s.tmp_key, s.tmp_f,
                                                                       want_fp64, b, s.counters, cap);
  return cudaGetLastError();
}

}  // namespace stem
