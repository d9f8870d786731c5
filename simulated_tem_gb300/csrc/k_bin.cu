// K1: findGdotR + link-cell binning as a counting sort.
//
// Follows Lib_DynamicalTwoBeamImaging.f90:1160-1265 (findGdotR) and
// Lib_LinkCell3D.f90:691-748 (add0): for every periodic replica nn and atom jj
//   y = RU (x + Ruvw(nn)) + delta,  z = y - lc_delta,
// the atom is kept when floor(ia z) lies inside the link-cell box; it goes to
// cell floor(ia z) with fractional offset ia z - floor(ia z), and its phase is
// g . y.
//
// FP64 path (k_bin_transform_exact): one thread per candidate (nn, jj); every kept
// candidate goes through the reference's rounded FP64 arithmetic in its order, so the
// offsets and the phase are bit-identical to the reference's.  An FP32 pass rejects
// candidates far outside the box first.
//
// FP32 path (k_bin_atoms_fp32): one thread per atom, looping over the replicas.  FP64
// runs at 1/64 of the FP32 rate on this GPU, so the FP64 work is done once per atom:
// c = A x + B(nn) with A = ia RU and B(nn) = ia (RU Ruvw(nn) + delta - lc_delta), and
// g.y / 2 pi = gA x + gB(nn); the x parts in FP64, rounded to 64-bit fixed point of
// 2^-36, then every replica is an integer add (B(nn) in the same fixed point, computed
// on the host).  The cell is the fixed-point value's integer part, which equals the
// reference's floor(c) unless c lies within 1e-9 cells of a cell face (the fixed-point
// value is within 3e-11 cells of the exact c, the reference's rounded c within 1e-12);
// those rare candidates, and atoms too far out for the fixed point, take the reference's
// arithmetic, so the cell assignment is bit-identical to the reference's either way.
// The phase, g.y reduced modulo one cycle, is exact in the fixed point to 1e-11 cycles.
// The kernel writes the FP32 records directly (offsets times the cell sides and the
// phasor), leaving the finalize pass only the ordering.
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
constexpr int kFixBits = 36;
constexpr long long kFracMask = (1LL << kFixBits) - 1;
constexpr long long kFixFace = 69;  // 1e-9 cells (or cycles) in units of 2^-36
constexpr double kFixScale = 68719476736.0;  // 2^36
constexpr double kFixLimit = 1125899906842624.0;  // 2^50: |A x| below 2^14 cells for the fixed point

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

// The reference's transform of candidate (nn, x), every operation rounded separately in
// its order: y = RU (x + Ruvw(nn)) + delta and the link-cell coordinates c = ia (y - lc_delta).
__device__ __forceinline__ void reference_transform(const BinParams& p, int nn, double x0, double x1, double x2,
                                                    double* y, double* c) {
  const double yy0 = __dadd_rn(x0, p.Ruvw[3 * nn + 0]);
  const double yy1 = __dadd_rn(x1, p.Ruvw[3 * nn + 1]);
  const double yy2 = __dadd_rn(x2, p.Ruvw[3 * nn + 2]);
  y[0] = __dadd_rn(dot3_rn(p.RU[0], p.RU[3], p.RU[6], yy0, yy1, yy2), p.delta[0]);
  y[1] = __dadd_rn(dot3_rn(p.RU[1], p.RU[4], p.RU[7], yy0, yy1, yy2), p.delta[1]);
  y[2] = __dadd_rn(dot3_rn(p.RU[2], p.RU[5], p.RU[8], yy0, yy1, yy2), p.delta[2]);
  const double z0 = __dsub_rn(y[0], p.lc_delta[0]);
  const double z1 = __dsub_rn(y[1], p.lc_delta[1]);
  const double z2 = __dsub_rn(y[2], p.lc_delta[2]);
  c[0] = dot3_rn(p.ia[0], p.ia[3], p.ia[6], z0, z1, z2);
  c[1] = dot3_rn(p.ia[1], p.ia[4], p.ia[7], z0, z1, z2);
  c[2] = dot3_rn(p.ia[2], p.ia[5], p.ia[8], z0, z1, z2);
}

// Warp-aggregated slots: the compaction index of a kept candidate and its arrival slot in
// its cell.  Called by exactly the lanes in `mask` (the kept ones).
__device__ __forceinline__ void claim_slots(unsigned mask, int cell, int* counts, unsigned long long* counters,
                                            int64_t& idx, int& slot) {
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(&counters[0], (unsigned long long)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  idx = (int64_t)base + __popc(mask & ((1u << lane) - 1));
  // consecutive atoms often share a cell: one atomic per cell and warp
  const unsigned same = __match_any_sync(mask, cell);
  const int first = __ffs(same) - 1;
  int slot0 = 0;
  if (lane == first) slot0 = atomicAdd(&counts[cell], __popc(same));
  slot = __shfl_sync(same, slot0, first) + __popc(same & ((1u << lane) - 1));
}

// FP64 path: one thread per candidate (replica nn, atom jj) in the reference's insertion
// order t = nn * N + jj; every kept candidate in the reference's rounded arithmetic.
__global__ void __launch_bounds__(256) k_bin_transform_exact(const BinParams* __restrict__ jobs, int n_jobs,
                                                             int64_t total, int64_t cap, int* __restrict__ counts,
                                                             int* __restrict__ tmp_key, int* __restrict__ tmp_cell,
                                                             int* __restrict__ tmp_slot,
                                                             double4_32a* __restrict__ tmp_f,
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
    double c[3] = {0, 0, 0}, y[3] = {0, 0, 0};
    if (keep) {
      reference_transform(p, nn, x0, x1, x2, y, c);
      // pointInSupercell: floor(c) in [0, N) on every axis
      keep = c[0] >= 0.0 && c[0] < (double)p.Ex && c[1] >= 0.0 && c[1] < (double)p.Ey && c[2] >= 0.0 &&
             c[2] < (double)p.Ez;
    }
    const unsigned mask = __ballot_sync(__activemask(), keep);
    if (!keep) continue;
    const double fl0 = floor(c[0]), fl1 = floor(c[1]), fl2 = floor(c[2]);
    const int cell = (int)p.cell_base + (int)fl0 + p.Ex * ((int)fl1 + p.Ey * (int)fl2);
    int64_t idx;
    int slot;
    claim_slots(mask, cell, counts, counters, idx, slot);
    if (idx >= cap) continue;  // overflow: counted, not stored; the host grows the arrays and retries
    tmp_key[idx] = (int)t;
    tmp_cell[idx] = cell;
    tmp_slot[idx] = slot;
    tmp_f[idx] = make_double4_32a(__dsub_rn(c[0], fl0), __dsub_rn(c[1], fl1), __dsub_rn(c[2], fl2),
                                  dot3_rn(p.g[0], p.g[1], p.g[2], y[0], y[1], y[2]));
  }
}

// 2^-32 * (32 bits of a 2^-36 fixed-point fraction in [0, 1)), rounded to FP32
__device__ __forceinline__ float fix_frac_to_float(long long f) {
  return (float)(unsigned)(f >> 4) * 2.3283064365386963e-10f;
}

// The FP32 path's decision for candidate (nn, atom): kept or not, and, when kept, the
// fixed-point link-cell coordinates c[3] (cell << 36 | fraction) and phase gt (cycles,
// 2^-36).  `fixed` atoms use the fixed point (the reference's arithmetic decides within
// 1e-9 cells of a face), the others the reference's arithmetic throughout.
struct AtomFix {
  double x0, x1, x2;
  long long q0, q1, q2, gq;  // A x and gA x in 2^-36 fixed point
  float v0, v1, v2;          // A x in cells, FP32, for the prefilter
  bool fixed;
};

__device__ __forceinline__ bool prefilter(const BinParams& p, const AtomFix& a, int nn) {
  if (!a.fixed) return true;
  const float margin = 2e-3f;  // cells; the prefilter's error is below 1e-4 cells
  const float cf0 = a.v0 + p.Bf[3 * nn + 0], cf1 = a.v1 + p.Bf[3 * nn + 1], cf2 = a.v2 + p.Bf[3 * nn + 2];
  return cf0 >= -margin && cf0 < p.Ex + margin && cf1 >= -margin && cf1 < p.Ey + margin && cf2 >= -margin &&
         cf2 < p.Ez + margin;
}

__device__ __forceinline__ bool decide(const BinParams& p, const AtomFix& a, int nn, long long* c, long long& gt) {
  bool exact = !a.fixed, keep = false;
  if (a.fixed) {
    c[0] = a.q0 + p.Bfx[3 * nn + 0];
    c[1] = a.q1 + p.Bfx[3 * nn + 1];
    c[2] = a.q2 + p.Bfx[3 * nn + 2];
    gt = a.gq + p.gBfx[nn];
    const int k0 = (int)(c[0] >> kFixBits), k1 = (int)(c[1] >> kFixBits), k2 = (int)(c[2] >> kFixBits);
    const long long f0 = c[0] & kFracMask, f1 = c[1] & kFracMask, f2 = c[2] & kFracMask;
    const bool near = f0 < kFixFace || f0 > kFracMask - kFixFace || f1 < kFixFace || f1 > kFracMask - kFixFace ||
                      f2 < kFixFace || f2 > kFracMask - kFixFace;
    const bool reach = k0 >= -1 && k0 <= p.Ex && k1 >= -1 && k1 <= p.Ey && k2 >= -1 && k2 <= p.Ez;
    exact = near && reach;
    keep = !exact && (unsigned)k0 < (unsigned)p.Ex && (unsigned)k1 < (unsigned)p.Ey && (unsigned)k2 < (unsigned)p.Ez;
  }
  if (exact) {
    // the reference's arithmetic decides (a cell face within 1e-9 cells, or coordinates
    // beyond the fixed point's range)
    double y[3], cd[3];
    reference_transform(p, nn, a.x0, a.x1, a.x2, y, cd);
    keep = cd[0] >= 0.0 && cd[0] < (double)p.Ex && cd[1] >= 0.0 && cd[1] < (double)p.Ey && cd[2] >= 0.0 &&
           cd[2] < (double)p.Ez;
    if (keep) {
      for (int k = 0; k < 3; ++k) {
        const double fl = floor(cd[k]);
        const long long fr = __double2ll_rn(__dsub_rn(cd[k], fl) * kFixScale);
        c[k] = ((long long)fl << kFixBits) | (fr > kFracMask ? kFracMask : fr);
      }
      if (!a.fixed) {
        const double cyc = dot3_rn(p.g[0], p.g[1], p.g[2], y[0], y[1], y[2]) * kInv2Pi;
        gt = __double2ll_rn((cyc - rint(cyc)) * kFixScale);
      }
    }
  }
  return keep;
}

// FP32 path: one thread per atom, all replicas.  Warps stay converged: every lane runs
// the same replica loop, lanes past the end or past their job's replicas keep nothing.
// (Counting first and claiming one compaction range per block halves the atomics on the
// kept-atom counter but decides every candidate twice: slower.)
__global__ void __launch_bounds__(256) k_bin_atoms_fp32(const BinParams* __restrict__ jobs, int n_jobs,
                                                        int64_t total_atoms, int64_t cap, int* __restrict__ counts,
                                                        int* __restrict__ tmp_key, int* __restrict__ tmp_cell,
                                                        int* __restrict__ tmp_slot, Rec32* __restrict__ tmp_r,
                                                        unsigned long long* __restrict__ counters) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total_atoms; base += stride) {
    const int64_t ag = base + lane;  // warp-uniform loop
    const bool valid = ag < total_atoms;
    const int job = (!valid || n_jobs == 1) ? 0 : find_job(n_jobs, ag, [&](int k) { return jobs[k].atom_base; });
    const BinParams& p = jobs[job];
    const int64_t jj = valid ? ag - p.atom_base : 0;
    const int nrep = valid ? p.nuvw : 0;
    AtomFix a;
    a.x0 = a.x1 = a.x2 = 0.0;
    if (valid) {
      const double* xa = p.x + jj * p.ldx;
      a.x0 = xa[0];
      a.x1 = xa[1];
      a.x2 = xa[2];
    }
    // the atom's part, in FP64, then in fixed point
    const double u0 = fma(p.Afx[2], a.x2, fma(p.Afx[1], a.x1, p.Afx[0] * a.x0));
    const double u1 = fma(p.Afx[5], a.x2, fma(p.Afx[4], a.x1, p.Afx[3] * a.x0));
    const double u2 = fma(p.Afx[8], a.x2, fma(p.Afx[7], a.x1, p.Afx[6] * a.x0));
    const double gu = fma(p.gAfx[2], a.x2, fma(p.gAfx[1], a.x1, p.gAfx[0] * a.x0));
    a.fixed = p.fix_ok && fabs(u0) < kFixLimit && fabs(u1) < kFixLimit && fabs(u2) < kFixLimit &&
              fabs(gu) < kFixLimit;
    a.q0 = a.q1 = a.q2 = a.gq = 0;
    if (a.fixed) {
      a.q0 = __double2ll_rn(u0);
      a.q1 = __double2ll_rn(u1);
      a.q2 = __double2ll_rn(u2);
      a.gq = __double2ll_rn(gu);
    }
    a.v0 = (float)(int)(a.q0 >> 20) * 1.52587890625e-05f;  // 2^-16 cells
    a.v1 = (float)(int)(a.q1 >> 20) * 1.52587890625e-05f;
    a.v2 = (float)(int)(a.q2 >> 20) * 1.52587890625e-05f;
    const int nmax = __reduce_max_sync(0xffffffffu, nrep);
    for (int nn = 0; nn < nmax; ++nn) {
      const bool cand = nn < nrep && prefilter(p, a, nn);
      if (__any_sync(0xffffffffu, cand)) {
        long long c[3] = {0, 0, 0}, gt = 0;
        const bool keep = cand && decide(p, a, nn, c, gt);
        const unsigned mask = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int k0 = (int)(c[0] >> kFixBits), k1 = (int)(c[1] >> kFixBits), k2 = (int)(c[2] >> kFixBits);
          const int cell = (int)p.cell_base + k0 + p.Ex * (k1 + p.Ey * k2);
          int64_t idx;
          int slot;
          claim_slots(mask, cell, counts, counters, idx, slot);
          if (idx < cap) {  // else overflow: counted, not stored; the host grows the arrays and retries
            // phase: g.y / 2 pi reduced to [-1/2, 1/2) cycles (sign-extended 36-bit fraction)
            const long long r = (long long)((unsigned long long)gt << (64 - kFixBits)) >> (64 - kFixBits);
            const float tc = (float)(int)(r >> 4) * 2.3283064365386963e-10f;
            tmp_key[idx] = (int)((int64_t)nn * p.n_atoms + jj);
            tmp_cell[idx] = cell;
            tmp_slot[idx] = slot;
            // both 16-byte halves of the 32-byte record, so no sector is partly written
            float4* rec = reinterpret_cast<float4*>(tmp_r + idx);
            rec[0] = make_float4(p.a_colf[0] * fix_frac_to_float(c[0] & kFracMask),
                                 p.a_colf[1] * fix_frac_to_float(c[1] & kFracMask),
                                 p.a_colf[2] * fix_frac_to_float(c[2] & kFracMask),
                                 __int_as_float(pack_cell(k0, k1, k2)));
            rec[1] = make_float4(tc, __uint_as_float((unsigned)((c[0] & kFracMask) >> 4)),
                                 __uint_as_float((unsigned)((c[1] & kFracMask) >> 4)),
                                 __uint_as_float((unsigned)((c[2] & kFracMask) >> 4)));
          }
        }
      }
      __syncwarp();
    }
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

// Ordering: the entry at sorted position q (cell c, arrival slot order) moves to
// start[c] + its rank by candidate index among the cell's entries (the reference's
// insertion order).  One thread per kept atom; the threads of a cell read the same few
// keys (L1 hits).
__device__ __forceinline__ void write_record(const BinnedAtoms& b, int dst, const double4_32a& f, int packed,
                                             double a11, double a22, double a33) {
  b.p32[dst] = make_float4((float)(a11 * f.x), (float)(a22 * f.y), (float)(a33 * f.z), __int_as_float(packed));
  double sn, cs;
  sincos(f.w, &sn, &cs);
  b.f64[dst] = make_double4_32a(f.x, f.y, f.z, 0.0);
  b.cs64[dst] = make_double2(cs, sn);
}

template <bool kFp32>
__global__ void __launch_bounds__(256) k_bin_finalize(const BinParams* __restrict__ jobs, int n_jobs,
                                                      const int* __restrict__ start, const int* __restrict__ counts,
                                                      const int* __restrict__ perm, const int* __restrict__ tmp_key,
                                                      const int* __restrict__ tmp_cell,
                                                      const double4_32a* __restrict__ tmp_f, BinnedAtoms b,
                                                      const unsigned long long* __restrict__ counters, int64_t cap) {
  const int64_t nkept = (int64_t)counters[0];
  if (nkept > cap) return;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nkept; q += (int64_t)gridDim.x * blockDim.x) {
    const int t = perm[q];
    const int cell = tmp_cell[t];
    const int key = tmp_key[t];
    const int s = start[cell], n = counts[cell];
    int r = 0;
    for (int j = 0; j < n; ++j) r += (tmp_key[perm[s + j]] < key);
    if constexpr (kFp32) {
      // the binning wrote the records; they move to their place, with the phasor of the
      // FP64-reduced phase and the cell fractions for the column kernels' cutoff recheck
      const float4* rec = reinterpret_cast<const float4*>(tmp_f + t);
      const float4 hi = rec[1];
      float sf, cf;
      sincospif(2.0f * hi.x, &sf, &cf);
      b.p32[s + r] = rec[0];
      b.cs32[s + r] = make_float2(cf, sf);
      b.fr32[s + r] = make_uint4(__float_as_uint(hi.y), __float_as_uint(hi.z), __float_as_uint(hi.w), 0u);
      b.ph32[s + r] = hi.x;
    } else {
      const int job = n_jobs == 1 ? 0 : find_job(n_jobs, cell, [&](int k) { return jobs[k].cell_base; });
      const BinParams& p = jobs[job];
      const int64_t cl = cell - p.cell_base;
      const int cz = (int)(cl / ((int64_t)p.Ex * p.Ey));
      const int rem = (int)(cl - (int64_t)cz * p.Ex * p.Ey);
      const int cy = rem / p.Ex, cx = rem - cy * p.Ex;
      write_record(b, s + r, tmp_f[t], pack_cell(cx, cy, cz), p.a_col[0], p.a_col[1], p.a_col[2]);
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

cudaError_t launch_bin(const BinParams* d_jobs, int n_jobs, int64_t total_atoms, int64_t total_cand,
                       int64_t total_cells, int64_t cap, Scratch& s, BinnedAtoms& b, bool fp32, cudaStream_t st) {
  cudaMemsetAsync(b.cell_count, 0, sizeof(int) * total_cells, st);
  cudaMemsetAsync(s.counters, 0, sizeof(unsigned long long) * 8, st);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (fp32)
    k_bin_atoms_fp32<<<grid_for(total_atoms, 256, sms * 16), 256, 0, st>>>(
        d_jobs, n_jobs, total_atoms, cap, b.cell_count, s.tmp_key, s.tmp_cell, s.tmp_slot,
        reinterpret_cast<Rec32*>(s.tmp_f), s.counters);
  else
    k_bin_transform_exact<<<grid_for(total_cand, 256, sms * 16), 256, 0, st>>>(
        d_jobs, n_jobs, total_cand, cap, b.cell_count, s.tmp_key, s.tmp_cell, s.tmp_slot, s.tmp_f, s.counters);
  const int nb = (int)((total_cells + kScanBlock - 1) / kScanBlock);
  launch_count() += 5;  // the kernel above, three scans and the placement
  k_scan_blocks<<<nb, 256, 0, st>>>(b.cell_count, total_cells, s.block_sums, s.counters);
  k_scan_top<<<1, 1024, 0, st>>>(s.block_sums, nb);
  k_scan_final<<<nb, 256, 0, st>>>(b.cell_count, total_cells, s.block_sums, b.cell_start);
  k_bin_place<<<sms * 8, 256, 0, st>>>(s.tmp_cell, s.tmp_slot, b.cell_start, s.counters, cap, s.perm);
  return cudaGetLastError();
}

cudaError_t launch_bin_finalize(const BinParams* d_jobs, int n_jobs, int64_t total_cells, int64_t cap, Scratch& s,
                                BinnedAtoms& b, bool fp32, cudaStream_t st) {
  (void)total_cells;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = grid_for(cap, 256, sms * 8);  // the kernel reads the kept count on the device
  ++launch_count();
  if (fp32)
    k_bin_finalize<true><<<grid, 256, 0, st>>>(d_jobs, n_jobs, b.cell_start, b.cell_count, s.perm, s.tmp_key,
                                               s.tmp_cell, s.tmp_f, b, s.counters, cap);
  else
    k_bin_finalize<false><<<grid, 256, 0, st>>>(d_jobs, n_jobs, b.cell_start, b.cell_count, s.perm, s.tmp_key,
                                                s.tmp_cell, s.tmp_f, b, s.counters, cap);
  return cudaGetLastError();
}

}  // namespace stem
