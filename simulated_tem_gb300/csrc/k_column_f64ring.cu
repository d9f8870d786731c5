// K2+K3, FP64: the slab-ring column kernel of the plain FP64 path.
//
// The pixel loop of computeD2BI_img (Lib_DynamicalTwoBeamImaging.f90:1870-1900) with the
// neighbour search of Lib_LinkCell3D.f90:1515-1605 and the integrator of :2316-2480, in
// the reference's FP64 arithmetic, on the FP32 path's slab ring (k_column_v3.cuh): one
// warp per 8 x 4 pixel columns, two depth slices per step (four with one angle per pass
// where every image's steps of four slices fit the ring), the atoms of the link-cell slabs
// staged once in warp-private shared memory and ordered by z bin.
//
// What is exact, and how:
// * The accept decision is the reference's: d_a = a_aa (f_a + (k_a - zi_frac_a)) for
//   each axis, d.d = (d_x^2 + d_y^2) + d_z^2 <= (3 sigma)^2, every operation rounded
//   alike, with the fractions f the FP64 binning keeps (bit-identical to the reference's)
//   and the unwrapped 27-cell offsets k.  An FP32 test with a margin only skips atoms far
//   from the cutoff, so the accepted set and count equal the reference's.
// * The weight: the reference evaluates exp(-d.d / 2 sigma^2) per pair.  Here the Gaussian
//   is split, exp(-(d_x^2 + d_y^2) / 2 sigma^2) per atom and column for all slices of a
//   step, times exp(-d_z^2 / 2 sigma^2) per atom and slice, formed once by the warp: the
//   product differs from the reference's weight by a few ulp.  Each slice's sum takes the
//   same accepted atoms in the same order at two or four slices per step, so both give the
//   same image to the bit.
// * The sums S run in the step buffer's order rather than the 27-cell loop's; both are
//   FP64 sums of the same terms.
// The field sample, the density and the RK4 double step are fp64_column.cuh's, the
// reference's operations in order.  Images agree with the reference's to about 1e-15.
#include <cuda_runtime.h>

#include <cfloat>

#include "fp64_column.cuh"
#include "internal.h"
#include "k_column_v3.cuh"

namespace stem {
namespace ring64 {

using namespace fp64col;
using ring3::Geo;
using ring3::kBins;
using ring3::kRing;
using ring3::load_slab3;
using ring3::pos_mod;

constexpr int kWarps = 4;
constexpr float kPreMargin = 1e-3f;      // scaled r^2: the FP32 prefilter's margin over its error

// SL slices per step (2, or 4 where every image's steps of four slices fit the ring); the
// step buffer holds kN atoms and is flushed at kN - 32, before a round of 32 may add more.
template <int CAPS, int SL>
struct WarpSmem64 {
  static_assert(CAPS % 32 == 0, "the z sort holds CAPS / 32 atoms per lane");
  static constexpr int kN = SL == 4 ? 48 : 64;
  static constexpr int kFlush = kN - 32;
  float4 p[kRing][CAPS];  // X', Y', z (scaled FP32, for the prefilter), cell code
  int gi[kRing][CAPS];    // index of the kept atom
  int bin[kRing][kBins + 1];
  int count[kRing];
  float4 ba[kN];          // X', Y', the largest hmax of the step's slices + margin (FP32 prefilter), 0
  double2 bf[kN];         // f_x, f_y (the reference's cell fractions)
  double2 be[kN][SL];     // per slice: exp(-d_z^2 / 2 sigma^2) (cos, sin)
  double bz[kN][SL];      // per slice: d_z^2 (+inf where the slab does not serve the slice)
  int bc[kN];             // cell code (unwrapped x, y cell relative to the warp's reference cells)
};

template <int SL>
struct Acc64 {
  double sr[SL], si[SL], rm[SL];
  unsigned n_acc;
};

// Every buffered atom against this lane's column at the step's SL slices.  One in-plane
// exp per accepted atom serves all of them.
template <int CAPS, int SL>
__device__ __forceinline__ void consume64(const WarpSmem64<CAPS, SL>& W, int n, float Xv, float Yv, int hxo, int hyo,
                                          const double* dzx, const double* dzy, double a11, double a22, double cut2,
                                          double i2s2, Acc64<SL>& A) {
  for (int i = 0; i < n; ++i) {
    const float4 q = W.ba[i];
    const float dx = q.x - Xv, dy = q.y - Yv;
    const float h = fmaf(dx, dx, dy * dy);
    if (!(h <= q.z)) continue;  // beyond the cutoff at every slice, with margin
    const int code = W.bc[i];
    const int kx = (code & 255) - hxo, ky = ((code >> 8) & 255) - hyo;
    if (kx < -1 || kx > 1 || ky < -1 || ky > 1) continue;  // outside the lane's 27 cells
    const double2 f = W.bf[i];
    const double d0 = DM(a11, DA(f.x, dzx[kx + 1]));
    const double d1 = DM(a22, DA(f.y, dzy[ky + 1]));
    const double dxy = DA(DM(d0, d0), DM(d1, d1));
    double dd[SL];
    bool acc[SL], any = false;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      dd[k] = DA(dxy, W.bz[i][k]);
      acc[k] = dd[k] <= cut2;
      any = any || acc[k];
    }
    if (!any) continue;
    const double wxy = exp(DM(-dxy, i2s2));
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      if (acc[k]) {
        const double2 e = W.be[i][k];
        A.sr[k] = DA(A.sr[k], DM(wxy, e.x));
        A.si[k] = DA(A.si[k], DM(wxy, e.y));
        A.rm[k] = fmin(A.rm[k], dd[k]);
        ++A.n_acc;
      }
    }
  }
}

// The field sample of one voxel from its sum (:1877-1895, 1973-1994).
__device__ __forceinline__ Sample64 sample64(const ColumnParams& p, double sr, double si, double r2min) {
  double ww = hypot(sr, si);
  ww = __ddiv_rn(1.0, fmax(1.0e-16, ww));
  const double xr = DM(sr, ww), xi = DM(si, ww);
  const double rho = p.use_density ? rho64(r2min, p.sigma) : 1.0;
  const double bgr = DM(p.bg, rho);
  return Sample64{DM(p.b0, rho), DM(p.b0, rho), DM(bgr, xr), DM(bgr, xi)};
}

template <int NP, int CAPS, bool kMasked, int SL>
__device__ __noinline__ bool column_tile64(const ColumnParams& p, WarpSmem64<CAPS, SL>& W, int tile, int lane) {
  constexpr int TX = 8, TY = 4;
  const int Wd = p.ix1 - p.ix0;
  const int tiles_x = (Wd + TX - 1) / TX;
  const int tx = tile % tiles_x, ty = tile / tiles_x;
  const int ix = p.ix0 + tx * TX + (lane % TX);
  const int iy = p.iy0 + ty * TY + lane / TX;
  const bool active = ix < p.ix1 && iy < p.iy1;
  bool wanted = true;
  if constexpr (kMasked) {
    if (p.tile_mask) wanted = active && p.tile_mask[(iy / p.mask_T) * p.mask_ntx + ix / p.mask_T] != 0;
    if (!__any_sync(0xffffffffu, wanted)) return true;
  }

  const double sd = sqrt(p.i2s2 * 1.4426950408889634);
  Geo G;
  G.scale = (float)sd;
  const int ixc = min(ix, p.ix1 - 1), iyc = min(iy, p.iy1 - 1);
  const int hx = p.xtab[ixc].x, hy = p.ytab[iyc].x;
  const double fvx = p.xfv[ixc], fvy = p.yfv[iyc];
  {
    const int big = 1 << 29;
    const int mnx = __reduce_min_sync(0xffffffffu, active ? hx : big);
    const int mxx = __reduce_max_sync(0xffffffffu, active ? hx : -big);
    const int mny = __reduce_min_sync(0xffffffffu, active ? hy : big);
    const int mxy = __reduce_max_sync(0xffffffffu, active ? hy : -big);
    G.ux_lo = mnx - 1;
    G.ux_hi = mxx + 1;
    G.uy_lo = mny - 1;
    G.uy_hi = mxy + 1;
    G.ux_ref = mnx;
    G.uy_ref = mny;
  }
  G.a11s = (float)(p.a11 * sd);
  G.a22s = (float)(p.a22 * sd);
  G.a33s = (float)(p.a33 * sd);
  const float Xv = (float)(p.a11 * (fvx + (double)(hx - G.ux_ref)) * sd);
  const float Yv = (float)(p.a22 * (fvy + (double)(hy - G.uy_ref)) * sd);
  {
    const float big = 1e30f;
    float v = active ? Xv : big, w = active ? -Xv : big, y = active ? Yv : big, z = active ? -Yv : big;
    for (int o = 16; o > 0; o >>= 1) {
      v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
      w = fminf(w, __shfl_xor_sync(0xffffffffu, w, o));
      y = fminf(y, __shfl_xor_sync(0xffffffffu, y, o));
      z = fminf(z, __shfl_xor_sync(0xffffffffu, z, o));
    }
    G.xmin = v;
    G.xmax = -w;
    G.ymin = y;
    G.ymax = -z;
  }
  const float cut2f = (float)(p.cut2 * sd * sd);
  const float r3 = sqrtf(cut2f) * 1.0001f + 1e-3f;  // z-window half width, rounded up
  G.pre2 = cut2f * 1.0002f + 1e-2f;
  const float inv_bin = kBins / G.a33s;
  // k - zi_frac for k = -1, 0, 1 (:1576-1588), and this lane's cells relative to the frame
  double dzx[3], dzy[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dzx[k] = DS((double)(k - 1), fvx);
    dzy[k] = DS((double)(k - 1), fvy);
  }
  const int hxo = hx - G.ux_ref + 8, hyo = hy - G.uy_ref + 8;
  const unsigned lt = (1u << lane) - 1;

  const int np = min(NP, p.n_prec - p.prec_offset);
  double aa[NP], ph[NP][4];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    aa[k] = (k < np) ? p.aa[p.prec_offset + k] : 0.0;
    ph[k][0] = 1.0;
    ph[k][1] = ph[k][2] = ph[k][3] = 0.0;
  }
  Sample64 s_first{0, 0, 0, 0}, s_prev{0, 0, 0, 0}, s_mid{0, 0, 0, 0};
  int ring_lo = 1 << 30, ring_hi = (1 << 30) - 1;
  unsigned n_acc = 0;
  unsigned long long n_tst = 0;

  using WS = WarpSmem64<CAPS, SL>;
  for (int z0 = 0; z0 < p.Mz; z0 += SL) {
    // the step's slices: home z cells, FP32 depths in the frame of home cell hz[0] (the
    // table gives each pair's from its even slice's home cell), FP64 fractions
    int hz[SL];
    float zv[SL];
    double fz[SL];
    bool has[SL];
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      has[k] = z0 + k < p.Mz;
      const int2 e = p.ztab[has[k] ? z0 + k : z0];
      hz[k] = has[k] ? e.x : hz[0];
      zv[k] = has[k] ? __int_as_float(e.y) : 0.f;
      fz[k] = has[k] ? p.zfv[z0 + k] : 0.0;
    }
#pragma unroll
    for (int k = 2; k < SL; ++k)
      if (has[k]) zv[k] = __fadd_rn(zv[k], __fmul_rn(G.a33s, (float)(hz[k & ~1] - hz[0])));
    int hz_last = hz[0];
#pragma unroll
    for (int k = 1; k < SL; ++k)
      if (has[k]) hz_last = hz[k];
    const int need_lo = hz[0] - 1, need_hi = hz_last + 1;
    if (need_hi - need_lo + 1 > kRing) {  // the host takes four slices only where they fit
      if (lane == 0) atomicExch(&p.counters[4], 1ull);
      return false;
    }
    if (need_lo > ring_hi || need_hi < ring_lo) {
      ring_lo = need_lo;
      ring_hi = need_lo - 1;
    }
    if (ring_lo < need_lo) ring_lo = need_lo;
    bool ok = true;
    while (ring_hi < need_hi && ok) {
      ++ring_hi;
      ok = load_slab3<CAPS, true>(p, G, ring_hi, W, lane);
    }
    if (!ok) {
      if (lane == 0) atomicExch(&p.counters[4], 1ull);
      return false;
    }
    Acc64<SL> A;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      A.sr[k] = A.si[k] = 0.0;
      A.rm[k] = (double)FLT_MAX;
    }
    A.n_acc = 0u;
    int nb = 0;
    for (int u = need_lo; u <= need_hi; ++u) {
      const int slot = u & (kRing - 1);
      const float zoff = __fmul_rn(G.a33s, (float)(u - hz[0]));
      // the reference's 27 cells in z: slab u serves slice k within one cell of its home cell
      float t[SL];
      bool v[SL];
      float w_lo = 1e30f, w_hi = -1e30f;
#pragma unroll
      for (int k = 0; k < SL; ++k) {
        t[k] = __fsub_rn(zv[k], zoff);
        v[k] = has[k] && u - hz[k] >= -1 && u - hz[k] <= 1;
        if (v[k]) {
          w_lo = fminf(w_lo, t[k]);
          w_hi = fmaxf(w_hi, t[k]);
        }
      }
      if (w_lo > w_hi) continue;
      const int b_lo = max(0, min(kBins, (int)floorf((w_lo - r3) * inv_bin)));
      const int b_hi = max(0, min(kBins, (int)ceilf((w_hi + r3) * inv_bin)));
      const int lo = W.bin[slot][b_lo];
      const int hi = W.bin[slot][b_hi];
      for (int b = lo; b < hi; b += 32) {
        // one atom per lane: the FP32 prefilter bound, the z distances and z factors in FP64
        const int j = b + lane;
        bool keep = false;
        float4 A4;
        double2 F, E[SL];
        double Z[SL];
        int code = 0;
        if (j < hi) {
          const float4 q = W.p[slot][j];
          float hmax = -1.f;
#pragma unroll
          for (int k = 0; k < SL; ++k) {
            const float dz = q.z - t[k];
            hmax = fmaxf(hmax, v[k] ? cut2f - dz * dz + kPreMargin : -1.f);
          }
          const float dxr = fmaxf(0.f, fmaxf(G.xmin - q.x, q.x - G.xmax));
          const float dyr = fmaxf(0.f, fmaxf(G.ymin - q.y, q.y - G.ymax));
          keep = fmaf(dxr, dxr, dyr * dyr) <= hmax + kPreMargin;
          if (keep) {
            const int gi = W.gi[slot][j];
            const double4_32a f = p.f64[gi];
            const double2 cs = p.cs64[gi];
#pragma unroll
            for (int k = 0; k < SL; ++k) {
              const double d2 = DM(p.a33, DA(f.z, DS((double)(u - hz[k]), fz[k])));
              Z[k] = v[k] ? DM(d2, d2) : (double)INFINITY;
              const double ez = v[k] ? exp(DM(-Z[k], p.i2s2)) : 0.0;
              E[k] = make_double2(DM(ez, cs.x), DM(ez, cs.y));
            }
            A4 = make_float4(q.x, q.y, hmax, 0.f);
            F = make_double2(f.x, f.y);
            code = __float_as_int(q.w);
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int d = nb + __popc(m & lt);
          W.ba[d] = A4;
          W.bf[d] = F;
#pragma unroll
          for (int k = 0; k < SL; ++k) {
            W.bz[d][k] = Z[k];
            W.be[d][k] = E[k];
          }
          W.bc[d] = code;
        }
        nb += __popc(m);
        if (nb >= WS::kFlush) {
          __syncwarp();
          consume64<CAPS, SL>(W, nb, Xv, Yv, hxo, hyo, dzx, dzy, p.a11, p.a22, p.cut2, p.i2s2, A);
          n_tst += (unsigned long long)nb;
          __syncwarp();
          nb = 0;
        }
      }
    }
    if (nb > 0) {
      __syncwarp();
      consume64<CAPS, SL>(W, nb, Xv, Yv, hxo, hyo, dzx, dzy, p.a11, p.a22, p.cut2, p.i2s2, A);
      n_tst += (unsigned long long)nb;
      __syncwarp();
    }
    n_acc += A.n_acc;
    // the RK4 double steps: pair (z, z + 1) closes the double step (z - 2, z - 1, z) at z
#pragma unroll
    for (int pr = 0; pr < SL / 2; ++pr) {
      const int z = z0 + 2 * pr;
      if (z >= p.Mz) break;
      const Sample64 se = sample64(p, A.sr[2 * pr], A.si[2 * pr], A.rm[2 * pr]);
      if (z == 0) {
        s_first = se;
      } else {
#pragma unroll
        for (int k = 0; k < NP; ++k)
          if (k < np) rk4_64(s_prev, s_mid, se, aa[k], p.dz, ph[k]);
      }
      s_prev = se;
      if (z + 1 < p.Mz) s_mid = sample64(p, A.sr[2 * pr + 1], A.si[2 * pr + 1], A.rm[2 * pr + 1]);
    }
  }
  if ((p.Mz & 1) == 0) {
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) rk4_64(s_prev, s_mid, s_first, aa[k], p.dz, ph[k]);
  }
  if (active && wanted) {
    double* o = p.img + ix + (int64_t)p.Mx * iy;
    double acc = p.accumulate ? *o : 0.0;
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) acc = DA(acc, DA(DM(ph[k][2], ph[k][2]), DM(ph[k][3], ph[k][3])));
    if (p.finalize) {
      acc = __ddiv_rn(acc, p.fin_scale);
      if (p.fin_bright) acc = DS(1.0, acc);
    }
    *o = acc;
  }
  if (p.want_stats) {
    unsigned long long acc_w = active ? n_acc : 0u, tst_w = active ? (unsigned long long)SL * n_tst : 0u;
    for (int o = 16; o > 0; o >>= 1) {
      acc_w += __shfl_xor_sync(0xffffffffu, acc_w, o);
      tst_w += __shfl_xor_sync(0xffffffffu, tst_w, o);
    }
    if (lane == 0) {
      atomicAdd(&p.counters[2], tst_w);
      atomicAdd(&p.counters[3], acc_w);
    }
  }
  return true;
}

template <int NP, int CAPS, bool kMasked, int kMinBlocks, int SL>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks)
    k_column_fp64_ring(const ColumnJob* __restrict__ jobs, int n_jobs, int total_tiles, unsigned* __restrict__ work,
                       const unsigned long long* __restrict__ counters, int64_t cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpSmem64<CAPS, SL>& W = reinterpret_cast<WarpSmem64<CAPS, SL>*>(smem_raw)[warp];
  if ((int64_t)counters[0] > cap) return;
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = (int)atomicAdd(work, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= total_tiles) break;
    if (counters[4] != 0) break;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile_base[0] <= tile)
        lo = mid;
      else
        hi = mid - 1;
    }
    if (!column_tile64<NP, CAPS, kMasked, SL>(jobs[lo].p, W, tile - jobs[lo].tile_base[0], lane)) break;
  }
}

template <int CAPS, int SL, typename K>
cudaError_t launch64(K kernel, const ColumnJob* jobs, int n_jobs, int tiles, unsigned* work,
                     const unsigned long long* counters, int64_t cap, int blocks_per_sm, cudaStream_t st) {
  const size_t smem = sizeof(WarpSmem64<CAPS, SL>) * kWarps;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * blocks_per_sm;
  const int need = (tiles + kWarps - 1) / kWarps;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  ++launch_count();
  kernel<<<grid, kWarps * 32, smem, st>>>(jobs, n_jobs, tiles, work, counters, cap);
  return cudaGetLastError();
}

template <int NP, bool kMasked, int SL>
cudaError_t launch_tier(int tier, const ColumnJob* jobs, int n_jobs, int tiles, unsigned* work,
                        const unsigned long long* counters, int64_t cap, cudaStream_t st) {
  if (tier >= 2)
    return launch64<256, SL>(k_column_fp64_ring<NP, 256, kMasked, 1, SL>, jobs, n_jobs, tiles, work, counters, cap, 1,
                             st);
  if (tier == 1)
    return launch64<192, SL>(k_column_fp64_ring<NP, 192, kMasked, 2, SL>, jobs, n_jobs, tiles, work, counters, cap, 2,
                             st);
  return launch64<128, SL>(k_column_fp64_ring<NP, 128, kMasked, 3, SL>, jobs, n_jobs, tiles, work, counters, cap, 3,
                           st);
}

}  // namespace ring64

// The FP64 slab-ring launch over the jobs of one pass (at most 4 precession angles).
// `four`: every job's steps of four slices fit the ring (four_slices_fit), so a launch of
// one angle per pass marches four slices per step: each in-plane exp then serves four
// slices instead of two, and the images are the two-slice march's to the bit (each slice's
// sum takes the same accepted atoms in the same order).  Tile-masked launches march two.
cudaError_t launch_column_fp64_ring(const ColumnJob* d_jobs, int n_jobs, int tiles, int max_np, int slab_tier,
                                    bool masked, bool four, unsigned* work, const unsigned long long* counters,
                                    int64_t cap, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned), st);
  if (e != cudaSuccess || tiles <= 0) return e;
  if (masked) {
    if (max_np != 1) return cudaErrorInvalidValue;
    return ring64::launch_tier<1, true, 2>(slab_tier, d_jobs, n_jobs, tiles, work, counters, cap, st);
  }
  // four slices with one angle per pass (with more, the phases leave no registers for the
  // four slices' sums)
  if (four && max_np <= 1)
    return ring64::launch_tier<1, false, 4>(slab_tier, d_jobs, n_jobs, tiles, work, counters, cap, st);
  if (max_np <= 1) return ring64::launch_tier<1, false, 2>(slab_tier, d_jobs, n_jobs, tiles, work, counters, cap, st);
  if (max_np <= 2) return ring64::launch_tier<2, false, 2>(slab_tier, d_jobs, n_jobs, tiles, work, counters, cap, st);
  return ring64::launch_tier<4, false, 2>(slab_tier, d_jobs, n_jobs, tiles, work, counters, cap, st);
}

}  // namespace stem
