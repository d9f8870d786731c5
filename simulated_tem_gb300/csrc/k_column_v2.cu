// K2+K3, FP32, second generation: z-sorted slab ring and two slices per lane.
//
// Same computation as k_column_fp32 (the pixel loop of computeD2BI_img,
// Lib_DynamicalTwoBeamImaging.f90:1870-1900, with the neighbour search of
// Lib_LinkCell3D.f90:1515-1605 and the integrator of :2316-2480), organised to
// issue fewer instructions per voxel:
//
// * One warp owns an 8 x 4 patch of pixel columns, one lane per column, and
//   advances two depth slices per step.  Both slices share each candidate's
//   load and its x-y distance; their z distances and r^2 are one packed
//   FP32x2 subtraction and one packed FP32x2 fused multiply-add.
// * Candidates live in a ring of four link-cell slabs (unwrapped z cells)
//   in warp-private shared memory.  A slab is gathered once, when the march
//   first needs it: the atoms of its cells in the patch footprint that lie
//   within 3 sigma of the patch rectangle in x-y, then ordered by z bin (32
//   bins per cell height, a counting sort).  A step scans, per slab, only the
//   bins that overlap the z-window [z0 - 3 sigma, z1 + 3 sigma].
// * Lengths are scaled by s = sqrt(log2 e / (2 sigma^2)), so the weight
//   exp(-r^2 / 2 sigma^2) is one ex2 of the negated scaled r^2, selected to
//   zero beyond the cutoff without a branch; both slices accumulate with
//   packed FP32x2 multiply-adds.
// * The RK4 double step (ii, ii+1, ii+2) runs once per step in registers for
//   every precession angle; the periodic closure uses the saved first sample.
// * The march does no FP64 arithmetic: the slice depths come from a per-image
//   table of FP32 values that the host computes in FP64.
//
// It needs link cells at least 3 sigma wide in x and y (the reference's grid always
// makes them so); in z it applies the 27-cell rule itself, slab by slab, so cells
// shorter than 3 sigma (a z voxel a little smaller than the in-plane one) give the
// reference's truncated search.  At most CAPS staged atoms per
// slab (128, then 192 and 256 for dense footprints such as coarse voxel grids);
// otherwise it raises counters[4] and the host retries with the next capacity, then
// with k_column_fp32, which handles both cases.  The capacity does not change which
// candidates are tested or their order: every instance computes the same image.
#include <cuda_runtime.h>

#include <cfloat>

#include "internal.h"

namespace stem {
namespace {

constexpr int kWarps = 4;
constexpr int kTileX = 8, kTileY = 4;
constexpr int kRing = 4;    // resident slabs (unwrapped z cells u, slot u & 3)
constexpr float kHuge1 = FLT_MAX;

constexpr int kBins = 32;  // z bins per slab for the window lookup

template <int CAPS>  // staged atoms per slab
struct WarpSmem {
  float4 p[kRing][CAPS];      // X', Y' (warp frame), z (own cell), cos -- lengths scaled by s
  float s[kRing][CAPS];       // sin
  int bin[kRing][kBins + 1];  // bin[b]: first atom of z bin b (width a33 s / kBins); bin[kBins] = count
  int count[kRing];
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int pos_mod(int a, int n) {
  const int r = a % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ int floor_div(int a, int n) { return (a >= 0) ? a / n : -((-a + n - 1) / n); }

// Lengths inside the kernel are scaled by s = sqrt(log2(e) / (2 sigma^2)), so that the
// Gaussian weight exp(-r^2 / (2 sigma^2)) is ex2(-r'^2) of the scaled distance r'.
struct Geo {
  int ux_lo, ux_hi, uy_lo, uy_hi, ux_ref, uy_ref;
  float xmin, xmax, ymin, ymax, pre2;
  float a11s, a22s, a33s, scale;
};

// Gather slab u (its cells in the patch footprint, atoms within 3 sigma of the
// patch rectangle) into its ring slot and order it by z bin in place; false
// when it holds more than CAPS atoms.
template <int CAPS>
__device__ bool load_slab(const ColumnParams& p, const Geo& G, int u, WarpSmem<CAPS>& W, int lane) {
  const int cz = pos_mod(u, p.Ez);
  const int slot = u & (kRing - 1);
  float4* P = W.p[slot];
  float* S = W.s[slot];
  int n = 0;
  for (int uy = G.uy_lo; uy <= G.uy_hi; ++uy) {
    const int cy = pos_mod(uy, p.Ey);
    const int64_t row_base = (int64_t)p.Ex * (cy + (int64_t)p.Ey * cz);
    const float yoff = G.a22s * (float)(uy - G.uy_ref);
    for (int ux = G.ux_lo; ux <= G.ux_hi;) {
      const int k = floor_div(ux, p.Ex);
      const int run_hi = min(G.ux_hi, (k + 1) * p.Ex - 1);
      const int shift = k * p.Ex;
      const int a_lo = p.cell_start[row_base + (ux - shift)];
      const int a_hi = p.cell_start[row_base + (run_hi - shift) + 1];
      for (int b = a_lo; b < a_hi; b += 32) {
        const int j = b + lane;
        bool keep = false;
        float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
        float sn = 0.f;
        if (j < a_hi) {
          const float4 r = p.p32[j];
          const int packed = __float_as_int(r.w);
          const int cxu = (packed & 1023) + shift;
          const float X = fmaf(r.x, G.scale, G.a11s * (float)(cxu - G.ux_ref));
          const float Y = fmaf(r.y, G.scale, yoff);
          const float dx = fmaxf(0.f, fmaxf(G.xmin - X, X - G.xmax));
          const float dy = fmaxf(0.f, fmaxf(G.ymin - Y, Y - G.ymax));
          keep = dx * dx + dy * dy <= G.pre2;
          const float2 cs = p.cs32[j];
          rec = make_float4(X, Y, r.z * G.scale, cs.x);
          sn = cs.y;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        const int cnt = __popc(m);
        if (n + cnt > CAPS) return false;
        if (keep) {
          const int d = n + __popc(m & ((1u << lane) - 1));
          P[d] = rec;
          S[d] = sn;
        }
        n += cnt;
      }
      ux = run_hi + 1;
    }
  }
  __syncwarp();
  // counting sort by z bin, in place: every lane first holds its atoms in registers;
  // within a bin the gather order is kept (deterministic)
  constexpr int kPer = CAPS / 32;
  const float inv_bin = kBins / G.a33s;
  int* hist = W.bin[slot];
  for (int b = lane; b <= kBins; b += 32) hist[b] = 0;
  __syncwarp();
  float4 e[kPer];
  float es[kPer];
  int eb[kPer], er[kPer];
  const unsigned lt = (1u << lane) - 1;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int i = lane + 32 * k;
    const bool valid = i < n;
    e[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    es[k] = 0.f;
    eb[k] = 0;
    er[k] = 0;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      e[k] = P[i];
      es[k] = S[i];
      eb[k] = min(kBins - 1, max(0, (int)floorf(e[k].z * inv_bin)));
      const unsigned m = __match_any_sync(act, eb[k]);
      er[k] = hist[eb[k]] + __popc(m & lt);
      __syncwarp(act);
      if ((m & lt) == 0) hist[eb[k]] += __popc(m);  // the group's first lane counts it
    }
    __syncwarp();
  }
  // exclusive scan of the 32 bin counts: bin starts, bin[kBins] = n
  {
    const int v = hist[lane];
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    __syncwarp();
    hist[lane] = incl - v;
    if (lane == 0) hist[kBins] = n;
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    if (lane + 32 * k < n) {
      const int d = hist[eb[k]] + er[k];
      P[d] = e[k];
      S[d] = es[k];
    }
  }
  __syncwarp();
  if (lane == 0) W.count[slot] = n;
  __syncwarp();
  return true;
}

struct Sample {
  float c0, cgr, cgi;
};

__device__ __forceinline__ void deriv(const Sample& s, float a, const float* ph, float* d) {
  const float ca = s.c0 + a;
  d[0] = -s.c0 * ph[1] - s.cgi * ph[2] - s.cgr * ph[3];
  d[1] = s.c0 * ph[0] + s.cgr * ph[2] - s.cgi * ph[3];
  d[2] = s.cgi * ph[0] - s.cgr * ph[1] - ca * ph[3];
  d[3] = s.cgr * ph[0] + s.cgi * ph[1] + ca * ph[2];
}

__device__ __forceinline__ void rk4(const Sample& s0, const Sample& s1, const Sample& s2, float a, float dz,
                                    float* ph) {
  float d[4], p1[4], q[4];
  const float dz3 = dz / 3.f, dz23 = 2.f * dz / 3.f, dz2 = 2.f * dz;
  deriv(s0, a, ph, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    p1[i] = ph[i] + d[i] * dz3;
    q[i] = ph[i] + d[i] * dz;
  }
  deriv(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = ph[i] + d[i] * dz;
    p1[i] = p1[i] + d[i] * dz23;
  }
  deriv(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = ph[i] + d[i] * dz2;
    p1[i] = p1[i] + d[i] * dz23;
  }
  deriv(s2, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = p1[i] + d[i] * dz3;
  const float inv = rsqrtf(ph[0] * ph[0] + ph[1] * ph[1] + ph[2] * ph[2] + ph[3] * ph[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] *= inv;
}

__device__ __forceinline__ float rho_of(float r2min, float sig) {
  if (r2min < sig * sig) return 1.f;
  if (r2min > 4.f * sig * sig) return 0.f;
  const float xx = sqrtf(r2min) / sig - 1.f;
  return 1.f - xx * xx * xx * (10.f - 15.f * xx + 6.f * xx * xx);
}

template <bool kDensity>
__device__ __forceinline__ Sample make_sample(float sr, float si, float r2min, float b0, float bg, float sig,
                                              bool use_density) {
  const float inv = rsqrtf(fmaxf(fmaf(sr, sr, si * si), 1e-32f));  // x = S / max(1e-16, |S|)
  const float rho = (kDensity && use_density) ? rho_of(r2min, sig) : 1.f;
  return Sample{b0 * rho, bg * rho * (sr * inv), bg * rho * (si * inv)};
}

// One warp tile of one image: the 8 x 4 columns of tile `tile` marched through
// the depth.  Returns false when a slab overflows its staging (counters[4]).
template <int NP, bool kDensity, bool kStats, int CAPS>
__device__ __noinline__ bool column_tile(const ColumnParams& p, WarpSmem<CAPS>& W, int tile, int lane) {
  const int Wd = p.ix1 - p.ix0;
  const int tiles_x = (Wd + kTileX - 1) / kTileX;
  const int tx = tile % tiles_x, ty = tile / tiles_x;
  const int ix = p.ix0 + tx * kTileX + (lane & (kTileX - 1));
  const int iy = p.iy0 + ty * kTileY + lane / kTileX;
  const bool active = ix < p.ix1 && iy < p.iy1;

  // s = sqrt(log2(e) / (2 sigma^2)): exp(-r^2 / (2 sigma^2)) = ex2(-(s r)^2)
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
  const float cut2 = (float)(p.cut2 * sd * sd);        // (3 sigma)^2 in scaled units
  const float r3 = sqrtf(cut2) * 1.0001f + 1e-4f;      // z-window half width, rounded up
  G.pre2 = cut2 * 1.0002f + 1e-3f;
  const float inv_bin = kBins / G.a33s;
  const float sig = (float)p.sigma, b0 = (float)p.b0, bg = (float)p.bg, dzs = (float)p.dz;
  const float r2_to_A2 = (float)(1.0 / (sd * sd));    // scaled r^2 back to A^2 (density)

  const int np = min(NP, p.n_prec - p.prec_offset);
  // the precession coefficients a_k stay in registers for few angles; for many they are
  // read from L1 at each step, which leaves the registers to the phases
  constexpr bool kAaReg = NP <= 4;
  const float* __restrict__ aag = p.aaf + p.prec_offset;
  float aa[kAaReg ? NP : 1], ph[NP][4];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    if (kAaReg) aa[k] = (k < np) ? aag[k] : 0.f;
    ph[k][0] = 1.f;
    ph[k][1] = ph[k][2] = ph[k][3] = 0.f;
  }
  Sample s_first{0.f, 0.f, 0.f}, s_prev{0.f, 0.f, 0.f}, s_mid{0.f, 0.f, 0.f};
  int ring_lo = 1 << 30, ring_hi = (1 << 30) - 1;  // empty
  unsigned n_acc = 0;
  unsigned long long n_tst = 0;

  for (int z0 = 0; z0 < p.Mz; z0 += 2) {
    const bool has1 = z0 + 1 < p.Mz;
    // home cells and slice depths (scaled, relative to the origin of home cell hz0)
    const int2 e0 = p.ztab[z0];
    const int2 e1 = has1 ? p.ztab[z0 + 1] : e0;
    const int hz0 = e0.x, hz1 = e1.x;
    const float zv0 = __int_as_float(e0.y), zv1 = __int_as_float(e1.y);
    const int need_lo = hz0 - 1, need_hi = hz1 + 1;
    if (need_lo > ring_hi || need_hi < ring_lo) {
      ring_lo = need_lo;
      ring_hi = need_lo - 1;
    }
    if (ring_lo < need_lo) ring_lo = need_lo;
    bool ok = true;
    while (ring_hi < need_hi && ok) {
      ++ring_hi;
      ok = load_slab<CAPS>(p, G, ring_hi, W, lane);
    }
    if (!ok) {
      if (lane == 0) atomicExch(&p.counters[4], 1ull);
      return false;  // the host recomputes the image with the general kernel
    }
    // two accumulator sets (even / odd candidates) for instruction-level parallelism;
    // .x is slice z0, .y slice z0 + 1
    float2 srA = make_float2(0.f, 0.f), siA = srA, srB = srA, siB = srA;
    float2 rmA = make_float2(kHuge1, kHuge1), rmB = rmA;
    for (int u = need_lo; u <= need_hi; ++u) {
      const int slot = u & (kRing - 1);
      const float zoff = G.a33s * (float)(u - hz0);  // cell u's origin relative to hz0's
      const float t0 = zv0 - zoff, t1 = zv1 - zoff;
      float w_lo = t0, w_hi = t1;
      // a missing second slice (odd depth) sits far away and accepts nothing
      float2 tt = make_float2(-t0, has1 ? -t1 : -1e30f);
      if (p.trunc_z) {
        // z cells shorter than 3 sigma: the reference searches only the 27 cells around each
        // voxel's home cell, so slab u serves a slice only within one cell of its home z cell
        // (with taller cells nothing farther lies within the cutoff)
        const bool v0 = u - hz0 >= -1 && u - hz0 <= 1;
        const bool v1 = has1 && u - hz1 >= -1 && u - hz1 <= 1;
        w_lo = v0 ? t0 : t1;
        w_hi = v1 ? t1 : t0;
        tt = make_float2(v0 ? -t0 : -1e30f, v1 ? -t1 : -1e30f);
      }
      const int b_lo = max(0, min(kBins, (int)floorf((w_lo - r3) * inv_bin)));
      const int b_hi = max(0, min(kBins, (int)ceilf((w_hi + r3) * inv_bin)));
      const int lo = W.bin[slot][b_lo];
      const int hi = W.bin[slot][b_hi];
      if (kStats) n_tst += (unsigned long long)(hi - lo);
      const float4* P = W.p[slot];
      const float* S = W.s[slot];
      int j = lo;
      for (; j + 1 < hi; j += 2) {
        const float4 qa = P[j], qb = P[j + 1];
        const float sa = S[j], sb = S[j + 1];
        const float dxa = qa.x - Xv, dya = qa.y - Yv, dxb = qb.x - Xv, dyb = qb.y - Yv;
        const float ha = fmaf(dxa, dxa, dya * dya), hb = fmaf(dxb, dxb, dyb * dyb);
        const float2 dza = __fadd2_rn(make_float2(qa.z, qa.z), tt);
        const float2 dzb = __fadd2_rn(make_float2(qb.z, qb.z), tt);
        const float2 ra = __ffma2_rn(dza, dza, make_float2(ha, ha));
        const float2 rb = __ffma2_rn(dzb, dzb, make_float2(hb, hb));
        const float2 wa = make_float2(ra.x <= cut2 ? ex2_approx(-ra.x) : 0.f, ra.y <= cut2 ? ex2_approx(-ra.y) : 0.f);
        const float2 wb = make_float2(rb.x <= cut2 ? ex2_approx(-rb.x) : 0.f, rb.y <= cut2 ? ex2_approx(-rb.y) : 0.f);
        srA = __ffma2_rn(wa, make_float2(qa.w, qa.w), srA);
        siA = __ffma2_rn(wa, make_float2(sa, sa), siA);
        srB = __ffma2_rn(wb, make_float2(qb.w, qb.w), srB);
        siB = __ffma2_rn(wb, make_float2(sb, sb), siB);
        if (kDensity) {
          // r_min over all tested candidates: a candidate beyond 3 sigma only lowers r_min
          // to a value beyond 2 sigma, where the density is 0 either way
          rmA.x = fminf(rmA.x, ra.x);
          rmA.y = fminf(rmA.y, ra.y);
          rmB.x = fminf(rmB.x, rb.x);
          rmB.y = fminf(rmB.y, rb.y);
        }
        if (kStats) n_acc += (ra.x <= cut2) + (ra.y <= cut2) + (rb.x <= cut2) + (rb.y <= cut2);
      }
      if (j < hi) {
        const float4 qa = P[j];
        const float sa = S[j];
        const float dxa = qa.x - Xv, dya = qa.y - Yv;
        const float ha = fmaf(dxa, dxa, dya * dya);
        const float2 dza = __fadd2_rn(make_float2(qa.z, qa.z), tt);
        const float2 ra = __ffma2_rn(dza, dza, make_float2(ha, ha));
        const float2 wa = make_float2(ra.x <= cut2 ? ex2_approx(-ra.x) : 0.f, ra.y <= cut2 ? ex2_approx(-ra.y) : 0.f);
        srA = __ffma2_rn(wa, make_float2(qa.w, qa.w), srA);
        siA = __ffma2_rn(wa, make_float2(sa, sa), siA);
        if (kDensity) {
          rmA.x = fminf(rmA.x, ra.x);
          rmA.y = fminf(rmA.y, ra.y);
        }
        if (kStats) n_acc += (ra.x <= cut2) + (ra.y <= cut2);
      }
    }
    const float2 sr = __fadd2_rn(srA, srB), si = __fadd2_rn(siA, siB);
    const float rm0 = fminf(rmA.x, rmB.x) * r2_to_A2, rm1 = fminf(rmA.y, rmB.y) * r2_to_A2;
    // field samples z0 (even) and z0 + 1 (odd), then the RK4 double step (z0-2, z0-1, z0)
    const Sample s0 = make_sample<kDensity>(sr.x, si.x, rm0, b0, bg, sig, p.use_density != 0);
    if (z0 == 0) {
      s_first = s0;
    } else {
#pragma unroll
      for (int k = 0; k < NP; ++k)
        if (k < np) rk4(s_prev, s_mid, s0, kAaReg ? aa[k] : __ldg(aag + k), dzs, ph[k]);
    }
    s_prev = s0;
    if (has1) s_mid = make_sample<kDensity>(sr.y, si.y, rm1, b0, bg, sig, p.use_density != 0);
  }
  if ((p.Mz & 1) == 0) {  // closure x(Mz) = x(0)
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) rk4(s_prev, s_mid, s_first, kAaReg ? aa[k] : __ldg(aag + k), dzs, ph[k]);
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < NP; ++k)
    if (k < np) acc += ph[k][2] * ph[k][2] + ph[k][3] * ph[k][3];
  if (active) {
    double* o = p.img + ix + (int64_t)p.Mx * iy;
    *o = p.accumulate ? *o + (double)acc : (double)acc;
  }
  if (kStats) {
    unsigned long long acc_w = active ? n_acc : 0u, tst_w = active ? 2 * n_tst : 0u;
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

// Persistent launch over the warp tiles of every job of a batch: each warp
// takes the next tile from a global counter, so images of uneven size share
// the GPU without a tail per image.
// kMasked: jobs may carry a tile mask (warp tiles outside it are skipped here, before the
// march, so that the unmasked instances carry no code for it).
template <int NP, bool kDensity, bool kStats, int kMinBlocks, int CAPS, bool kMasked = false>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks)
    k_column_fp32_v2(const ColumnJob* __restrict__ jobs, int n_jobs, int total_tiles, unsigned* __restrict__ work,
                     const unsigned long long* __restrict__ counters, int64_t cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpSmem<CAPS>& W = reinterpret_cast<WarpSmem<CAPS>*>(smem_raw)[warp];
  if ((int64_t)counters[0] > cap) return;  // the binning overflowed: the host retries
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = (int)atomicAdd(work, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= total_tiles) break;
    if (counters[4] != 0) break;  // a slab overflowed: the batch is recomputed image by image
    int lo = 0, hi = n_jobs - 1;  // job of this tile
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile_base[0] <= tile)
        lo = mid;
      else
        hi = mid - 1;
    }
    if constexpr (kMasked) {
      const ColumnParams& P = jobs[lo].p;
      const int local = tile - jobs[lo].tile_base[0];
      const int tiles_x = (P.ix1 - P.ix0 + kTileX - 1) / kTileX;
      if (!tile_wanted(P, local % tiles_x, local / tiles_x, kTileX, kTileY)) continue;
    }
    if (!column_tile<NP, kDensity, kStats, CAPS>(jobs[lo].p, W, tile - jobs[lo].tile_base[0], lane)) break;
  }
}

template <int CAPS, typename K>
cudaError_t launch(K kernel, const ColumnJob* jobs, int n_jobs, int total_tiles, unsigned* work,
                   const unsigned long long* counters, int64_t cap, int blocks_per_sm, cudaStream_t st) {
  const size_t smem = sizeof(WarpSmem<CAPS>) * kWarps;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * blocks_per_sm;
  const int need = (total_tiles + kWarps - 1) / kWarps;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  ++launch_count();
  kernel<<<grid, kWarps * 32, smem, st>>>(jobs, n_jobs, total_tiles, work, counters, cap);
  return cudaGetLastError();
}

// Occupancy variants: variant v sets the register budget for (base - v) CTAs per SM,
// base = 5 for up to 8 precession angles per pass (96 registers), 4 for 16 (128).  The
// arithmetic is the same in every variant; the host's autotuner picks by timing.
constexpr int kVariants = 2;

template <int NP, bool kDensity, bool kStats>
cudaError_t launch_v(int v, int tier, const ColumnJob* jobs, int n_jobs, int total_tiles, unsigned* work,
                     const unsigned long long* counters, int64_t cap, cudaStream_t st) {
  constexpr int B = NP <= 8 ? 5 : 4;
  if (tier >= 2)  // 256-atom slabs: 84 KB of shared memory per CTA, two CTAs per SM
    return launch<256>(k_column_fp32_v2<NP, kDensity, kStats, 2, 256>, jobs, n_jobs, total_tiles, work, counters,
                       cap, 2, st);
  if (tier == 1)  // 192-atom slabs: 63.6 KB per CTA, three CTAs per SM
    return launch<192>(k_column_fp32_v2<NP, kDensity, kStats, 3, 192>, jobs, n_jobs, total_tiles, work, counters,
                       cap, 3, st);
  if constexpr (!kStats) {
    if (v == 1)
      return launch<128>(k_column_fp32_v2<NP, kDensity, kStats, B - 1, 128>, jobs, n_jobs, total_tiles, work, counters,
                         cap, B - 1, st);
  }
  return launch<128>(k_column_fp32_v2<NP, kDensity, kStats, B, 128>, jobs, n_jobs, total_tiles, work, counters, cap, B,
                     st);
}

template <bool kDensity, bool kStats>
cudaError_t launch_np(int np, int v, int big, const ColumnJob* jobs, int n_jobs, int total_tiles, unsigned* work,
                      const unsigned long long* counters, int64_t cap, cudaStream_t st) {
  if (np <= 1) return launch_v<1, kDensity, kStats>(v, big, jobs, n_jobs, total_tiles, work, counters, cap, st);
  if (np <= 2) return launch_v<2, kDensity, kStats>(v, big, jobs, n_jobs, total_tiles, work, counters, cap, st);
  if (np <= 4) return launch_v<4, kDensity, kStats>(v, big, jobs, n_jobs, total_tiles, work, counters, cap, st);
  if (np <= 8) return launch_v<8, kDensity, kStats>(v, big, jobs, n_jobs, total_tiles, work, counters, cap, st);
  return launch_v<16, kDensity, kStats>(v, big, jobs, n_jobs, total_tiles, work, counters, cap, st);
}

}  // namespace

cudaError_t launch_column_fp32_ring_v2(const ColumnJob* d_jobs, int n_jobs, int total_tiles, int max_np, bool density,
                                       bool stats, int variant, int slab_tier, bool masked, unsigned* work,
                                       const unsigned long long* counters, int64_t cap, cudaStream_t st) {
  cudaMemsetAsync(work, 0, sizeof(unsigned), st);
  if (total_tiles <= 0) return cudaSuccess;
  if (masked) {  // tile-masked jobs: one precession angle, no statistics (the host sends others elsewhere)
    if (max_np != 1 || stats) return cudaErrorInvalidValue;
    if (slab_tier >= 2)
      return density ? launch<256>(k_column_fp32_v2<1, true, false, 2, 256, true>, d_jobs, n_jobs, total_tiles, work,
                                   counters, cap, 2, st)
                     : launch<256>(k_column_fp32_v2<1, false, false, 2, 256, true>, d_jobs, n_jobs, total_tiles, work,
                                   counters, cap, 2, st);
    if (slab_tier == 1)
      return density ? launch<192>(k_column_fp32_v2<1, true, false, 3, 192, true>, d_jobs, n_jobs, total_tiles, work,
                                   counters, cap, 3, st)
                     : launch<192>(k_column_fp32_v2<1, false, false, 3, 192, true>, d_jobs, n_jobs, total_tiles, work,
                                   counters, cap, 3, st);
    return density ? launch<128>(k_column_fp32_v2<1, true, false, 5, 128, true>, d_jobs, n_jobs, total_tiles, work,
                                 counters, cap, 5, st)
                   : launch<128>(k_column_fp32_v2<1, false, false, 5, 128, true>, d_jobs, n_jobs, total_tiles, work,
                                 counters, cap, 5, st);
  }
  const int v = (variant > 0 && variant < kVariants && !stats) ? variant : 0;  // statistics: variant 0
  const int b = slab_tier;
  if (density)
    return stats ? launch_np<true, true>(max_np, v, b, d_jobs, n_jobs, total_tiles, work, counters, cap, st)
                 : launch_np<true, false>(max_np, v, b, d_jobs, n_jobs, total_tiles, work, counters, cap, st);
  return stats ? launch_np<false, true>(max_np, v, b, d_jobs, n_jobs, total_tiles, work, counters, cap, st)
               : launch_np<false, false>(max_np, v, b, d_jobs, n_jobs, total_tiles, work, counters, cap, st);
}

}  // namespace stem
