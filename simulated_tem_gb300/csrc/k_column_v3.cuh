// K2+K3, FP32: the slab-ring column kernel with separable weights and a per-step
// candidate buffer.
//
// The pixel loop of computeD2BI_img (Lib_DynamicalTwoBeamImaging.f90:1870-1900), with the
// neighbour search of Lib_LinkCell3D.f90:1515-1605 and the integrator of :2316-2480, for
// the FP32 path (k_column_fp32 in k_column.cu is the general form, for any cell size and
// slab occupancy).
//
// One warp owns a patch of 32 pixel columns (8 x 4, 4 x 8 or 16 x 2), one lane per
// column, advancing two depth slices per step.  The atoms of the link-cell slabs the
// march needs (one slab per z cell, a ring of four) are staged in warp-private shared
// memory once, prefiltered to 3 sigma of the patch and ordered by z bin, so that a step
// visits only the bins overlapping its depth window.  Within a step:
//
// * Every column of a patch samples the same two depths, so everything that depends
//   only on an atom and the depth is the same in all 32 lanes.  A cooperative pass
//   (one candidate per lane) computes it once per atom and step: the z distances,
//   the largest in-plane r^2 each slice still accepts (hmax_k = (3 sigma)^2 - dz_k^2,
//   or -1 where the reference's 27-cell rule excludes the slab for that slice), and
//   the z factor of the Gaussian times the atom's phasor, ex2(-dz_k^2) (cos, sin).
// * The Gaussian is separable, exp(-r^2/2s^2) = exp(-dxy^2/2s^2) exp(-dz^2/2s^2), so a
//   lane needs one ex2 per atom (its in-plane factor) for both slices, and the
//   inclusive cutoff r^2 <= (3 sigma)^2 becomes dxy^2 <= hmax_k.
// * The same pass drops atoms that no column of the patch accepts at either slice
//   (distance to the patch's sample rectangle beyond sqrt(hmax)), so the lanes test
//   the patch's sphere-dilated box instead of its cylinder-dilated one, and compacts
//   the rest into a small per-warp buffer (ballot + popc, order kept) that all lanes
//   then read with two 16-byte loads per atom.
//
// Per atom and lane: two loads, the in-plane distance (3 FP32 ops), one ex2, two
// compares and two predicated FP32x2 multiply-adds (both slices' cos and sin); the loop
// runs four atom pairs per iteration, because at the 18-20 warps per SM that the
// registers and shared memory allow, the kernel is bound by dependent-instruction
// latency rather than by any pipe.
//
// Precision: FP32 throughout the march; the weight is the product of two ex2 values (a
// few ulp).  The FP32 cutoff test may decide an atom within rounding of the cutoff
// differently from the reference; columns whose field sum is small enough for that to
// matter re-decide those atoms in the reference's FP64 arithmetic (exact_fix below).
#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <type_traits>

#include "internal.h"

namespace stem {
namespace ring3 {

constexpr int kWarps = 4;
constexpr int kRing = 4;    // resident slabs (unwrapped z cells u, slot u & 3)
constexpr int kBins = 32;   // z bins per slab for the window lookup (at most 32: one lane each)
constexpr int kBuf = 64;    // per-step candidate buffer (flushed at 32)
constexpr float kHuge = FLT_MAX;

// Lengths inside the kernel are scaled by s = sqrt(log2(e) / (2 sigma^2)), so that the
// Gaussian weight exp(-r^2 / (2 sigma^2)) is ex2(-r'^2) of the scaled distance r'.
struct Geo {
  int ux_lo, ux_hi, uy_lo, uy_hi, ux_ref, uy_ref;
  float xmin, xmax, ymin, ymax, pre2;
  float a11s, a22s, a33s, scale;
};

// Scalars of a tile's march, the same in every lane (scaled units where lengths).
struct TileConst {
  float cut2;      // (3 sigma)^2
  float r3;        // z-window half width, rounded up
  float inv_bin;   // z bins per scaled length
  float b0, bg, sig, dzs;
  float r2_to_A2;  // scaled r^2 back to A^2 (density)
};

template <int CAPS>  // staged atoms per slab
struct WarpSmem3 {
  static_assert(CAPS % 32 == 0, "the z sort holds CAPS / 32 atoms per lane");
  float4 p[kRing][CAPS];      // X', Y' (warp frame), z (own cell), phase (cycles) -- lengths scaled by s
  int gi[kRing][CAPS];        // index of the kept atom (its records in global memory)
  int bin[kRing][kBins + 1];  // bin[b]: first atom of z bin b; bin[kBins] = count
  int count[kRing];
  float4 ba[kBuf];            // step buffer: X', Y', hmax_0, hmax_1
  float4 be[kBuf];            // ex2(-dz_0^2) (cos, sin), ex2(-dz_1^2) (cos, sin)
  Geo geo;                    // the tile's footprint and frame (one angle per pass: here, not in registers)
  TileConst tc;               // the tile's scalar constants (likewise)
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

// One gathered candidate: atom j of a cell in row uy, x cells shifted by `shift` (an
// unwrapped run), in the warp's scaled frame; keep when within 3 sigma of the patch.
template <bool kCellCode>
__device__ __forceinline__ bool slab_candidate(const ColumnParams& p, const Geo& G, int j, int shift, int uy,
                                               float4& rec) {
  const float4 r = p.p32[j];
  const int packed = __float_as_int(r.w);
  const int cxu = (packed & 1023) + shift;
  const float X = __fmaf_rn(r.x, G.scale, __fmul_rn(G.a11s, (float)(cxu - G.ux_ref)));
  const float Y = __fmaf_rn(r.y, G.scale, __fmul_rn(G.a22s, (float)(uy - G.uy_ref)));
  const float dx = fmaxf(0.f, fmaxf(G.xmin - X, X - G.xmax));
  const float dy = fmaxf(0.f, fmaxf(G.ymin - Y, Y - G.ymax));
  const float w4 = kCellCode ? __int_as_float((cxu - G.ux_ref + 8) | ((uy - G.uy_ref + 8) << 8)) : p.ph32[j];
  rec = make_float4(X, Y, __fmul_rn(r.z, G.scale), w4);
  return dx * dx + dy * dy <= G.pre2;
}

// Appends the kept candidates of one 32-lane round (ballot + popc, order kept); false
// when the slab would exceed CAPS.
template <int CAPS>
__device__ __forceinline__ bool slab_append(float4* P, int* GI, int& n, bool keep, const float4& rec, int j,
                                            int lane) {
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  const int cnt = __popc(m);
  if (n + cnt > CAPS) return false;
  if (keep) {
    const int d = n + __popc(m & ((1u << lane) - 1));
    P[d] = rec;
    GI[d] = j;
  }
  n += cnt;
  return true;
}

// Gather slab u (its cells in the patch footprint, atoms within 3 sigma of the
// patch rectangle) into its ring slot and order it by z bin in place; false
// when it holds more than CAPS atoms.
// kCellCode: the fourth float of an entry holds the atom's unwrapped cell relative to the warp's
// reference cells, (ux - ux_ref + 8) | (uy - uy_ref + 8) << 8 (the FP64 kernel's exact
// distances need it), instead of its phase.  WS: any warp-memory layout with the slab
// arrays p, gi, bin and count.
//
// The footprint is rows uy of x runs (a run ends where x wraps): segments of consecutive
// atoms.  With kJoined and up to 8 segments, the lanes look up all segment ranges at once,
// join them into one index space (the slot's bin array, free until the sort, holds the
// table) and gather two 32-lane rounds at a time; otherwise row by row, one round at a
// time (with more than one angle per pass the march's phases leave no registers for a
// second round: measured, 16 angles spilled more and ran 10 % slower).  Both
// routes visit the atoms in the same order (rows, runs, atoms), so the slab's contents
// and order do not depend on the route.
template <int CAPS, bool kCellCode = false, bool kJoined = true, typename WS>
__device__ bool load_slab3(const ColumnParams& p, const Geo& G, int u, WS& W, int lane) {
  const int cz = pos_mod(u, p.Ez);
  const int slot = u & (kRing - 1);
  float4* P = W.p[slot];
  int* GI = W.gi[slot];
  int n = 0;
  constexpr int kMaxSeg = 8;
  static_assert(4 * kMaxSeg + 1 <= kBins + 1, "the segment table lives in a slot's bin array");
  const int k_lo = floor_div(G.ux_lo, p.Ex), k_hi = floor_div(G.ux_hi, p.Ex);
  const int n_run = max(0, k_hi - k_lo + 1), n_seg = max(0, G.uy_hi - G.uy_lo + 1) * n_run;
  if (kJoined && n_seg >= 1 && n_seg <= kMaxSeg) {
    int* seg = W.bin[slot];  // per segment: first index, first atom, x shift, row; then the total
    int len = 0, a_lo = 0, shift = 0, uy = 0;
    if (lane < n_seg) {
      const int k = k_lo + lane % n_run;
      uy = G.uy_lo + lane / n_run;
      shift = k * p.Ex;
      const int x0 = max(G.ux_lo, shift), x1 = min(G.ux_hi, shift + p.Ex - 1);
      const int64_t row_base = (int64_t)p.Ex * (pos_mod(uy, p.Ey) + (int64_t)p.Ey * cz);
      a_lo = p.cell_start[row_base + (x0 - shift)];
      len = p.cell_start[row_base + (x1 - shift) + 1] - a_lo;
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < kMaxSeg; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, kMaxSeg - 1);
    if (lane < n_seg) {
      seg[4 * lane] = incl - len;
      seg[4 * lane + 1] = a_lo;
      seg[4 * lane + 2] = shift;
      seg[4 * lane + 3] = uy;
    }
    if (lane == 0) seg[4 * n_seg] = total;
    __syncwarp();
    int sg = 0;  // this lane's segment (its indices only grow)
    auto locate = [&](int i, int& j, int& sh, int& y) {
      while (i >= seg[4 * (sg + 1)]) ++sg;
      j = seg[4 * sg + 1] + (i - seg[4 * sg]);
      sh = seg[4 * sg + 2];
      y = seg[4 * sg + 3];
    };
    constexpr int kRounds = 2;
    for (int b = 0; b < total; b += 32 * kRounds) {
      int j[kRounds];
      bool keep[kRounds];
      float4 rec[kRounds];
#pragma unroll
      for (int r = 0; r < kRounds; ++r) {
        const int i = b + 32 * r + lane;
        int sh = 0, y = 0;
        j[r] = 0;
        keep[r] = false;
        rec[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < total) {
          locate(i, j[r], sh, y);
          keep[r] = slab_candidate<kCellCode>(p, G, j[r], sh, y, rec[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < kRounds; ++r)
        if (b + 32 * r < total && !slab_append<CAPS>(P, GI, n, keep[r], rec[r], j[r], lane)) return false;
    }
  } else {
    for (int uy = G.uy_lo; uy <= G.uy_hi; ++uy) {
      const int64_t row_base = (int64_t)p.Ex * (pos_mod(uy, p.Ey) + (int64_t)p.Ey * cz);
      for (int k = k_lo; k <= k_hi; ++k) {
        const int shift = k * p.Ex;
        const int x0 = max(G.ux_lo, shift), x1 = min(G.ux_hi, shift + p.Ex - 1);
        const int a_lo = p.cell_start[row_base + (x0 - shift)];
        const int a_hi = p.cell_start[row_base + (x1 - shift) + 1];
        for (int b = a_lo; b < a_hi; b += 32) {
          const int j = b + lane;
          bool keep = false;
          float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j < a_hi) keep = slab_candidate<kCellCode>(p, G, j, shift, uy, rec);
          if (!slab_append<CAPS>(P, GI, n, keep, rec, j, lane)) return false;
        }
      }
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
  int es[kPer];
  int eb[kPer], er[kPer];
  const unsigned lt = (1u << lane) - 1;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int i = lane + 32 * k;
    const bool valid = i < n;
    e[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    es[k] = 0;
    eb[k] = 0;
    er[k] = 0;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      e[k] = P[i];
      es[k] = GI[i];
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
    const int v = lane < kBins ? hist[lane] : 0;
    int incl = v;
    for (int o = 1; o < kBins; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    __syncwarp();
    if (lane < kBins) hist[lane] = incl - v;
    if (lane == 0) hist[kBins] = n;
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    if (lane + 32 * k < n) {
      const int d = hist[eb[k]] + er[k];
      P[d] = e[k];
      GI[d] = es[k];
    }
  }
  __syncwarp();
  if (lane == 0) W.count[slot] = n;
  __syncwarp();
  return true;
}

// The RK4 double step in explicitly rounded operations, on one precession angle
// (float) or two (float2: .x angle k, .y angle k + 1, one FP32x2 instruction per
// operation).  Both forms round every operation the same way, so an angle's result
// does not depend on how many angles share the pass.
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float2 fma_(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float2 mul_(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float2 add_(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float neg_(float a) { return -a; }
__device__ __forceinline__ float2 neg_(float2 a) { return make_float2(-a.x, -a.y); }
template <typename T>
__device__ __forceinline__ T bc(float v);
template <>
__device__ __forceinline__ float bc<float>(float v) { return v; }
template <>
__device__ __forceinline__ float2 bc<float2>(float v) { return make_float2(v, v); }
__device__ __forceinline__ float rsq_(float a) { return rsqrtf(a); }
__device__ __forceinline__ float2 rsq_(float2 a) { return make_float2(rsqrtf(a.x), rsqrtf(a.y)); }

struct Sample {
  float c0, cgr, cgi;
};

template <typename T>
struct SampleT {
  T c0, cgr, cgi;
};

template <typename T>
__device__ __forceinline__ SampleT<T> widen(const Sample& s) {
  return SampleT<T>{bc<T>(s.c0), bc<T>(s.cgr), bc<T>(s.cgi)};
}

// d/dz (phi_0, phi_g) of the reference's two-beam equations (:2375-2380), phases as
// (Re phi_0, Im phi_0, Re phi_g, Im phi_g)
template <typename T>
__device__ __forceinline__ void deriv(const SampleT<T>& s, T a, const T* ph, T* d) {
  const T ca = add_(s.c0, a);
  d[0] = fma_(neg_(s.cgr), ph[3], fma_(neg_(s.cgi), ph[2], mul_(neg_(s.c0), ph[1])));
  d[1] = fma_(neg_(s.cgi), ph[3], fma_(s.cgr, ph[2], mul_(s.c0, ph[0])));
  d[2] = fma_(neg_(ca), ph[3], fma_(neg_(s.cgr), ph[1], mul_(s.cgi, ph[0])));
  d[3] = fma_(ca, ph[2], fma_(s.cgi, ph[1], mul_(s.cgr, ph[0])));
}

// One RK4 double step over samples (z-2, z-1, z) with weights dz/3, 2dz/3 (:2389-2464)
// and the renormalisation of the phases (:2466-2472).
template <typename T>
__device__ __forceinline__ void rk4(const SampleT<T>& s0, const SampleT<T>& s1, const SampleT<T>& s2, T a, float dzf,
                                    T* ph) {
  T d[4], p1[4], q[4];
  const T dz = bc<T>(dzf), dz3 = bc<T>(dzf / 3.f), dz23 = bc<T>(2.f * dzf / 3.f), dz2 = bc<T>(2.f * dzf);
  deriv(s0, a, ph, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    p1[i] = fma_(d[i], dz3, ph[i]);
    q[i] = fma_(d[i], dz, ph[i]);
  }
  deriv(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = fma_(d[i], dz, ph[i]);
    p1[i] = fma_(d[i], dz23, p1[i]);
  }
  deriv(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = fma_(d[i], dz2, ph[i]);
    p1[i] = fma_(d[i], dz23, p1[i]);
  }
  deriv(s2, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = fma_(d[i], dz3, p1[i]);
  const T inv = rsq_(fma_(ph[3], ph[3], fma_(ph[2], ph[2], fma_(ph[1], ph[1], mul_(ph[0], ph[0])))));
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = mul_(ph[i], inv);
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

// The lanes' half of a step: every buffered atom against the lane's column at both
// slices.  Two accumulator sets (even and odd atoms) for instruction-level
// parallelism; a*.x / a*.y are the real / imaginary sums, a0 slice z0, a1 slice z0 + 1.
// r2 minima (density) are kept as min(dxy^2 - hmax_k) = r^2 - (3 sigma)^2.
template <bool kDensity, bool kStats>
__device__ __forceinline__ void consume(const float4* __restrict__ BA, const float4* __restrict__ BE, int n, float Xv,
                                        float Yv, float2& a0A, float2& a1A, float2& a0B, float2& a1B, float2& rmA,
                                        float2& rmB, unsigned& n_acc) {
  int i = 0;
  // four pairs per iteration: their independent loads and chains hide the latencies that
  // bind this loop at 18-20 warps per SM (measured: 3.02 -> 2.81 ms on the 1.2M-atom image,
  // 5.23 -> 4.88 ms with 16 angles)
#pragma unroll 4
  for (; i + 1 < n; i += 2) {
    const float4 qa = BA[i], qb = BA[i + 1];
    const float4 ea = BE[i], eb = BE[i + 1];
    const float dxa = __fsub_rn(qa.x, Xv), dya = __fsub_rn(qa.y, Yv), dxb = __fsub_rn(qb.x, Xv),
                dyb = __fsub_rn(qb.y, Yv);
    const float ha = __fmaf_rn(dxa, dxa, __fmul_rn(dya, dya)), hb = __fmaf_rn(dxb, dxb, __fmul_rn(dyb, dyb));
    const float wa = ex2_approx(-ha), wb = ex2_approx(-hb);
    const float2 wa2 = make_float2(wa, wa), wb2 = make_float2(wb, wb);
    if (ha <= qa.z) a0A = __ffma2_rn(wa2, make_float2(ea.x, ea.y), a0A);
    if (ha <= qa.w) a1A = __ffma2_rn(wa2, make_float2(ea.z, ea.w), a1A);
    if (hb <= qb.z) a0B = __ffma2_rn(wb2, make_float2(eb.x, eb.y), a0B);
    if (hb <= qb.w) a1B = __ffma2_rn(wb2, make_float2(eb.z, eb.w), a1B);
    if (kDensity) {
      rmA.x = fminf(rmA.x, ha - qa.z);
      rmA.y = fminf(rmA.y, ha - qa.w);
      rmB.x = fminf(rmB.x, hb - qb.z);
      rmB.y = fminf(rmB.y, hb - qb.w);
    }
    if (kStats) n_acc += (ha <= qa.z) + (ha <= qa.w) + (hb <= qb.z) + (hb <= qb.w);
  }
  if (i < n) {
    const float4 qa = BA[i];
    const float4 ea = BE[i];
    const float dxa = __fsub_rn(qa.x, Xv), dya = __fsub_rn(qa.y, Yv);
    const float ha = __fmaf_rn(dxa, dxa, __fmul_rn(dya, dya));
    const float wa = ex2_approx(-ha);
    const float2 wa2 = make_float2(wa, wa);
    if (ha <= qa.z) a0A = __ffma2_rn(wa2, make_float2(ea.x, ea.y), a0A);
    if (ha <= qa.w) a1A = __ffma2_rn(wa2, make_float2(ea.z, ea.w), a1A);
    if (kDensity) {
      rmA.x = fminf(rmA.x, ha - qa.z);
      rmA.y = fminf(rmA.y, ha - qa.w);
    }
    if (kStats) n_acc += (ha <= qa.z) + (ha <= qa.w);
  }
}

// Precession coefficient (pair) k: from registers, or from the table (L1).  The table of
// a pass holds aa(prec_offset ...) and is read in pairs only below np, whose odd last
// angle pairs with a zero the host appends.
template <typename T, bool kReg>
__device__ __forceinline__ T aa_at(const T* aa, const float* __restrict__ aag, int k) {
  if constexpr (kReg) {
    return aa[k];
  } else if constexpr (std::is_same<T, float>::value) {
    return __ldg(aag + k);
  } else {
    return make_float2(__ldg(aag + 2 * k), __ldg(aag + 2 * k + 1));
  }
}

// The cutoff in the reference is an FP64 comparison, d.d <= (3 sigma)^2
// (Lib_LinkCell3D.f90:1594), and the phase field is discontinuous there: a voxel whose only
// neighbour lies at the cutoff has x = 0 on one side and a unit phasor on the other
// (S / max(1e-16, |S|), Lib_DynamicalTwoBeamImaging.f90:1877-1892).  The FP32 test may
// decide an atom within about 3e-5 (scaled r^2) of the cutoff differently.  That changes
// a voxel with many neighbours by a few 1e-6 in I at most, but a sparse one (a void's rim,
// or neighbours whose phases cancel) by up to 1e-2.  So after each step the columns whose
// field sum is small rescan the step's resident slabs, re-decide in the reference's FP64
// arithmetic every atom the FP32 test placed within kGuard of the cutoff, and correct the
// sum for each decision that changes.  The rescan repeats the march's FP32 operations on
// the same staged values, so it meets the same decisions; the FP64 distance uses the cell
// fractions the binning kept (2^-32 cells) and the reference's per-axis form
// d = a (f + (k - zi_frac)).
constexpr float kGuard = 1e-4f;  // scaled r^2; the FP32 test's error is below 3e-5
// |S|^2 below which a column re-decides its near-cutoff atoms.  A flipped atom weighs
// exp(-9/2) = 0.011 and moves x = S / |S| by at most 0.011 |e^(i phi) - x| / |S|; above
// |S| = 1/2, with the few-tenths-of-a-radian phase spread of neighbouring atoms, that
// changes I by a few 1e-5 at most.
constexpr float kSparse2 = 0.25f;

__device__ __forceinline__ int wrap_diff(int c, int h, int n) {  // c - h in -(n/2) .. n/2, periodic
  int d = c - h;
  if (d > n / 2) d -= n;
  else if (d < -(n / 2)) d += n;
  return d;
}

struct Slice {
  int hz;       // home z cell
  float zv;     // scaled depth from the origin of the step's even home cell
  double fz;    // fractional position in the home cell (FP64)
  bool want;    // this lane re-decides this slice
};

// One lane's exact re-decision of slice sl against staged atom j of `slot` (cell u).
template <int CAPS>
__device__ __forceinline__ void exact_one(const ColumnParams& p, const WarpSmem3<CAPS>& W, int slot, int j, float h,
                                          float dz, bool acc32, int hx, int hy, double fvx, double fvy,
                                          const Slice& sl, float2& S, int& dn) {
  const int gi = W.gi[slot][j];
  const int packed = __float_as_int(p.p32[gi].w);
  const int kx = wrap_diff(packed & 1023, hx, p.Ex), ky = wrap_diff((packed >> 10) & 1023, hy, p.Ey);
  const int kz = wrap_diff(packed >> 20, sl.hz, p.Ez);
  const uint4 fr = p.fr32[gi];
  const double fx = (double)fr.x * 2.3283064365386963e-10, fy = (double)fr.y * 2.3283064365386963e-10,
               fz = (double)fr.z * 2.3283064365386963e-10;
  const double d0 = __dmul_rn(p.a11, __dadd_rn(fx, __dsub_rn((double)kx, fvx)));
  const double d1 = __dmul_rn(p.a22, __dadd_rn(fy, __dsub_rn((double)ky, fvy)));
  const double d2 = __dmul_rn(p.a33, __dadd_rn(fz, __dsub_rn((double)kz, sl.fz)));
  const double dd = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
  const bool acc64 = dd <= p.cut2;
  if (acc64 == acc32) return;
  float sn, cs;
  __sincosf(6.28318531f * W.p[slot][j].w, &sn, &cs);
  const float w = ex2_approx(-h) * ex2_approx(-dz * dz) * (acc64 ? 1.f : -1.f);
  S.x = fmaf(w, cs, S.x);
  S.y = fmaf(w, sn, S.y);
  dn += acc64 ? 1 : -1;
}

struct Fix {
  float2 d0, d1;  // corrections of the two slices' sums
  int dn;         // change of the accepted count
};

// The rescan of one step (slabs need_lo .. need_hi of the ring) for the lanes that want it.
template <int CAPS>
__device__ __noinline__ Fix exact_fix(const ColumnParams& p, const WarpSmem3<CAPS>& W, int need_lo, int need_hi,
                                      int hz0, float a33s, float cut2, float r3, float inv_bin, float Xv, float Yv,
                                      int hx, int hy, double fvx, double fvy, Slice s0, Slice s1, bool has1) {
  Fix r{make_float2(0.f, 0.f), make_float2(0.f, 0.f), 0};
  for (int u = need_lo; u <= need_hi; ++u) {
    const int slot = u & (kRing - 1);
    const float zoff = __fmul_rn(a33s, (float)(u - hz0));
    const float t0 = __fsub_rn(s0.zv, zoff), t1 = __fsub_rn(s1.zv, zoff);
    bool v0 = true, v1 = has1;  // the march's slab rule (27 cells in z for short cells)
    if (p.trunc_z) {
      v0 = u - s0.hz >= -1 && u - s0.hz <= 1;
      v1 = has1 && u - s1.hz >= -1 && u - s1.hz <= 1;
    }
    if (!v0 && !v1) continue;
    const float w_lo = v0 ? t0 : t1, w_hi = v1 ? t1 : t0;
    const int b_lo = max(0, min(kBins, (int)floorf((w_lo - r3) * inv_bin)));
    const int b_hi = max(0, min(kBins, (int)ceilf((w_hi + r3) * inv_bin)));
    const int lo = W.bin[slot][b_lo], hi = W.bin[slot][b_hi];
    for (int j = lo; j < hi; ++j) {
      const float4 q = W.p[slot][j];
      const float dx = __fsub_rn(q.x, Xv), dy = __fsub_rn(q.y, Yv);
      const float h = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
      if (s0.want && v0) {
        const float dz = __fsub_rn(q.z, t0), hm = __fmaf_rn(-dz, dz, cut2);
        if (fabsf(h - hm) <= kGuard) exact_one(p, W, slot, j, h, dz, h <= hm, hx, hy, fvx, fvy, s0, r.d0, r.dn);
      }
      if (s1.want && v1) {
        const float dz = __fsub_rn(q.z, t1), hm = __fmaf_rn(-dz, dz, cut2);
        if (fabsf(h - hm) <= kGuard) exact_one(p, W, slot, j, h, dz, h <= hm, hx, hy, fvx, fvy, s1, r.d1, r.dn);
      }
    }
  }
  return r;
}

// One warp tile of one image: the TX x (32 / TX) columns of tile `tile` marched through
// the depth.  Returns false when a slab overflows its staging (counters[4]).
template <int NP, bool kDensity, bool kStats, int CAPS, int TX, bool kMasked>
__device__ __noinline__ bool column_tile3(const ColumnParams& p, WarpSmem3<CAPS>& W, int tile, int lane) {
  constexpr int TY = 32 / TX;
  // one precession angle: scalar phases; more: pairs of angles in FP32x2 registers
  using T = typename std::conditional<NP == 1, float, float2>::type;
  constexpr int NH = NP == 1 ? 1 : NP / 2;
  const int Wd = p.ix1 - p.ix0;
  const int tiles_x = (Wd + TX - 1) / TX;
  const int tx = tile % tiles_x, ty = tile / tiles_x;
  const int ix = p.ix0 + tx * TX + (lane % TX);
  const int iy = p.iy0 + ty * TY + lane / TX;
  const bool active = ix < p.ix1 && iy < p.iy1;
  // tile mask: a column is written only when its mask tile is wanted; the warp marches
  // when any of its columns is (a warp tile may straddle mask tiles in any shape)
  bool wanted = true;
  if constexpr (kMasked) {
    if (p.tile_mask) wanted = active && p.tile_mask[(iy / p.mask_T) * p.mask_ntx + ix / p.mask_T] != 0;
    if (!__any_sync(0xffffffffu, wanted)) return true;
  }

  // s = sqrt(log2(e) / (2 sigma^2)): exp(-r^2 / (2 sigma^2)) = ex2(-(s r)^2)
  const double sd = sqrt(p.i2s2 * 1.4426950408889634);
  const int ixc = min(ix, p.ix1 - 1), iyc = min(iy, p.iy1 - 1);
  const int hx = p.xtab[ixc].x, hy = p.ytab[iyc].x;
  const double fvx = p.xfv[ixc], fvy = p.yfv[iyc];
  float Xv, Yv;
  // the tile's frame, footprint and scalars, warp-uniform: with one angle per pass the march
  // reads them from the warp's shared memory, which leaves its registers to the per-column
  // state (measured: 3.26 -> 3.06 ms on the 1.2M-atom image); with more angles the phases
  // take those registers anyway and the shared-memory reads cost (16 angles: 8 % slower),
  // so they stay in registers
  constexpr bool kSmemTile = NP == 1;
  Geo Gr;
  TileConst Cr;
  {
    Geo& G = Gr;
    G.scale = (float)sd;
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
    G.a11s = (float)(p.a11 * sd);
    G.a22s = (float)(p.a22 * sd);
    G.a33s = (float)(p.a33 * sd);
    Xv = (float)(p.a11 * (fvx + (double)(hx - G.ux_ref)) * sd);
    Yv = (float)(p.a22 * (fvy + (double)(hy - G.uy_ref)) * sd);
    const float fbig = 1e30f;
    float v = active ? Xv : fbig, w = active ? -Xv : fbig, y = active ? Yv : fbig, z = active ? -Yv : fbig;
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
    TileConst& C = Cr;
    C.cut2 = (float)(p.cut2 * sd * sd);
    C.r3 = sqrtf(C.cut2) * 1.0001f + 1e-4f;
    C.inv_bin = kBins / G.a33s;
    C.b0 = (float)p.b0;
    C.bg = (float)p.bg;
    C.sig = (float)p.sigma;
    C.dzs = (float)p.dz;
    C.r2_to_A2 = (float)(1.0 / (sd * sd));
    G.pre2 = C.cut2 * 1.0002f + 1e-3f;
    if constexpr (kSmemTile) {
      __syncwarp();  // a previous tile's march has finished reading the warp's copies
      if (lane == 0) {
        W.geo = G;
        W.tc = C;
      }
      __syncwarp();
    }
  }
  const Geo& G = kSmemTile ? W.geo : Gr;
  const TileConst& C = kSmemTile ? W.tc : Cr;
  const unsigned lt = (1u << lane) - 1;

  const int np = min(NP, p.n_prec - p.prec_offset);
  const float* __restrict__ aag = p.aaf + p.prec_offset;
  // the precession coefficients a_k stay in registers for few angles; for many they are
  // read from L1 at each step (pairs: the host pads the table to an even count), which
  // leaves the registers to the phases
  constexpr bool kAaReg = NP <= 4;
  T aa[kAaReg ? NH : 1], ph[NH][4];
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    if constexpr (kAaReg) {
      if constexpr (NP == 1) {
        aa[k] = aag[0];
      } else {
        aa[k] = make_float2(2 * k < np ? aag[2 * k] : 0.f, 2 * k + 1 < np ? aag[2 * k + 1] : 0.f);
      }
    }
    ph[k][0] = bc<T>(1.f);
    ph[k][1] = ph[k][2] = ph[k][3] = bc<T>(0.f);
  }
  const int nh = NP == 1 ? 1 : (np + 1) / 2;  // angle pairs in use
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
      ok = load_slab3<CAPS, false, (NP == 1)>(p, G, ring_hi, W, lane);
    }
    if (!ok) {
      if (lane == 0) atomicExch(&p.counters[4], 1ull);
      return false;  // the host recomputes with larger slabs, or the general kernel
    }
    float2 a0A = make_float2(0.f, 0.f), a1A = a0A, a0B = a0A, a1B = a0A;
    float2 rmA = make_float2(kHuge, kHuge), rmB = rmA;
    int nb = 0;       // atoms in the step buffer
    int n_step = 0;   // atoms buffered in this step (warp-uniform)
    for (int u = need_lo; u <= need_hi; ++u) {
      const int slot = u & (kRing - 1);
      const float zoff = __fmul_rn(G.a33s, (float)(u - hz0));  // cell u's origin relative to hz0's
      const float t0 = __fsub_rn(zv0, zoff), t1 = __fsub_rn(zv1, zoff);
      // slab u serves slice k within the cutoff; with z cells shorter than 3 sigma the
      // reference searches only the 27 cells around each voxel's home cell, so it serves
      // a slice only within one cell of that slice's home z cell
      bool v0 = true, v1 = has1;
      if (p.trunc_z) {
        v0 = u - hz0 >= -1 && u - hz0 <= 1;
        v1 = has1 && u - hz1 >= -1 && u - hz1 <= 1;
      }
      if (!v0 && !v1) continue;
      const float w_lo = v0 ? t0 : t1, w_hi = v1 ? t1 : t0;
      const int b_lo = max(0, min(kBins, (int)floorf((w_lo - C.r3) * C.inv_bin)));
      const int b_hi = max(0, min(kBins, (int)ceilf((w_hi + C.r3) * C.inv_bin)));
      const int lo = W.bin[slot][b_lo];
      const int hi = W.bin[slot][b_hi];
      const float4* P = W.p[slot];
      for (int b = lo; b < hi; b += 32) {
        // cooperative pass: one atom per lane, its depth-only terms, kept if some column
        // of the patch can accept it at some slice
        const int j = b + lane;
        bool keep = false;
        float4 A, E;
        if (j < hi) {
          const float4 q = P[j];
          float sn, cs;
          __sincosf(6.28318531f * q.w, &sn, &cs);  // the phase lies in [-1/2, 1/2) cycles
          const float dz0 = __fsub_rn(q.z, t0), dz1 = __fsub_rn(q.z, t1);
          const float hm0 = v0 ? __fmaf_rn(-dz0, dz0, C.cut2) : -1.f;
          const float hm1 = v1 ? __fmaf_rn(-dz1, dz1, C.cut2) : -1.f;
          const float dxr = fmaxf(0.f, fmaxf(G.xmin - q.x, q.x - G.xmax));
          const float dyr = fmaxf(0.f, fmaxf(G.ymin - q.y, q.y - G.ymax));
          // margin: the lanes' own rounding of dxy^2 must not reach below the rectangle's
          keep = fmaf(dxr, dxr, dyr * dyr) <= fmaxf(hm0, hm1) * 1.0001f + 1e-4f;
          const float wz0 = ex2_approx(-dz0 * dz0), wz1 = ex2_approx(-dz1 * dz1);
          A = make_float4(q.x, q.y, hm0, hm1);
          E = make_float4(wz0 * cs, wz0 * sn, wz1 * cs, wz1 * sn);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int d = nb + __popc(m & lt);
          W.ba[d] = A;
          W.be[d] = E;
        }
        nb += __popc(m);
        if (nb >= 32) {
          __syncwarp();
          consume<kDensity, kStats>(W.ba, W.be, nb, Xv, Yv, a0A, a1A, a0B, a1B, rmA, rmB, n_acc);
          if (kStats) n_tst += (unsigned long long)nb;
          __syncwarp();
          n_step += nb;
          nb = 0;
        }
      }
    }
    if (nb > 0) {
      __syncwarp();
      consume<kDensity, kStats>(W.ba, W.be, nb, Xv, Yv, a0A, a1A, a0B, a1B, rmA, rmB, n_acc);
      if (kStats) n_tst += (unsigned long long)nb;
      __syncwarp();
      n_step += nb;
    }
    float2 a0 = __fadd2_rn(a0A, a0B), a1 = __fadd2_rn(a1A, a1B);
    {
      // sparse or cancelling sums: re-decide the near-cutoff atoms exactly (see exact_fix)
      const bool f0 = active && n_step > 0 && fmaf(a0.x, a0.x, a0.y * a0.y) < kSparse2;
      const bool f1 = active && n_step > 0 && has1 && fmaf(a1.x, a1.x, a1.y * a1.y) < kSparse2;
      if (__any_sync(0xffffffffu, f0 || f1)) {
        if (f0 || f1) {
          const Slice sl0{hz0, zv0, p.zfv[z0], f0}, sl1{hz1, zv1, has1 ? p.zfv[z0 + 1] : 0.0, f1};
          const Fix fx = exact_fix<CAPS>(p, W, need_lo, need_hi, hz0, G.a33s, C.cut2, C.r3, C.inv_bin, Xv, Yv, hx, hy,
                                         fvx, fvy, sl0, sl1, has1);
          a0.x += fx.d0.x;
          a0.y += fx.d0.y;
          a1.x += fx.d1.x;
          a1.y += fx.d1.y;
          if (kStats) n_acc += (unsigned)fx.dn;
        }
        __syncwarp();
      }
    }
    const float rm0 = (C.cut2 + fminf(rmA.x, rmB.x)) * C.r2_to_A2;
    const float rm1 = (C.cut2 + fminf(rmA.y, rmB.y)) * C.r2_to_A2;
    // field samples z0 (even) and z0 + 1 (odd), then the RK4 double step (z0-2, z0-1, z0)
    const Sample s0 = make_sample<kDensity>(a0.x, a0.y, rm0, C.b0, C.bg, C.sig, p.use_density != 0);
    if (z0 == 0) {
      s_first = s0;
    } else {
      const SampleT<T> w0 = widen<T>(s_prev), w1 = widen<T>(s_mid), w2 = widen<T>(s0);
#pragma unroll
      for (int k = 0; k < NH; ++k)
        if (k < nh) rk4<T>(w0, w1, w2, aa_at<T, kAaReg>(aa, aag, k), C.dzs, ph[k]);
    }
    s_prev = s0;
    if (has1) s_mid = make_sample<kDensity>(a1.x, a1.y, rm1, C.b0, C.bg, C.sig, p.use_density != 0);
  }
  if ((p.Mz & 1) == 0) {  // closure x(Mz) = x(0)
    const SampleT<T> w0 = widen<T>(s_prev), w1 = widen<T>(s_mid), w2 = widen<T>(s_first);
#pragma unroll
    for (int k = 0; k < NH; ++k)
      if (k < nh) rk4<T>(w0, w1, w2, aa_at<T, kAaReg>(aa, aag, k), C.dzs, ph[k]);
  }
  // |phi_g|^2 summed over the angles in order, rounded the same way for either form
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    if constexpr (NP == 1) {
      acc = __fadd_rn(acc, __fmaf_rn(ph[k][2], ph[k][2], __fmul_rn(ph[k][3], ph[k][3])));
    } else {
      if (2 * k < np) acc = __fadd_rn(acc, __fmaf_rn(ph[k][2].x, ph[k][2].x, __fmul_rn(ph[k][3].x, ph[k][3].x)));
      if (2 * k + 1 < np)
        acc = __fadd_rn(acc, __fmaf_rn(ph[k][2].y, ph[k][2].y, __fmul_rn(ph[k][3].y, ph[k][3].y)));
    }
  }
  if (active && wanted) {
    // the precession average and the bright-field flip fold into the last pass's store,
    // in the separate epilogue's arithmetic (k_epilogue)
    double* o = p.img + ix + (int64_t)p.Mx * iy;
    double v = p.accumulate ? *o + (double)acc : (double)acc;
    if (p.finalize) {
      v = __ddiv_rn(v, p.fin_scale);
      if (p.fin_bright) v = __dsub_rn(1.0, v);
    }
    *o = v;
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

// Persistent launch over the warp tiles of every job of a batch: each warp takes the
// next tile from a global counter, so images of uneven size share the GPU without a tail
// per image.  kMasked: jobs may carry a tile mask (columns outside it are not written).
template <int NP, bool kDensity, bool kStats, int kMinBlocks, int CAPS, int TX, bool kMasked>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocks)
    k_column_fp32_v3(const ColumnJob* __restrict__ jobs, int n_jobs, int total_tiles, unsigned* __restrict__ work,
                     const unsigned long long* __restrict__ counters, int64_t cap) {
  constexpr int kShape = TX == 8 ? 0 : TX == 4 ? 1 : 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpSmem3<CAPS>& W = reinterpret_cast<WarpSmem3<CAPS>*>(smem_raw)[warp];
  if ((int64_t)counters[0] > cap) return;  // the binning overflowed: the host retries
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = (int)atomicAdd(work, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= total_tiles) break;
    if (counters[4] != 0) break;  // a slab overflowed: the host recomputes with larger slabs
    int lo = 0, hi = n_jobs - 1;  // job of this tile
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile_base[kShape] <= tile)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int local = tile - jobs[lo].tile_base[kShape];
    if (!column_tile3<NP, kDensity, kStats, CAPS, TX, kMasked>(jobs[lo].p, W, local, lane)) break;
  }
}

template <int CAPS, typename K>
cudaError_t launch3(K kernel, const Ring3Args& a, int tiles, int blocks_per_sm) {
  const size_t smem = sizeof(WarpSmem3<CAPS>) * kWarps;
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
  kernel<<<grid, kWarps * 32, smem, a.st>>>(a.jobs, a.n_jobs, tiles, a.work, a.counters, a.cap);
  return cudaGetLastError();
}

// Instances of one angle bucket NP.  Tuning variants (tier 0, no statistics, no mask):
// the tile shape (8 x 4, 4 x 8, 16 x 2 columns) and the slab capacity of the first tier
// (128 atoms, four CTAs per SM; 96 atoms, five -- both three with 16 angles, whose phases
// need more registers than four CTAs leave).  Tiers 1 and 2 (192 and 256 atoms per slab,
// three and two CTAs per SM), the statistics and the tile-masked instances use 8 x 4
// tiles.
template <int NP, bool kDensity>
cudaError_t ring3_dispatch(const Ring3Args& a) {
  constexpr int B96 = NP >= 16 ? 3 : 5;
  constexpr int B128 = NP >= 16 ? 3 : 4;  // 16 angles: 168 registers, no spills (at four CTAs they spill)
  const int* T = a.tiles;
  if (a.masked) {  // the variant's tile shape, so that a masked image equals the plain one on its tiles
    if constexpr (NP == 1) {
      if (a.tier >= 2) return launch3<256>(k_column_fp32_v3<1, kDensity, false, 2, 256, 8, true>, a, T[0], 2);
      if (a.tier == 1) return launch3<192>(k_column_fp32_v3<1, kDensity, false, 3, 192, 8, true>, a, T[0], 3);
      if (a.variant == 2 || a.variant == 3)
        return launch3<128>(k_column_fp32_v3<1, kDensity, false, 4, 128, 4, true>, a, T[1], 4);
      if (a.variant == 4 || a.variant == 5)
        return launch3<128>(k_column_fp32_v3<1, kDensity, false, 4, 128, 16, true>, a, T[2], 4);
      return launch3<128>(k_column_fp32_v3<1, kDensity, false, 4, 128, 8, true>, a, T[0], 4);
    }
    return cudaErrorInvalidValue;
  }
  if (a.stats) {
    if (a.tier >= 2) return launch3<256>(k_column_fp32_v3<NP, kDensity, true, 2, 256, 8, false>, a, T[0], 2);
    if (a.tier == 1) return launch3<192>(k_column_fp32_v3<NP, kDensity, true, 3, 192, 8, false>, a, T[0], 3);
    return launch3<128>(k_column_fp32_v3<NP, kDensity, true, 4, 128, 8, false>, a, T[0], 4);
  }
  if (a.tier >= 2) return launch3<256>(k_column_fp32_v3<NP, kDensity, false, 2, 256, 8, false>, a, T[0], 2);
  if (a.tier == 1) return launch3<192>(k_column_fp32_v3<NP, kDensity, false, 3, 192, 8, false>, a, T[0], 3);
  switch (a.variant) {
    case 1: return launch3<96>(k_column_fp32_v3<NP, kDensity, false, B96, 96, 8, false>, a, T[0], B96);
    case 2: return launch3<128>(k_column_fp32_v3<NP, kDensity, false, B128, 128, 4, false>, a, T[1], B128);
    case 3: return launch3<96>(k_column_fp32_v3<NP, kDensity, false, B96, 96, 4, false>, a, T[1], B96);
    case 4: return launch3<128>(k_column_fp32_v3<NP, kDensity, false, B128, 128, 16, false>, a, T[2], B128);
    case 5: return launch3<96>(k_column_fp32_v3<NP, kDensity, false, B96, 96, 16, false>, a, T[2], B96);
    default: return launch3<128>(k_column_fp32_v3<NP, kDensity, false, B128, 128, 8, false>, a, T[0], B128);
  }
}

template <int NP>
cudaError_t ring3_launch_np(const Ring3Args& a) {
  return a.density ? ring3_dispatch<NP, true>(a) : ring3_dispatch<NP, false>(a);
}

}  // namespace ring3
}  // namespace stem
