// K2+K3: voxel phase field and column integration, fused.
//
// Follows the pixel loop of computeD2BI_img (Lib_DynamicalTwoBeamImaging.f90
// :1870-1900), the neighbour search neighbourList1b (Lib_LinkCell3D.f90
// :1515-1605), convertScaledRangeToRho (:1973-1994) and the column integrator
// dynamicalTwoBeamIntegrationColumn_phaserho (:2316-2480).
//
// Work decomposition: one warp owns a patch of 8 x 4 pixel columns (one lane
// per column) and marches through the depth z.  All lanes share the voxel
// depth iz and therefore the home link cell in z, hz.  For each hz the warp
// gathers the atoms of the link-cell slabs hz-1, hz, hz+1 (periodic in z, with
// the reference's unwrapped cell offsets) in the x-y footprint of its columns
// from the cell-sorted arrays made by K1, keeps those within 3 sigma of the
// patch's column rectangle, and stages them in warp-private shared memory.
// Each lane then tests every staged atom against its own voxel: the field
// x(iz) = S/|S| with S = sum exp(-r^2 / 2 sigma^2) exp(i g.y), and r_min for
// the density.  The field never leaves registers: the RK4 double step of the
// integrator runs as soon as samples ii, ii+1, ii+2 exist, for every
// precession angle at once, and the periodic closure x(Mz) = x(0) is kept in
// registers.  No global atomics are used on the data path.
//
// The FP64 variant reproduces the reference arithmetic exactly (explicitly
// rounded operations in the reference's order, the reference's 27-cell rule,
// the reference's summation order); an FP32 bound test only skips candidates
// that are far outside the cutoff.  The FP32 variant computes distances from
// small relative coordinates and uses ex2.approx for the Gaussian weight.
#include <cuda_runtime.h>

#include <cfloat>

#include "fp64_column.cuh"
#include "internal.h"

namespace stem {
namespace {

constexpr int kWarps = 4;   // warps per CTA
constexpr int kTileX = 8;   // columns per warp in x
constexpr int kTileY = 4;   // columns per warp in y
constexpr int kCap32 = 512; // staged atoms per warp, FP32 kernel
constexpr int kCap64 = 256; // staged atoms per warp, FP64 kernel
constexpr float kHuge1 = FLT_MAX;  // huge(1.0)

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int pos_mod(int a, int n) {
  const int r = a % n;
  return r < 0 ? r + n : r;
}

// Per-warp geometry of the current patch.
struct WarpGeom {
  int ux_lo, ux_hi, uy_lo, uy_hi;  // unwrapped link cells to gather (x, y)
  int ux_ref, uy_ref;              // reference cells of the relative coordinates
  float xmin, xmax, ymin, ymax;    // column rectangle in relative coordinates
  float pre2;                      // prefilter radius^2
};

// Resumable position of the gather over slabs x rows x x-runs x atoms.  A
// run is a stretch of unwrapped x cells that maps to consecutive memory cells
// of one row; runs are found on the fly, so any span of cells is handled.
struct GatherPos {
  int slab, row, u, off;
};

__device__ __forceinline__ int floor_div(int a, int n) { return (a >= 0) ? a / n : -((-a + n - 1) / n); }

// Gather candidate atoms for home z-cell hz into the warp buffer until it is
// full or the slabs are exhausted.  Returns the number staged; `pos` is
// advanced (pos.slab == 3 when done).  Layouts: buf4 = (X', Y', Z', cos) with
// bufs = sin (FP32 kernel), or buf4 = (X', Y', Z', -) with bufxy = (fx, fy),
// bufz = fz and bufcs = (cos, sin) in FP64 (FP64 kernel); bufu = the
// unwrapped cell offsets relative to the warp's reference cells.
template <bool kFp64>
__device__ int gather(const ColumnParams& p, const WarpGeom& wg, int hz, GatherPos& pos, float4* buf4, float* bufs,
                      int* bufu, double2* bufxy, double* bufz, double2* bufcs, int cap, int lane) {
  const float a11f = (float)p.a11, a22f = (float)p.a22, a33f = (float)p.a33;
  const int nrows = wg.uy_hi - wg.uy_lo + 1;
  int nbuf = 0;
  if (pos.u < wg.ux_lo) pos.u = wg.ux_lo;
  while (pos.slab < 3) {
    const int uz = hz - 1 + pos.slab;
    const int cz = pos_mod(uz, p.Ez);
    const int uy = wg.uy_lo + pos.row;
    const int cy = pos_mod(uy, p.Ey);
    const int k = floor_div(pos.u, p.Ex);
    const int run_hi = min(wg.ux_hi, (k + 1) * p.Ex - 1);
    const int shift = k * p.Ex;
    const int64_t row_base = (int64_t)p.Ex * (cy + (int64_t)p.Ey * cz);
    const int a_lo = p.cell_start[row_base + (pos.u - shift)];
    const int a_hi = p.cell_start[row_base + (run_hi - shift) + 1];
    const float yoff = a22f * (float)(uy - wg.uy_ref);
    const float zoff = a33f * (float)(uz - hz);
    bool full = false;
    while (a_lo + pos.off < a_hi) {
      const int j = a_lo + pos.off + lane;
      bool keep = false;
      float X = 0.f, Y = 0.f, Z = 0.f;
      int ucode = 0;
      if (j < a_hi) {
        const float4 r = p.p32[j];
        const int packed = __float_as_int(r.w);
        const int ux = (packed & 1023) + shift;
        X = r.x + a11f * (float)(ux - wg.ux_ref);
        Y = r.y + yoff;
        Z = r.z + zoff;
        const float dx = fmaxf(0.f, fmaxf(wg.xmin - X, X - wg.xmax));
        const float dy = fmaxf(0.f, fmaxf(wg.ymin - Y, Y - wg.ymax));
        keep = dx * dx + dy * dy <= wg.pre2;
        ucode = (ux - wg.ux_ref + 8) | ((uy - wg.uy_ref + 8) << 8) | ((uz - hz + 8) << 16);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int cnt = __popc(m);
      if (nbuf + cnt > cap) {
        full = true;
        break;
      }
      if (keep) {
        const int d = nbuf + __popc(m & ((1u << lane) - 1));
        if (kFp64) {
          const double4_32a f = p.f64[j];
          buf4[d] = make_float4(X, Y, Z, 0.f);
          bufxy[d] = make_double2(f.x, f.y);
          bufz[d] = f.z;
          bufcs[d] = p.cs64[j];
        } else {
          const float2 cs = p.cs32[j];
          buf4[d] = make_float4(X, Y, Z, cs.x);
          bufs[d] = cs.y;
        }
        bufu[d] = ucode;
      }
      nbuf += cnt;
      pos.off += 32;
    }
    if (full) break;
    pos.off = 0;
    pos.u = run_hi + 1;
    if (pos.u > wg.ux_hi) {
      pos.u = wg.ux_lo;
      if (++pos.row == nrows) {
        pos.row = 0;
        ++pos.slab;
      }
    }
  }
  __syncwarp();
  return nbuf;
}

// ---------------------------------------------------------------------------
// FP32 column integrator state
// ---------------------------------------------------------------------------

struct Sample32 {
  float c0, cgr, cgi;
};

__device__ __forceinline__ void deriv32(const Sample32& s, float a, const float* ph, float* d) {
  const float ca = s.c0 + a;
  d[0] = -s.c0 * ph[1] - s.cgi * ph[2] - s.cgr * ph[3];
  d[1] = s.c0 * ph[0] + s.cgr * ph[2] - s.cgi * ph[3];
  d[2] = s.cgi * ph[0] - s.cgr * ph[1] - ca * ph[3];
  d[3] = s.cgr * ph[0] + s.cgi * ph[1] + ca * ph[2];
}

// One RK4 double step over samples (s0, s1, s2) (:2389-2472).
__device__ __forceinline__ void rk4_32(const Sample32& s0, const Sample32& s1, const Sample32& s2, float a,
                                       float dz, float* ph) {
  float d[4], p1[4], q[4];
  const float dz3 = dz / 3.f, dz23 = 2.f * dz / 3.f, dz2 = 2.f * dz;
  deriv32(s0, a, ph, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    p1[i] = ph[i] + d[i] * dz3;
    q[i] = ph[i] + d[i] * dz;
  }
  deriv32(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = ph[i] + d[i] * dz;
    p1[i] = p1[i] + d[i] * dz23;
  }
  deriv32(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = ph[i] + d[i] * dz2;
    p1[i] = p1[i] + d[i] * dz23;
  }
  deriv32(s2, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = p1[i] + d[i] * dz3;
  const float inv = rsqrtf(ph[0] * ph[0] + ph[1] * ph[1] + ph[2] * ph[2] + ph[3] * ph[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] *= inv;
}

__device__ __forceinline__ float rho32(float r2min, float sig) {
  if (r2min < sig * sig) return 1.f;
  if (r2min > 4.f * sig * sig) return 0.f;
  const float xx = sqrtf(r2min) / sig - 1.f;
  return 1.f - xx * xx * xx * (10.f - 15.f * xx + 6.f * xx * xx);
}

__device__ __forceinline__ void setup_warp(const ColumnParams& p, int ix, int iy, bool active, int lane, int& hx,
                                           double& fvx, int& hy, double& fvy, WarpGeom& wg) {
  const int ixc = min(ix, p.ix1 - 1), iyc = min(iy, p.iy1 - 1);
  hx = p.xtab[ixc].x;
  fvx = p.xfv[ixc];
  hy = p.ytab[iyc].x;
  fvy = p.yfv[iyc];
  const int big = 1 << 29;
  const int mnx = __reduce_min_sync(0xffffffffu, active ? hx : big);
  const int mxx = __reduce_max_sync(0xffffffffu, active ? hx : -big);
  const int mny = __reduce_min_sync(0xffffffffu, active ? hy : big);
  const int mxy = __reduce_max_sync(0xffffffffu, active ? hy : -big);
  wg.ux_lo = mnx - 1;
  wg.ux_hi = mxx + 1;
  wg.uy_lo = mny - 1;
  wg.uy_hi = mxy + 1;
  wg.ux_ref = mnx;
  wg.uy_ref = mny;
  (void)lane;
}

template <int NP>
__global__ void __launch_bounds__(kWarps * 32) k_column_fp32(const __grid_constant__ ColumnParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float4* buf4 = reinterpret_cast<float4*>(smem) + warp * kCap32;
  float* bufs = reinterpret_cast<float*>(reinterpret_cast<float4*>(smem) + kWarps * kCap32) + warp * kCap32;
  int* bufu = reinterpret_cast<int*>(reinterpret_cast<float*>(reinterpret_cast<float4*>(smem) + kWarps * kCap32) +
                                     kWarps * kCap32) +
              warp * kCap32;

  const int W = p.ix1 - p.ix0, H = p.iy1 - p.iy0;
  const int tiles_x = (W + kTileX - 1) / kTileX, tiles_y = (H + kTileY - 1) / kTileY;
  const int tile = blockIdx.x * kWarps + warp;
  if (tile >= tiles_x * tiles_y) return;
  if ((int64_t)p.counters[0] > p.cap) return;  // the binning overflowed: the host retries
  const int tx = tile % tiles_x, ty = tile / tiles_x;
  if (!tile_wanted(p, tx, ty, kTileX, kTileY)) return;
  const int ix = p.ix0 + tx * kTileX + (lane & (kTileX - 1));
  const int iy = p.iy0 + ty * kTileY + lane / kTileX;
  const bool active = ix < p.ix1 && iy < p.iy1;

  int hx, hy;
  double fvx, fvy;
  WarpGeom wg;
  setup_warp(p, ix, iy, active, lane, hx, fvx, hy, fvy, wg);
  const float Xv = (float)(p.a11 * (fvx + (double)(hx - wg.ux_ref)));
  const float Yv = (float)(p.a22 * (fvy + (double)(hy - wg.uy_ref)));
  {
    const float big = 1e30f;
    float v = active ? Xv : big;
    float w = active ? -Xv : big;
    float y = active ? Yv : big;
    float z = active ? -Yv : big;
    for (int o = 16; o > 0; o >>= 1) {
      v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
      w = fminf(w, __shfl_xor_sync(0xffffffffu, w, o));
      y = fminf(y, __shfl_xor_sync(0xffffffffu, y, o));
      z = fminf(z, __shfl_xor_sync(0xffffffffu, z, o));
    }
    wg.xmin = v;
    wg.xmax = -w;
    wg.ymin = y;
    wg.ymax = -z;
  }
  const float cut2f = (float)p.cut2;
  wg.pre2 = cut2f * 1.0001f + 1e-3f;
  const float kexp = (float)(-p.i2s2 * 1.4426950408889634);  // exp(-r2 i2s2) = 2^(r2 * kexp)
  const float sigf = (float)p.sigma;
  const float b0 = (float)p.b0, bg = (float)p.bg, dz = (float)p.dz;
  const int hx_o = hx - wg.ux_ref + 8, hy_o = hy - wg.uy_ref + 8;

  const int np = min(NP, p.n_prec - p.prec_offset);
  float aa[NP];
  float ph[NP][4];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    aa[k] = (k < np) ? p.aaf[p.prec_offset + k] : 0.f;
    ph[k][0] = 1.f;
    ph[k][1] = ph[k][2] = ph[k][3] = 0.f;
  }
  Sample32 s_first{0.f, 0.f, 0.f}, s_prev{0.f, 0.f, 0.f}, s_mid{0.f, 0.f, 0.f};

  int cur_hz = -1 << 30;
  int nbuf = 0;
  bool chunked = false;
  unsigned n_acc = 0;  // accepted pairs of this lane
  unsigned long long n_tst = 0;

  for (int iz = 0; iz < p.Mz; ++iz) {
    const int hz = p.ztab[iz].x;
    const float Zv = (float)(p.a33 * p.zfv[iz]);
    GatherPos gp{0, 0, -(1 << 30), 0};
    if (hz != cur_hz) {
      cur_hz = hz;
      nbuf = gather<false>(p, wg, hz, gp, buf4, bufs, bufu, nullptr, nullptr, nullptr, kCap32, lane);
      chunked = gp.slab < 3;
    }
    float sr = 0.f, si = 0.f, r2min = kHuge1;
    for (;;) {
      if (p.check_cells) {
        for (int j = 0; j < nbuf; ++j) {
          const float4 q = buf4[j];
          const float dx = q.x - Xv, dy = q.y - Yv, dzz = q.z - Zv;
          const float r2 = dx * dx + dy * dy + dzz * dzz;
          const int u = bufu[j];
          const bool in27 = abs((u & 255) - hx_o) <= 1 && abs(((u >> 8) & 255) - hy_o) <= 1 &&
                            abs(((u >> 16) & 255) - 8) <= 1;
          if (r2 <= cut2f && in27) {
            const float w = ex2_approx(r2 * kexp);
            sr = fmaf(w, q.w, sr);
            si = fmaf(w, bufs[j], si);
            r2min = fminf(r2min, r2);
            ++n_acc;
          }
        }
      } else {
#pragma unroll 4
        for (int j = 0; j < nbuf; ++j) {
          const float4 q = buf4[j];
          const float dx = q.x - Xv, dy = q.y - Yv, dzz = q.z - Zv;
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dzz * dzz));
          if (r2 <= cut2f) {
            const float w = ex2_approx(r2 * kexp);
            sr = fmaf(w, q.w, sr);
            si = fmaf(w, bufs[j], si);
            r2min = fminf(r2min, r2);
            ++n_acc;
          }
        }
      }
      if (active) n_tst += nbuf;
      if (!chunked) break;
      if (gp.slab >= 3) break;
      nbuf = gather<false>(p, wg, hz, gp, buf4, bufs, bufu, nullptr, nullptr, nullptr, kCap32, lane);
      if (nbuf == 0 && gp.slab >= 3) break;
    }
    if (chunked) {
      // the buffer holds the last chunk only: restart the gather next slice
      cur_hz = -1 << 30;
    }
    // x(iz) = S / max(1e-16, |S|)
    const float nrm2 = fmaf(sr, sr, si * si);
    const float inv = rsqrtf(fmaxf(nrm2, 1e-32f));
    const float xr = sr * inv, xi = si * inv;
    const float rho = p.use_density ? rho32(r2min, sigf) : 1.f;
    Sample32 s{b0 * rho, bg * rho * xr, bg * rho * xi};
    if (iz == 0) {
      s_first = s;
      s_prev = s;
    } else if (iz & 1) {
      s_mid = s;
    } else {
#pragma unroll
      for (int k = 0; k < NP; ++k)
        if (k < np) rk4_32(s_prev, s_mid, s, aa[k], dz, ph[k]);
      s_prev = s;
    }
  }
  if ((p.Mz & 1) == 0) {
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) rk4_32(s_prev, s_mid, s_first, aa[k], dz, ph[k]);
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < NP; ++k)
    if (k < np) acc += ph[k][2] * ph[k][2] + ph[k][3] * ph[k][3];
  if (active) {
    double* o = p.img + ix + (int64_t)p.Mx * iy;
    *o = p.accumulate ? *o + (double)acc : (double)acc;
  }
  if (p.want_stats) {
    unsigned long long acc_w = active ? n_acc : 0u, tst_w = n_tst;
    for (int o = 16; o > 0; o >>= 1) {
      acc_w += __shfl_xor_sync(0xffffffffu, acc_w, o);
      tst_w += __shfl_xor_sync(0xffffffffu, tst_w, o);
    }
    if (lane == 0) {
      atomicAdd(&p.counters[2], tst_w);
      atomicAdd(&p.counters[3], acc_w);
    }
  }
}

// ---------------------------------------------------------------------------
// FP64: the reference arithmetic, operation by operation
// ---------------------------------------------------------------------------

using namespace fp64col;

template <int NP>
__global__ void __launch_bounds__(kWarps * 32) k_column_fp64(const __grid_constant__ ColumnParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // per warp: (fx, fy) | fz | (cos, sin) | (X', Y', Z', -) | cell offsets, all 16-byte aligned
  double2* bufxy = reinterpret_cast<double2*>(smem) + warp * kCap64;
  double* bufz = reinterpret_cast<double*>(smem + kWarps * kCap64 * sizeof(double2)) + warp * kCap64;
  double2* bufcs =
      reinterpret_cast<double2*>(smem + kWarps * kCap64 * (sizeof(double2) + sizeof(double))) + warp * kCap64;
  float4* buf4 =
      reinterpret_cast<float4*>(smem + kWarps * kCap64 * (2 * sizeof(double2) + sizeof(double))) + warp * kCap64;
  int* bufu = reinterpret_cast<int*>(smem + kWarps * kCap64 * (2 * sizeof(double2) + sizeof(double) + sizeof(float4))) +
              warp * kCap64;

  const int W = p.ix1 - p.ix0, H = p.iy1 - p.iy0;
  const int tiles_x = (W + kTileX - 1) / kTileX, tiles_y = (H + kTileY - 1) / kTileY;
  const int tile = blockIdx.x * kWarps + warp;
  if (tile >= tiles_x * tiles_y) return;
  if ((int64_t)p.counters[0] > p.cap) return;  // the binning overflowed: the host retries
  const int tx = tile % tiles_x, ty = tile / tiles_x;
  if (!tile_wanted(p, tx, ty, kTileX, kTileY)) return;
  const int ix = p.ix0 + tx * kTileX + (lane & (kTileX - 1));
  const int iy = p.iy0 + ty * kTileY + lane / kTileX;
  const bool active = ix < p.ix1 && iy < p.iy1;

  int hx, hy;
  double fvx, fvy;
  WarpGeom wg;
  setup_warp(p, ix, iy, active, lane, hx, fvx, hy, fvy, wg);
  const float Xv = (float)(p.a11 * (fvx + (double)(hx - wg.ux_ref)));
  const float Yv = (float)(p.a22 * (fvy + (double)(hy - wg.uy_ref)));
  {
    const float big = 1e30f;
    float v = active ? Xv : big, w = active ? -Xv : big, y = active ? Yv : big, z = active ? -Yv : big;
    for (int o = 16; o > 0; o >>= 1) {
      v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
      w = fminf(w, __shfl_xor_sync(0xffffffffu, w, o));
      y = fminf(y, __shfl_xor_sync(0xffffffffu, y, o));
      z = fminf(z, __shfl_xor_sync(0xffffffffu, z, o));
    }
    wg.xmin = v;
    wg.xmax = -w;
    wg.ymin = y;
    wg.ymax = -z;
  }
  const float pre_f = (float)p.cut2 + 1e-2f;  // FP32 bound test (exact test follows)
  wg.pre2 = pre_f;
  // dzi(k) = k - zi_frac for k = -1, 0, 1 (:1576-1588)
  double dzx[3], dzy[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dzx[k] = DS((double)(k - 1), fvx);
    dzy[k] = DS((double)(k - 1), fvy);
  }
  const int hx_o = hx - wg.ux_ref + 8, hy_o = hy - wg.uy_ref + 8;

  const int np = min(NP, p.n_prec - p.prec_offset);
  double aa[NP];
  double ph[NP][4];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    aa[k] = (k < np) ? p.aa[p.prec_offset + k] : 0.0;
    ph[k][0] = 1.0;
    ph[k][1] = ph[k][2] = ph[k][3] = 0.0;
  }
  Sample64 s_first{0, 0, 0, 0}, s_prev{0, 0, 0, 0}, s_mid{0, 0, 0, 0};

  int cur_hz = -1 << 30;
  int nbuf = 0;
  bool chunked = false;
  unsigned n_acc = 0;  // accepted pairs of this lane
  unsigned long long n_tst = 0;

  for (int iz = 0; iz < p.Mz; ++iz) {
    const int hz = p.ztab[iz].x;
    const double fvz = p.zfv[iz];
    const float Zv = (float)(p.a33 * fvz);
    double dzz3[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dzz3[k] = DS((double)(k - 1), fvz);
    GatherPos gp{0, 0, -(1 << 30), 0};
    if (hz != cur_hz) {
      cur_hz = hz;
      nbuf = gather<true>(p, wg, hz, gp, buf4, nullptr, bufu, bufxy, bufz, bufcs, kCap64, lane);
      chunked = gp.slab < 3;
    }
    double sr = 0.0, si = 0.0, r2min = (double)kHuge1;
    for (;;) {
      for (int j = 0; j < nbuf; ++j) {
        const float4 q = buf4[j];
        const float dx = q.x - Xv, dy = q.y - Yv, dzf = q.z - Zv;
        if (dx * dx + dy * dy + dzf * dzf > pre_f) continue;
        const int u = bufu[j];
        const int kx = (u & 255) - hx_o, ky = ((u >> 8) & 255) - hy_o, kz = ((u >> 16) & 255) - 8;
        if (kx < -1 || kx > 1 || ky < -1 || ky > 1 || kz < -1 || kz > 1) continue;  // the 27 cells
        const double2 fxy = bufxy[j];
        const double d0 = DM(p.a11, DA(fxy.x, dzx[kx + 1]));
        const double d1 = DM(p.a22, DA(fxy.y, dzy[ky + 1]));
        const double d2 = DM(p.a33, DA(bufz[j], dzz3[kz + 1]));
        const double dd = DA(DA(DM(d0, d0), DM(d1, d1)), DM(d2, d2));
        if (dd <= p.cut2) {
          const double w = exp(DM(-dd, p.i2s2));
          const double2 cs = bufcs[j];
          sr = DA(sr, DM(w, cs.x));
          si = DA(si, DM(w, cs.y));
          r2min = fmin(r2min, dd);
          ++n_acc;
        }
      }
      if (active) n_tst += nbuf;
      if (!chunked) break;
      if (gp.slab >= 3) break;
      nbuf = gather<true>(p, wg, hz, gp, buf4, nullptr, bufu, bufxy, bufz, bufcs, kCap64, lane);
      if (nbuf == 0 && gp.slab >= 3) break;
    }
    if (chunked) cur_hz = -1 << 30;
    double ww = hypot(sr, si);
    ww = __ddiv_rn(1.0, fmax(1.0e-16, ww));
    const double xr = DM(sr, ww), xi = DM(si, ww);
    const double rho = p.use_density ? rho64(r2min, p.sigma) : 1.0;
    const double bgr = DM(p.bg, rho);
    Sample64 s{DM(p.b0, rho), DM(p.b0, rho), DM(bgr, xr), DM(bgr, xi)};
    if (iz == 0) {
      s_first = s;
      s_prev = s;
    } else if (iz & 1) {
      s_mid = s;
    } else {
#pragma unroll
      for (int k = 0; k < NP; ++k)
        if (k < np) rk4_64(s_prev, s_mid, s, aa[k], p.dz, ph[k]);
      s_prev = s;
    }
  }
  if ((p.Mz & 1) == 0) {
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) rk4_64(s_prev, s_mid, s_first, aa[k], p.dz, ph[k]);
  }
  if (active) {
    double* o = p.img + ix + (int64_t)p.Mx * iy;
    double acc = p.accumulate ? *o : 0.0;
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (k < np) acc = DA(acc, DA(DM(ph[k][2], ph[k][2]), DM(ph[k][3], ph[k][3])));
    *o = acc;
  }
  if (p.want_stats) {
    unsigned long long acc_w = active ? n_acc : 0u, tst_w = n_tst;
    for (int o = 16; o > 0; o >>= 1) {
      acc_w += __shfl_xor_sync(0xffffffffu, acc_w, o);
      tst_w += __shfl_xor_sync(0xffffffffu, tst_w, o);
    }
    if (lane == 0) {
      atomicAdd(&p.counters[2], tst_w);
      atomicAdd(&p.counters[3], acc_w);
    }
  }
}

template <typename K>
cudaError_t launch_cols(K kernel, const ColumnParams& p, size_t smem, cudaStream_t st) {
  const int W = p.ix1 - p.ix0, H = p.iy1 - p.iy0;
  const int tiles = ((W + kTileX - 1) / kTileX) * ((H + kTileY - 1) / kTileY);
  const int grid = (tiles + kWarps - 1) / kWarps;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_count();
  kernel<<<grid, kWarps * 32, smem, st>>>(p);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_column_fp32(const ColumnParams& p, cudaStream_t st) {
  const size_t smem = (size_t)kWarps * kCap32 * (sizeof(float4) + sizeof(float) + sizeof(int));
  const int np = p.n_prec - p.prec_offset;
  if (np <= 1) return launch_cols(k_column_fp32<1>, p, smem, st);
  if (np <= 2) return launch_cols(k_column_fp32<2>, p, smem, st);
  if (np <= 4) return launch_cols(k_column_fp32<4>, p, smem, st);
  if (np <= 8) return launch_cols(k_column_fp32<8>, p, smem, st);
  return launch_cols(k_column_fp32<16>, p, smem, st);
}

cudaError_t launch_column_fp64(const ColumnParams& p, cudaStream_t st) {
  const size_t smem =
      (size_t)kWarps * kCap64 * (sizeof(double2) + sizeof(double) + sizeof(double2) + sizeof(float4) + sizeof(int));
  const int np = p.n_prec - p.prec_offset;
  if (np <= 1) return launch_cols(k_column_fp64<1>, p, smem, st);
  if (np <= 2) return launch_cols(k_column_fp64<2>, p, smem, st);
  return launch_cols(k_column_fp64<4>, p, smem, st);
}

int column_pass_width_fp32() { return 16; }
int column_pass_width_fp64() { return 4; }

// Average over precession angles and the bright-field flip, over the patch.
__global__ void k_epilogue(double* img, int Mx, int ix0, int ix1, int iy0, int iy1, double scale, int bright) {
  const int W = ix1 - ix0;
  const int64_t n = (int64_t)W * (iy1 - iy0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = ix0 + (int)(i % W), iy = iy0 + (int)(i / W);
    double* o = img + ix + (int64_t)Mx * iy;
    double v = __ddiv_rn(*o, scale);
    if (bright) v = DS(1.0, v);
    *o = v;
  }
}

cudaError_t launch_epilogue(double* img, int Mx, int My, int ix0, int ix1, int iy0, int iy1, double scale,
                            int bright, cudaStream_t st) {
  (void)My;
  ++launch_count();
  k_epilogue<<<256, 256, 0, st>>>(img, Mx, ix0, ix1, iy0, iy1, scale, bright);
  return cudaGetLastError();
}

}  // namespace stem
