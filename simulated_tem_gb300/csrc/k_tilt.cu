// The two passes of the -ng tilt search that scale with the problem, on the GPU.
//
// k_tilt_scores: findBestRotationMatrix gives every candidate incident vector khat a
// score, the sum over the permitted reflections g (all but [000] and [hkl]) of the
// perfect-crystal intensity |phi_g(L)|^2 at the deviation parameter of g under khat
// (src/Lib_DiffractionConditions.f90:267-276, scoreForIncidentVector1 :1835-1867,
// energy_deviation_parameter :1265-1299, intensityAtDepthZ :1209-1259).  A task is one
// incident vector and one slice of kTiltSlice reflections; a persistent grid of warps
// takes the tasks in turn (even load over the SMs), each lane every 32nd reflection of
// the slice, the lanes' sums added in a fixed tree; the host adds the slices of a vector
// in order, so the scores are deterministic.  Every product, sum and quotient is
// the reference's own, in its order, rounded separately (no fused multiply-adds): a
// score differs from the host's only through the sine and cosine of the two phases and
// the order of the final sum, which the host bounds when it resolves near-ties.
//
// k_foil_thickness: findFoilThickness (src/Lib_DynamicalTwoBeamImaging.f90:486-564)
// with -surf: the highest and lowest atom of each column of about 3 a0 over the 27
// periodic replicas.  Minima and maxima are exact, so the grid equals the host's bit
// for bit whatever the order; doubles are compared through an order-preserving 64-bit
// key so the block-level and global merges are integer atomics.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace stem {
namespace {

__global__ void __launch_bounds__(256) k_tilt_scores(TiltScores p, const double* __restrict__ khat,
                                                     const double* __restrict__ ghkl, const double* __restrict__ bg,
                                                     double* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const int n_slices = (p.nn - 2 + kTiltSlice - 1) / kTiltSlice;
  const int64_t tasks = (int64_t)p.nk * n_slices;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = (int64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); t < tasks; t += warps) {  // warp-uniform
    const int w = (int)(t / n_slices), sl = (int)(t % n_slices);
    const double k0 = khat[3 * w], k1 = khat[3 * w + 1], k2 = khat[3 * w + 2];
    const int j1 = min(p.nn, 2 + (sl + 1) * kTiltSlice);
    double s = 0.0;
    for (int j = 2 + sl * kTiltSlice + lane; j < j1; j += 32) {
      const double g0 = ghkl[3 * j], g1 = ghkl[3 * j + 1], g2 = ghkl[3 * j + 2];
      // energy_deviation_parameter: ((k.g) cst + g1 g1 + g2 g2 + g3 g3) HBAR^2 / 2 ME
      double eps = __dadd_rn(__dadd_rn(__dmul_rn(k0, g0), __dmul_rn(k1, g1)), __dmul_rn(k2, g2));
      eps = __dmul_rn(p.cst, eps);
      eps = __dadd_rn(__dadd_rn(__dadd_rn(eps, __dmul_rn(g0, g0)), __dmul_rn(g1, g1)), __dmul_rn(g2, g2));
      eps = __dmul_rn(eps, p.hbar2on2m);
      const double sg = -__ddiv_rn(eps, p.den);  // energyToLengthDeviationParameter
      // intensityAtDepthZ(xi_g(1), xi_g(j), sg, L)
      const double aa = __dmul_rn(p.twopi, sg);
      const double b = bg[j];
      const double dd = __dsqrt_rn(__dadd_rn(__dmul_rn(__dmul_rn(aa, aa), 0.25), __dmul_rn(b, b)));
      const double c = __dadd_rn(p.b0, __dmul_rn(aa, 0.5));
      const double l1 = __dadd_rn(c, dd), l2 = __dsub_rn(c, dd);
      double s1, c1, s2, c2;
      sincos(__dmul_rn(l1, p.foil), &s1, &c1);
      sincos(__dmul_rn(l2, p.foil), &s2, &c2);
      const double d2 = __dmul_rn(2.0, dd);
      const double re = __ddiv_rn(__dmul_rn(__dsub_rn(c1, c2), b), d2);
      const double im = __ddiv_rn(__dmul_rn(__dsub_rn(s1, s2), b), d2);
      s = __dadd_rn(s, __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
    if (lane == 0) part[t] = s;
  }
}

// The FP32 screen of the same scores, with a bound on each screened score's error.  Per
// term the phases lambda L carry the FP32 rounding of the energy deviation (a difference
// of terms up to cst |g| and |g|^2) and of the phase products; a phase error e moves the
// term by at most 3 e (bg / dd)^2, and the term's own rounding adds a few ulps of it.
// part2 holds (partial score, partial error bound) per task.
__global__ void __launch_bounds__(256) k_tilt_screen(TiltScores p, const float* __restrict__ khat,
                                                     const float* __restrict__ ghkl, const float* __restrict__ bg,
                                                     float* __restrict__ part2) {
  const int lane = threadIdx.x & 31;
  const int n_slices = (p.nn - 2 + kTiltSlice - 1) / kTiltSlice;
  const int64_t tasks = (int64_t)p.nk * n_slices;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const float cst = (float)p.cst, h2 = (float)p.hbar2on2m, den = (float)p.den, twopi = (float)p.twopi;
  const float b0 = (float)p.b0, L = (float)p.foil;
  const float u = 1.1920929e-07f;  // 2^-23
  const float k_eps = L * 3.1415927f * (h2 / den) * 16.f * u;  // phase error per unit of |cst k.g| + |g|^2
  for (int64_t t = (int64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); t < tasks; t += warps) {
    const int w = (int)(t / n_slices), sl = (int)(t % n_slices);
    const float k0 = khat[3 * w], k1 = khat[3 * w + 1], k2 = khat[3 * w + 2];
    const int j1 = min(p.nn, 2 + (sl + 1) * kTiltSlice);
    float s = 0.f, err = 0.f;
    for (int j = 2 + sl * kTiltSlice + lane; j < j1; j += 32) {
      const float g0 = ghkl[3 * j], g1 = ghkl[3 * j + 1], g2 = ghkl[3 * j + 2];
      const float kg = cst * (k0 * g0 + k1 * g1 + k2 * g2), gg = g0 * g0 + g1 * g1 + g2 * g2;
      const float aa = twopi * (-((kg + gg) * h2) / den);
      const float b = bg[j];
      const float dd = sqrtf(aa * aa * 0.25f + b * b);
      const float c = b0 + aa * 0.5f;
      const float ph1 = (c + dd) * L, ph2 = (c - dd) * L;
      float s1, c1, s2, c2;
      sincosf(ph1, &s1, &c1);
      sincosf(ph2, &s2, &c2);
      const float f = b / (2.f * dd);
      const float re = (c1 - c2) * f, im = (s1 - s2) * f;
      const float term = re * re + im * im;
      s += term;
      const float e = 8.f * u * (fabsf(ph1) + fabsf(ph2) + 1.f) + k_eps * (fabsf(kg) + gg);
      err += 3.f * e * (4.f * f * f) + 16.f * u * term;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      err += __shfl_down_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
      part2[2 * t] = s;
      part2[2 * t + 1] = err;
    }
  }
}

// order-preserving key of a double (no NaNs on this path)
__device__ __forceinline__ unsigned long long order_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_foil_init(unsigned long long* __restrict__ top, unsigned long long* __restrict__ thick, int n,
                            unsigned long long top0, unsigned long long thick0) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    top[i] = top0;
    thick[i] = thick0;
  }
}

// The column of the replica nn of atom x, or -1 (src/Lib_DynamicalTwoBeamImaging.f90:541-546).
__device__ __forceinline__ int foil_column(const FoilGrid& f, const double* x, int nn, double& z) {
  const double* r = f.Ruvw + 3 * nn;
  const double y0 = __dadd_rn(x[0], r[0]), y1 = __dadd_rn(x[1], r[1]), y2 = __dadd_rn(x[2], r[2]);
  double xx[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    xx[i] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(f.RU[i], y0), __dmul_rn(f.RU[3 + i], y1)),
                                __dmul_rn(f.RU[6 + i], y2)),
                      f.delta[i]);
  const double fx = floor(__dmul_rn(f.ddx, xx[0]));
  if (!(fx >= 0.0 && fx <= (double)(f.Nx - 1))) return -1;
  const double fy = floor(__dmul_rn(f.ddy, xx[1]));
  if (!(fy >= 0.0 && fy <= (double)(f.Ny - 1))) return -1;
  if (floor(__dmul_rn(f.id3, xx[2])) != 0.0) return -1;
  z = xx[2];
  return (int)fx + f.Nx * (int)fy;
}

// shared-memory grid: 2 * Nx * Ny keys per block, merged into the global grid at the end
__global__ void __launch_bounds__(256) k_foil_thickness_smem(FoilGrid f, const double* __restrict__ x, int64_t ldx,
                                                             int64_t n, unsigned long long* __restrict__ top,
                                                             unsigned long long* __restrict__ thick) {
  extern __shared__ unsigned long long sm[];
  const int cells = f.Nx * f.Ny;
  unsigned long long* stop = sm;
  unsigned long long* sthick = sm + cells;
  for (int c = threadIdx.x; c < cells; c += blockDim.x) {
    stop[c] = ~0ull;
    sthick[c] = 0ull;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* xi = x + i * ldx;
    const double xa[3] = {xi[0], xi[1], xi[2]};
    for (int nn = 0; nn < f.nuvw; ++nn) {
      double z;
      const int c = foil_column(f, xa, nn, z);
      if (c < 0) continue;
      const unsigned long long k = order_key(z);
      atomicMin(&stop[c], k);
      atomicMax(&sthick[c], k);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < cells; c += blockDim.x) {
    if (stop[c] != ~0ull) atomicMin(&top[c], stop[c]);
    if (sthick[c] != 0ull) atomicMax(&thick[c], sthick[c]);
  }
}

__global__ void __launch_bounds__(256) k_foil_thickness_global(FoilGrid f, const double* __restrict__ x,
                                                               int64_t ldx, int64_t n,
                                                               unsigned long long* __restrict__ top,
                                                               unsigned long long* __restrict__ thick) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* xi = x + i * ldx;
    const double xa[3] = {xi[0], xi[1], xi[2]};
    for (int nn = 0; nn < f.nuvw; ++nn) {
      double z;
      const int c = foil_column(f, xa, nn, z);
      if (c < 0) continue;
      const unsigned long long k = order_key(z);
      atomicMin(&top[c], k);
      atomicMax(&thick[c], k);
    }
  }
}

unsigned long long host_order_key(double v) {
  unsigned long long b;
  static_assert(sizeof b == sizeof v, "64-bit double");
  __builtin_memcpy(&b, &v, sizeof b);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

}  // namespace

double order_key_value(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double v;
  __builtin_memcpy(&v, &b, sizeof v);
  return v;
}

int tilt_slices(int nn) { return nn > 2 ? (nn - 2 + kTiltSlice - 1) / kTiltSlice : 0; }

cudaError_t launch_tilt_scores(const TiltScores& p, const double* d_khat, const double* d_ghkl, const double* d_bg,
                               double* d_part, cudaStream_t st) {
  const int64_t tasks = (int64_t)p.nk * tilt_slices(p.nn);
  if (tasks <= 0) return cudaSuccess;
  // persistent: five resident blocks of eight warps per SM (48 registers a thread)
  const int64_t want = (tasks + 7) / 8;
  const int blocks = (int)(want < 5 * 152 ? want : 5 * 152);
  k_tilt_scores<<<blocks, 256, 0, st>>>(p, d_khat, d_ghkl, d_bg, d_part);
  return cudaGetLastError();
}

cudaError_t launch_tilt_screen(const TiltScores& p, const float* d_khat, const float* d_ghkl, const float* d_bg,
                               float* d_part2, cudaStream_t st) {
  const int64_t tasks = (int64_t)p.nk * tilt_slices(p.nn);
  if (tasks <= 0) return cudaSuccess;
  const int64_t want = (tasks + 7) / 8;
  const int blocks = (int)(want < 8 * 152 ? want : 8 * 152);
  k_tilt_screen<<<blocks, 256, 0, st>>>(p, d_khat, d_ghkl, d_bg, d_part2);
  return cudaGetLastError();
}

cudaError_t launch_foil_thickness(const FoilGrid& f, const double* d_x, int64_t ldx, int64_t n,
                                  unsigned long long* d_top, unsigned long long* d_thick, double top0, double thick0,
                                  cudaStream_t st) {
  const int cells = f.Nx * f.Ny;
  if (cells <= 0) return cudaErrorInvalidValue;
  k_foil_init<<<(cells + 255) / 256 < 1024 ? (cells + 255) / 256 : 1024, 256, 0, st>>>(
      d_top, d_thick, cells, host_order_key(top0), host_order_key(thick0));
  if (n <= 0) return cudaGetLastError();
  const int64_t want = (n + 255) / 256;
  const size_t smem = 2 * (size_t)cells * sizeof(unsigned long long);
  if (smem <= kFoilSmemMax) {
    const int blocks = (int)(want < 4 * 152 ? want : 4 * 152);
    if (smem > 48 * 1024) {
      const cudaError_t e =
          cudaFuncSetAttribute(k_foil_thickness_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    k_foil_thickness_smem<<<blocks, 256, smem, st>>>(f, d_x, ldx, n, d_top, d_thick);
  } else {
    const int blocks = (int)(want < 16 * 152 ? want : 16 * 152);
    k_foil_thickness_global<<<blocks, 256, 0, st>>>(f, d_x, ldx, n, d_top, d_thick);
  }
  return cudaGetLastError();
}

}  // namespace stem
