// Output formats of d2bi on the GPU: the 16-bit PNG levels of outputImgAsPng /
// write_greyscale_png (src/d2bi.f90:1509-1538, src/Lib_Png.f90:117-181,
// src/Lib_Greyscale.c:162-260) and the '(1000f12.7)' value records of the .dat file
// (src/d2bi.f90:1429-1457).
//
// PNG levels.  Normalise mode (iso_min == iso_max): a = ONE / (max - min), b = -a min with
// ONE = 1 - 1/65536 (a = 0, b = 1/2 for a flat image); contrast mode: v = clamp((v -
// iso_min) / (iso_max - iso_min), 0, 1), a = 1, b = 0.  Then f = (float)(a v + b) (the
// product and the sum rounded separately), f clamped to [0, 0.999984741] and the level
// is (int)(f * 65536) in float arithmetic; image row y is img[x + nx y].
//
// f12.7 records.  |v| x 10^7 is rounded to the nearest integer of the exact product (its
// rounding error recovered with a fused multiply-add, 10^7 being exact in FP64, and
// consulted when the rounded product lies half-way; an exact tie cannot occur because
// 10^7 has the factor 5^7), then printed right-justified in 12
// characters with at least one integer digit, '-' for negative values, 12 asterisks when
// it does not fit, 1000 values per line.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace stem {
namespace {

__global__ void k_minmax_part(const double* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double smin[8], smax[8];
  double lo = INFINITY, hi = -INFINITY;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    lo = fmin(lo, v[i]);
    hi = fmax(hi, v[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smin[threadIdx.x >> 5] = lo;
    smax[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      lo = fmin(lo, smin[w]);
      hi = fmax(hi, smax[w]);
    }
    part[2 * blockIdx.x] = lo;
    part[2 * blockIdx.x + 1] = hi;
  }
}

// the two coefficients of the level map (a, b), from the partial minima and maxima
__global__ void k_level_coeffs(const double* __restrict__ part, int nparts, int normalise,
                               double* __restrict__ ab) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 1.0, b = 0.0;
  if (normalise) {
    double lo = part[0], hi = part[1];
    for (int i = 1; i < nparts; ++i) {
      lo = fmin(lo, part[2 * i]);
      hi = fmax(hi, part[2 * i + 1]);
    }
    const double one = __dsub_rn(1.0, 1.0 / 65536.0);
    if (__dsub_rn(hi, lo) < 1.0e-16) {
      a = 0.0;
      b = 0.5;
    } else {
      a = __ddiv_rn(one, __dsub_rn(hi, lo));
      b = -__dmul_rn(a, lo);
    }
  }
  ab[0] = a;
  ab[1] = b;
}

__global__ void k_png_levels(const double* __restrict__ img, int nx, int ny, const double* __restrict__ ab,
                             int contrast, double iso_min, double iso_max, uint16_t* __restrict__ levels) {
  const int64_t n = (int64_t)nx * ny;
  const double a = ab[0], b = ab[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = img[i];
    if (contrast) {
      v = __ddiv_rn(__dsub_rn(v, iso_min), __dsub_rn(iso_max, iso_min));
      v = fmax(0.0, fmin(1.0, v));
    }
    float f = __double2float_rn(__dadd_rn(__dmul_rn(a, v), b));
    if ((double)f > 0.999984741)
      f = __double2float_rn(0.999984741);
    else if (f < 0.0f)
      f = 0.0f;
    levels[i] = (uint16_t)(int)__fmul_rn(f, 65536.0f);
  }
}

__device__ __forceinline__ void put12(char* o, const char* s, int len) {
  for (int k = 0; k < 12 - len; ++k) o[k] = ' ';
  for (int k = 0; k < len; ++k) o[12 - len + k] = s[k];
}

__global__ void k_format_f12_7(const double* __restrict__ v, int64_t n, char* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    char* o = out + i * 12 + i / 1000;  // a newline ends every 1000 values
    const double x = v[i];
    char s[24];
    int len = 0;
    if (x != x) {
      s[0] = 'N'; s[1] = 'a'; s[2] = 'N';
      len = 3;
    } else if (isinf(x)) {
      const char* t = x > 0 ? "Infinity" : "-Infinity";
      while (t[len]) {
        s[len] = t[len];
        ++len;
      }
    } else {
      const double ax = fabs(x);
      const double hi = ax * 1.0e7;
      long long q = -1;  // rounded |x| 10^7, or -1 when it needs more than 12 characters
      if (hi < 1.0e12) {
        // ax 10^7 = hi + lo exactly; rint(hi) is the nearest integer unless hi lies exactly
        // half-way, where the sign of lo decides (lo = 0 there would be an exact tie, which
        // 10^7's factor 5^7 rules out; rint's even choice stands then)
        const double lo = fma(ax, 1.0e7, -hi);
        double nr = rint(hi);
        const double dd = hi - nr;  // exact
        if (dd == 0.5 && lo > 0.0) nr += 1.0;
        else if (dd == -0.5 && lo < 0.0) nr -= 1.0;
        q = (long long)nr;
      }
      const bool neg = signbit(x);
      char d[24];
      int nd = 0;
      if (q >= 0) {
        long long ip = q / 10000000LL, fp = q - ip * 10000000LL;
        for (int k = 0; k < 7; ++k) {
          d[nd++] = (char)('0' + fp % 10);
          fp /= 10;
        }
        d[nd++] = '.';
        do {
          d[nd++] = (char)('0' + ip % 10);
          ip /= 10;
        } while (ip > 0);
        if (neg) d[nd++] = '-';
      }
      if (q < 0 || nd > 12) {
        for (int k = 0; k < 12; ++k) o[k] = '*';
        len = -1;
      } else {
        for (int k = 0; k < nd; ++k) s[k] = d[nd - 1 - k];
        len = nd;
      }
    }
    if (len >= 0) put12(o, s, len);
    if (i % 1000 == 999 || i == n - 1) o[12] = '\n';
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 8192) g = 8192;
  return (int)g;
}

}  // namespace

cudaError_t launch_png_levels(const double* d_img, int nx, int ny, double iso_min, double iso_max, double* d_part,
                              double* d_ab, uint16_t* d_levels, cudaStream_t st) {
  const int64_t n = (int64_t)nx * ny;
  const bool contrast = !(iso_max - iso_min == 0.0);
  if (!contrast) {
    k_minmax_part<<<kLevelParts, 256, 0, st>>>(d_img, n, d_part);
    k_level_coeffs<<<1, 32, 0, st>>>(d_part, kLevelParts, 1, d_ab);
  } else {
    k_level_coeffs<<<1, 32, 0, st>>>(d_part, 0, 0, d_ab);
  }
  k_png_levels<<<grid_for(n), 256, 0, st>>>(d_img, nx, ny, d_ab, contrast ? 1 : 0, iso_min, iso_max, d_levels);
  return cudaGetLastError();
}

cudaError_t launch_format_dat(const double* d_v, int64_t n, char* d_text, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_format_f12_7<<<grid_for(n), 256, 0, st>>>(d_v, n, d_text);
  return cudaGetLastError();
}

}  // namespace stem
