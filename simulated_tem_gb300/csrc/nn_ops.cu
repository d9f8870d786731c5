// Element-wise and reduction layers of the learned corrector (NHWC, BF16 activations,
// FP32 where a sum or a parameter update needs it).  Memory-bound: grid-stride loops
// over 16-byte vectors where the channel count allows.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nn.h"

namespace stem {
namespace nn {
namespace {

constexpr int kBlock = 256;

int grid_for(long long n) {
  long long g = (n + kBlock - 1) / kBlock;
  if (g < 1) g = 1;
  if (g > 16384) g = 16384;
  return (int)g;
}

__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 tobf(float v) { return __float2bfloat16_rn(v); }

// Eight BF16 channels as one 16-byte vector, and their FP32 values.
struct V8 {
  float f[8];
};
__device__ __forceinline__ V8 load8(const __nv_bfloat16* p) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
  V8 r;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    r.f[2 * i] = f.x;
    r.f[2 * i + 1] = f.y;
  }
  return r;
}
__device__ __forceinline__ void store8(__nv_bfloat16* p, const V8& v) {
  __align__(16) __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v.f[2 * i], v.f[2 * i + 1]);
  *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(h);
}

// The layers below run one thread per (pixel, 8 channels) with 32-bit pixel indices (the
// convolutions limit a tensor to fewer than 2^31 pixels); C is a multiple of 8.

// y[b, i, j, c] = (x[b, 2i, 2j] + x[b, 2i, 2j + 1] + x[b, 2i + 1, 2j] + x[b, 2i + 1, 2j + 1]) / 4
__global__ void k_avgpool2(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int B, int H, int W,
                           int C) {
  const int Ho = H / 2, Wo = W / 2, V = C / 8;
  const long long n = (long long)B * Ho * Wo * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % V) * 8;
    const unsigned po = (unsigned)(i / V);  // output pixel
    const unsigned j = po % Wo, r = po / Wo;
    const unsigned ii = r % Ho, b = r / Ho;
    const __nv_bfloat16* s = x + ((size_t)(b * H + 2 * ii) * W + 2 * j) * C + c;
    const V8 a = load8(s), bb = load8(s + C), cc = load8(s + (size_t)W * C), d = load8(s + (size_t)W * C + C);
    V8 o;
#pragma unroll
    for (int k = 0; k < 8; ++k) o.f[k] = 0.25f * ((a.f[k] + bb.f[k]) + (cc.f[k] + d.f[k]));
    store8(y + (size_t)po * C + c, o);
  }
}

// gx[b, y, x, c] = gy[b, y / 2, x / 2, c] / 4
__global__ void k_avgpool2_bwd(const __nv_bfloat16* __restrict__ gy, __nv_bfloat16* __restrict__ gx, int B, int H,
                               int W, int C) {
  const int Ho = H / 2, Wo = W / 2, V = C / 8;
  const long long n = (long long)B * H * W * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % V) * 8;
    const unsigned p = (unsigned)(i / V);
    const unsigned xw = p % W, r = p / W;
    const unsigned yh = r % H, b = r / H;
    V8 v = load8(gy + ((size_t)(b * Ho + yh / 2) * Wo + xw / 2) * C + c);
#pragma unroll
    for (int k = 0; k < 8; ++k) v.f[k] *= 0.25f;
    store8(gx + (size_t)p * C + c, v);
  }
}

// nearest 2x upsampling: y[b, y, x, c] = x[b, y / 2, x / 2, c]
__global__ void k_upsample2(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int B, int H, int W,
                            int C) {
  const int Ho = 2 * H, Wo = 2 * W, V = C / 8;
  const long long n = (long long)B * Ho * Wo * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % V) * 8;
    const unsigned p = (unsigned)(i / V);
    const unsigned xw = p % Wo, r = p / Wo;
    const unsigned yh = r % Ho, b = r / Ho;
    *reinterpret_cast<uint4*>(y + (size_t)p * C + c) =
        *reinterpret_cast<const uint4*>(x + ((size_t)(b * H + yh / 2) * W + xw / 2) * C + c);
  }
}

// y = concat(upsample2(d), e): y[b, y, x, 0:Cd] = d[b, y / 2, x / 2], y[b, y, x, Cd:] =
// e[b, y, x] (H, W: the full-resolution sizes); the upsampled tensor is never stored
__global__ void k_upsample2_concat(const __nv_bfloat16* __restrict__ d, const __nv_bfloat16* __restrict__ e,
                                   __nv_bfloat16* __restrict__ y, int B, int H, int W, int Cd, int Ce) {
  const int C = Cd + Ce, V = C / 8, Hd = H / 2, Wd = W / 2;
  const long long n = (long long)B * H * W * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % V) * 8;
    const unsigned p = (unsigned)(i / V);
    uint4 v;
    if (c < Cd) {
      const unsigned xw = p % W, r = p / W;
      const unsigned yh = r % H, b = r / H;
      v = *reinterpret_cast<const uint4*>(d + ((size_t)(b * Hd + yh / 2) * Wd + xw / 2) * Cd + c);
    } else {
      v = *reinterpret_cast<const uint4*>(e + (size_t)p * Ce + (c - Cd));
    }
    *reinterpret_cast<uint4*>(y + (size_t)p * C + c) = v;
  }
}

// the same on a grid of (vectors of one row, rows): 32-bit index arithmetic in the row
__global__ void k_upsample2_concat_rows(const __nv_bfloat16* __restrict__ d, const __nv_bfloat16* __restrict__ e,
                                        __nv_bfloat16* __restrict__ y, int H, int W, int Cd, int Ce) {
  const int C = Cd + Ce, V = C / 8, Hd = H / 2, Wd = W / 2;
  const int row = blockIdx.y, b = row / H, yh = row % H;
  const size_t drow = (size_t)(b * Hd + yh / 2) * Wd;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < W * V; j += gridDim.x * blockDim.x) {
    const int c = (j % V) * 8, xw = j / V;
    const size_t p = (size_t)row * W + xw;
    const uint4 v = c < Cd ? *reinterpret_cast<const uint4*>(d + (drow + xw / 2) * Cd + c)
                           : *reinterpret_cast<const uint4*>(e + p * Ce + (c - Cd));
    *reinterpret_cast<uint4*>(y + p * C + c) = v;
  }
}

// gx[b, i, j, c] = sum of gy over the 2 x 2 block it was copied to (FP32 sum, one rounding)
__global__ void k_upsample2_bwd(const __nv_bfloat16* __restrict__ gy, __nv_bfloat16* __restrict__ gx, int B, int H,
                                int W, int C) {
  const int Wo = 2 * W, V = C / 8;
  const long long n = (long long)B * H * W * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % V) * 8;
    const unsigned p = (unsigned)(i / V);
    const unsigned j = p % W, r = p / W;
    const unsigned ii = r % H, b = r / H;
    const __nv_bfloat16* s = gy + ((size_t)(b * 2 * H + 2 * ii) * Wo + 2 * j) * C + c;
    const V8 a = load8(s), bb = load8(s + C), cc = load8(s + (size_t)Wo * C), dd = load8(s + (size_t)Wo * C + C);
    V8 o;
#pragma unroll
    for (int k = 0; k < 8; ++k) o.f[k] = (a.f[k] + bb.f[k]) + (cc.f[k] + dd.f[k]);
    store8(gx + (size_t)p * C + c, o);
  }
}

// y[p, 0:Ca] = a[p], y[p, Ca:Ca+Cb] = b[p]  (both channel counts multiples of 8)
__global__ void k_concat(const __nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b,
                         __nv_bfloat16* __restrict__ y, long long npix, int Ca, int Cb) {
  const int C = Ca + Cb, V = C / 8;
  const long long n = npix * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long p = i / V;
    const int c = (int)(i % V) * 8;
    const uint4 v = c < Ca ? *reinterpret_cast<const uint4*>(a + p * Ca + c)
                           : *reinterpret_cast<const uint4*>(b + p * Cb + (c - Ca));
    *reinterpret_cast<uint4*>(y + p * C + c) = v;
  }
}

// the inverse: ga[p] = gy[p, 0:Ca], gb[p] = gy[p, Ca:Ca+Cb] (either output may be null)
__global__ void k_split(const __nv_bfloat16* __restrict__ gy, __nv_bfloat16* __restrict__ ga,
                        __nv_bfloat16* __restrict__ gb, long long npix, int Ca, int Cb) {
  const int C = Ca + Cb, V = C / 8;
  const long long n = npix * V;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long p = i / V;
    const int c = (int)(i % V) * 8;
    const uint4 v = *reinterpret_cast<const uint4*>(gy + p * C + c);
    if (c < Ca) {
      if (ga) *reinterpret_cast<uint4*>(ga + p * Ca + c) = v;
    } else if (gb) {
      *reinterpret_cast<uint4*>(gb + p * Cb + (c - Ca)) = v;
    }
  }
}

// g *= (y > 0): the gradient through a ReLU whose output was y
__global__ void k_relu_mask(__nv_bfloat16* __restrict__ g, const __nv_bfloat16* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (!(bf(y[i]) > 0.f)) g[i] = tobf(0.f);
}

// gb[c] += sum_p g[p, c] in a fixed order: block b sums the pixels of its range (thread
// (r, c) the pixels r, r + R, ... of it, R = 256 / C rows of threads, then the rows in
// order) into part[b][c]; a second kernel adds the blocks' sums in block order.
constexpr int kBiasBlocks = 256;

__global__ void k_bias_grad_part(const __nv_bfloat16* __restrict__ g, float* __restrict__ part, long long npix,
                                 int C) {
  extern __shared__ float rows_sum[];  // [R][Cg]
  const long long per = (npix + gridDim.x - 1) / gridDim.x;
  const long long p0 = blockIdx.x * per, p1 = min(npix, p0 + per);
  for (int c0 = 0; c0 < C; c0 += blockDim.x) {
    const int Cg = min((int)blockDim.x, C - c0);
    const int R = blockDim.x / Cg;
    const int r = threadIdx.x / Cg, c = threadIdx.x - r * Cg;
    float s = 0.f;
    if (r < R)
      for (long long p = p0 + r; p < p1; p += R) s += bf(g[p * C + c0 + c]);
    if (r < R) rows_sum[r * Cg + c] = s;
    __syncthreads();
    if (threadIdx.x < Cg) {
      float t = 0.f;
      for (int k = 0; k < R; ++k) t += rows_sum[k * Cg + threadIdx.x];
      part[(size_t)blockIdx.x * C + c0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

__global__ void k_bias_grad_sum(const float* __restrict__ part, int nb, int C, float* __restrict__ gb) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    float t = 0.f;
    for (int b = 0; b < nb; ++b) t += part[(size_t)b * C + c];
    gb[c] += t;
  }
}

// loss = mean_p (pred[p, 0] - target[p])^2 + w1 mean_p (pred[p, 1] - t1[p])^2 over npix
// pixels (pred FP32 [npix][Cp]), t1 = target1[p] or, without target1, |target[p]|: channel
// 0 regresses the target, channel 1 (when w1 > 0) a magnitude; g (BF16 [npix][Cp]) = the
// loss gradient, 0 in the other channels.  The loss is added to *loss.
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target,
                      const float* __restrict__ target1, __nv_bfloat16* __restrict__ g, float* __restrict__ loss,
                      long long npix, int Cp, float w1) {
  __shared__ float red[kBlock / 32];
  float s = 0.f;
  const float scale = 2.f / (float)npix;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const float t = target[p];
    const float d = pred[p * Cp] - t;
    const float d1 = w1 > 0.f ? pred[p * Cp + 1] - (target1 ? target1[p] : fabsf(t)) : 0.f;
    s += d * d + w1 * d1 * d1;
    if (g) {
      g[p * Cp] = tobf(scale * d);
      for (int c = 1; c < Cp; ++c) g[p * Cp + c] = tobf(c == 1 ? scale * w1 * d1 : 0.f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w];
    atomicAdd(loss, t / (float)npix);
  }
}

// Adam on FP32 master parameters; the BF16 copy (if any) is refreshed.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ w16, long long n, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, float wd) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (w16) w16[i] = tobf(wi);
  }
}

// pack FP32 planes [nplanes][npix] into BF16 NHWC [npix][C] (channels >= nplanes zero)
__global__ void k_pack(const float* __restrict__ planes, int nplanes, __nv_bfloat16* __restrict__ y, long long npix,
                       int C) {
  const long long n = npix * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long long p = i / C;
    y[i] = tobf(c < nplanes ? planes[(long long)c * npix + p] : 0.f);
  }
}

// the same, one thread per pixel: C / 8 vectors of 8 channels (y 16-byte aligned)
__global__ void k_pack_vec(const float* __restrict__ planes, int nplanes, __nv_bfloat16* __restrict__ y,
                           long long npix, int C) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    for (int c0 = 0; c0 < C; c0 += 8) {
      __align__(16) __nv_bfloat16 h[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) h[k] = tobf(c0 + k < nplanes ? planes[(long long)(c0 + k) * npix + p] : 0.f);
      *reinterpret_cast<uint4*>(y + p * C + c0) = *reinterpret_cast<const uint4*>(h);
    }
  }
}

// FP32 -> BF16 copy
__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = tobf(x[i]);
}

// a += b (BF16, FP32 arithmetic)
__global__ void k_add(__nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = tobf(bf(a[i]) + bf(b[i]));
}

// mean[0] = sum of img / n (FP64), one block in a fixed order (the images are coarse:
// a few 1e5 pixels)
__global__ void __launch_bounds__(1024) k_image_mean(const double* __restrict__ img, long long n,
                                                     double* __restrict__ mean) {
  __shared__ double red[32];
  double s = 0.0;
  // each thread adds img[t], img[t + 1024], ... in that order; eight loads in flight
  const long long step = blockDim.x;
  for (long long base = threadIdx.x; base < n; base += 8 * step) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = base + k * step < n ? img[base + k * step] : 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (base + k * step < n) s += v[k];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w];
    mean[0] = t / (double)n;
  }
}

// The corrector's planes on the fine (M = 8) pixel grid, Hp x Wp (the image My8 x Mx8,
// extended by its last row and column).  DF is the coarse (M = 2) image interpolated
// bilinearly at the fine pixels' positions (pixel i of an N-pixel axis sits at i d / N on
// both grids); the fine pixels past the last coarse pixel extrapolate from the last two
// (the tilted crystal makes the image non-periodic, and a clamped edge would be a step
// the network must learn).  mu is the coarse image's mean.  Planes (FP32 [5][Hp][Wp]):
// 0: (DF - mu) * contrast, 1: (BF - (1 - mu)) * contrast with BF = 1 - DF, 2: sg_value,
// 3: mu, 4: DF (the base the correction is added to).  Planes 0-3 are the network's input:
// the contrast, a few 1e-3 on a level near 0.1-0.7, would not survive BF16 unshifted.
// img2: FP64 (Mx2, My2) column-major.
__global__ void k_resample_planes(const double* __restrict__ img2, int Mx2, int My2, int Mx8, int My8, int Wp, int Hp,
                                  float sg_value, const double* __restrict__ mean, float contrast,
                                  float* __restrict__ planes) {
  // grid: x over the row's pixels, y over the rows, striding by the grid's height (at most
  // 65,535 rows per launch) -- no 64-bit division per pixel
  const long long n = (long long)Wp * Hp;
  const int qx = blockIdx.x * blockDim.x + threadIdx.x;
  if (qx >= Wp) return;
  const double sx = (double)Mx2 / Mx8, sy = (double)My2 / My8;
  const double mu = *mean;
  for (int qy = blockIdx.y; qy < Hp; qy += gridDim.y) {
    const long long i = (long long)qy * Wp + qx;
    // bilinear between the two nearest coarse pixels; past the last coarse pixel (the
    // fine grid's last quarter pixel-row and column) the last two extrapolate linearly
    const int px = min(qx, Mx8 - 1), py = min(qy, My8 - 1);
    const double u = px * sx, v = py * sy;
    const int i0 = max(0, min((int)floor(u), Mx2 - 2)), j0 = max(0, min((int)floor(v), My2 - 2));
    const double fu = u - i0, fv = v - j0;
    const int i1 = min(i0 + 1, Mx2 - 1), j1 = min(j0 + 1, My2 - 1);
    const double a = img2[i0 + (long long)Mx2 * j0], b = img2[i1 + (long long)Mx2 * j0];
    const double c = img2[i0 + (long long)Mx2 * j1], d = img2[i1 + (long long)Mx2 * j1];
    const double df = (1.0 - fv) * ((1.0 - fu) * a + fu * b) + fv * ((1.0 - fu) * c + fu * d);
    planes[i] = (float)((df - mu) * contrast);
    planes[n + i] = (float)(-(df - mu) * contrast);
    planes[2 * n + i] = sg_value;
    planes[3 * n + i] = (float)mu;
    planes[4 * n + i] = (float)df;
  }
}

// out (FP64, Mx8 x My8 column-major) = base + pred[p][0] * scale, p over the Hp x Wp
// grid's top-left My8 x Mx8 block.
// grid: (pixels of a row, rows), the rows striding by the grid's height
__global__ void k_apply_correction(const float* __restrict__ base, const float* __restrict__ pred, int Cp, int Mx8,
                                   int My8, int Wp, float scale, double* __restrict__ out) {
  for (int y = blockIdx.y; y < My8; y += gridDim.y)
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < Mx8; x += gridDim.x * blockDim.x) {
      const long long i = (long long)y * Mx8 + x, p = (long long)y * Wp + x;
      out[i] = (double)base[p] + (double)pred[p * Cp] * (double)scale;
    }
}

// tile_max[ty][tx] = max |pred[p][ch]| over the T x T tile (inside Mx8 x My8); one block per tile
__global__ void k_tile_maxabs(const float* __restrict__ pred, int Cp, int ch, int Mx8, int My8, int Wp, int T,
                              float* __restrict__ tile_max) {
  const int tx = blockIdx.x, ty = blockIdx.y;
  float m = 0.f;
  for (int k = threadIdx.x; k < T * T; k += blockDim.x) {
    const int x = tx * T + k % T, y = ty * T + k / T;
    if (x < Mx8 && y < My8) m = fmaxf(m, fabsf(pred[((long long)y * Wp + x) * Cp + ch]));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float red[kBlock / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) t = fmaxf(t, red[w]);
    tile_max[ty * gridDim.x + tx] = t;
  }
}

// mask[t] = tile_max[t] > thresh, or t on the grid's outer ring when border != 0; *count =
// the flagged tiles.  One block: a fixed-order count, no atomics, nothing to clear first.
__global__ void __launch_bounds__(1024) k_tile_flags(const float* __restrict__ tile_max, int ntx, int nty, float thresh,
                                                     int border, unsigned char* __restrict__ mask, int* __restrict__ count) {
  const int n = ntx * nty;
  int c = 0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int tx = t % ntx, ty = t / ntx;
    const bool edge = border && (tx == 0 || ty == 0 || tx == ntx - 1 || ty == nty - 1);
    const unsigned char f = (edge || tile_max[t] > thresh) ? 1 : 0;
    mask[t] = f;
    c += f;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ int red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w];
    *count = t;
  }
}

// out[tile] = fine[tile] for every tile whose mask byte is nonzero (FP64 images, Mx x My
// column-major)
// grid: (pixels of a row, rows), the rows striding by the grid's height
__global__ void k_merge_tiles(const double* __restrict__ fine, const unsigned char* __restrict__ mask, int ntx, int T,
                              int Mx, int My, double* __restrict__ out) {
  for (int y = blockIdx.y; y < My; y += gridDim.y) {
    const unsigned char* mrow = mask + (y / T) * ntx;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < Mx; x += gridDim.x * blockDim.x) {
      const long long i = (long long)y * Mx + x;
      if (mrow[x / T]) out[i] = fine[i];
    }
  }
}

int status() { return cudaGetLastError() == cudaSuccess ? 0 : 2; }

}  // namespace

bool pix_ok(int B, int H, int W, int C) {
  return B >= 1 && H >= 1 && W >= 1 && C >= 8 && C % 8 == 0 && (long long)B * H * W < (1LL << 31);
}
int avgpool2(const __nv_bfloat16* x, __nv_bfloat16* y, int B, int H, int W, int C, cudaStream_t st) {
  if (!x || !y || H % 2 || W % 2 || !pix_ok(B, H, W, C)) return 1;
  k_avgpool2<<<grid_for((long long)B * H * W * C / 32), kBlock, 0, st>>>(x, y, B, H, W, C);
  return status();
}
int avgpool2_bwd(const __nv_bfloat16* gy, __nv_bfloat16* gx, int B, int H, int W, int C, cudaStream_t st) {
  if (!gy || !gx || H % 2 || W % 2 || !pix_ok(B, H, W, C)) return 1;
  k_avgpool2_bwd<<<grid_for((long long)B * H * W * C / 8), kBlock, 0, st>>>(gy, gx, B, H, W, C);
  return status();
}
int upsample2(const __nv_bfloat16* x, __nv_bfloat16* y, int B, int H, int W, int C, cudaStream_t st) {
  if (!x || !y || !pix_ok(B, 2 * H, 2 * W, C)) return 1;
  k_upsample2<<<grid_for((long long)B * H * W * C / 2), kBlock, 0, st>>>(x, y, B, H, W, C);
  return status();
}
int upsample2_concat(const __nv_bfloat16* d, const __nv_bfloat16* e, __nv_bfloat16* y, int B, int H, int W, int Cd,
                     int Ce, cudaStream_t st) {
  if (!d || !e || !y || H % 2 || W % 2 || Cd % 8 || !pix_ok(B, H, W, Cd + Ce) || Ce < 8 || Ce % 8) return 1;
  const long long rows = (long long)B * H, per_row = (long long)W * (Cd + Ce) / 8;
  if (rows <= 65535) {
    const dim3 grid((unsigned)((per_row + kBlock - 1) / kBlock), (unsigned)rows);
    k_upsample2_concat_rows<<<grid, kBlock, 0, st>>>(d, e, y, H, W, Cd, Ce);
  } else {
    k_upsample2_concat<<<grid_for(rows * per_row), kBlock, 0, st>>>(d, e, y, B, H, W, Cd, Ce);
  }
  return status();
}
int upsample2_bwd(const __nv_bfloat16* gy, __nv_bfloat16* gx, int B, int H, int W, int C, cudaStream_t st) {
  if (!gy || !gx || !pix_ok(B, 2 * H, 2 * W, C)) return 1;
  k_upsample2_bwd<<<grid_for((long long)B * H * W * C / 8), kBlock, 0, st>>>(gy, gx, B, H, W, C);
  return status();
}
int concat(const __nv_bfloat16* a, const __nv_bfloat16* b, __nv_bfloat16* y, long long npix, int Ca, int Cb,
           cudaStream_t st) {
  if (!a || !b || !y || Ca % 8 || Cb % 8) return 1;
  k_concat<<<grid_for(npix * (Ca + Cb) / 8), kBlock, 0, st>>>(a, b, y, npix, Ca, Cb);
  return status();
}
int split(const __nv_bfloat16* gy, __nv_bfloat16* ga, __nv_bfloat16* gb, long long npix, int Ca, int Cb,
          cudaStream_t st) {
  if (!gy || Ca % 8 || Cb % 8) return 1;
  k_split<<<grid_for(npix * (Ca + Cb) / 8), kBlock, 0, st>>>(gy, ga, gb, npix, Ca, Cb);
  return status();
}
int relu_mask(__nv_bfloat16* g, const __nv_bfloat16* y, long long n, cudaStream_t st) {
  if (!g || !y) return 1;
  k_relu_mask<<<grid_for(n), kBlock, 0, st>>>(g, y, n);
  return status();
}
size_t bias_grad_workspace(int C) { return C < 1 ? 0 : (size_t)kBiasBlocks * C; }
int bias_grad(const __nv_bfloat16* g, float* gb, long long npix, int C, float* ws, size_t ws_floats, cudaStream_t st) {
  if (!g || !gb || !ws || C < 1 || C > 4096 || npix < 0 || ws_floats < bias_grad_workspace(C)) return 1;
  k_bias_grad_part<<<kBiasBlocks, 256, 256 * sizeof(float), st>>>(g, ws, npix, C);
  k_bias_grad_sum<<<(C + 255) / 256, 256, 0, st>>>(ws, kBiasBlocks, C, gb);
  return status();
}
int mse(const float* pred, const float* target, const float* target1, __nv_bfloat16* g, float* loss, long long npix,
        int Cp, float w1, cudaStream_t st) {
  if (!pred || !target || !loss || Cp < 1 || (w1 > 0.f && Cp < 2)) return 1;
  k_mse<<<grid_for(npix / 4), kBlock, 0, st>>>(pred, target, target1, g, loss, npix, Cp, w1);
  return status();
}
int adam(float* w, float* m, float* v, const float* g, __nv_bfloat16* w16, long long n, float lr, float b1, float b2,
         float eps, int step, float wd, cudaStream_t st) {
  if (!w || !m || !v || !g || step < 1) return 1;
  float bc1 = 1.f, bc2 = 1.f;
  for (int i = 0; i < step && i < 100000; ++i) {
    bc1 *= b1;
    bc2 *= b2;
  }
  k_adam<<<grid_for(n), kBlock, 0, st>>>(w, m, v, g, w16, n, lr, b1, b2, eps, 1.f - bc1, 1.f - bc2, wd);
  return status();
}
int pack(const float* planes, int nplanes, __nv_bfloat16* y, long long npix, int C, cudaStream_t st) {
  if (!planes || !y || nplanes < 1 || nplanes > C) return 1;
  if (C % 8 == 0 && ((uintptr_t)y & 15) == 0)
    k_pack_vec<<<grid_for(npix), kBlock, 0, st>>>(planes, nplanes, y, npix, C);
  else
    k_pack<<<grid_for(npix * C), kBlock, 0, st>>>(planes, nplanes, y, npix, C);
  return status();
}
int add(__nv_bfloat16* a, const __nv_bfloat16* b, long long n, cudaStream_t st) {
  if (!a || !b) return 1;
  k_add<<<grid_for(n), kBlock, 0, st>>>(a, b, n);
  return status();
}
int image_mean(const double* img, long long n, double* mean, cudaStream_t st) {
  if (!img || !mean || n < 1) return 1;
  k_image_mean<<<1, 1024, 0, st>>>(img, n, mean);
  return status();
}
int resample_planes(const double* img2, int Mx2, int My2, int Mx8, int My8, int Wp, int Hp, float sg_value,
                    const double* mean, float contrast, float* planes, cudaStream_t st) {
  if (!img2 || !planes || !mean || Mx2 < 1 || My2 < 1 || Mx8 < 1 || My8 < 1 || Wp < Mx8 || Hp < My8) return 1;
  const dim3 grid((Wp + kBlock - 1) / kBlock, Hp < 65535 ? Hp : 65535);
  k_resample_planes<<<grid, kBlock, 0, st>>>(img2, Mx2, My2, Mx8, My8, Wp, Hp, sg_value, mean, contrast, planes);
  return status();
}
int apply_correction(const float* base, const float* pred, int Cp, int Mx8, int My8, int Wp, float scale, double* out,
                     cudaStream_t st) {
  if (!base || !pred || !out || Wp < Mx8) return 1;
  if (Mx8 < 1 || My8 < 1) return 0;
  k_apply_correction<<<dim3((Mx8 + kBlock - 1) / kBlock, My8 < 65535 ? My8 : 65535), kBlock, 0, st>>>(
      base, pred, Cp, Mx8, My8, Wp, scale, out);
  return status();
}
int tile_maxabs(const float* pred, int Cp, int ch, int Mx8, int My8, int Wp, int T, float* tile_max, cudaStream_t st) {
  if (!pred || !tile_max || T < 1 || Wp < Mx8 || ch < 0 || ch >= Cp) return 1;
  dim3 grid((Mx8 + T - 1) / T, (My8 + T - 1) / T);
  k_tile_maxabs<<<grid, kBlock, 0, st>>>(pred, Cp, ch, Mx8, My8, Wp, T, tile_max);
  return status();
}
int tile_flags(const float* tile_max, int ntx, int nty, float thresh, int border, unsigned char* mask, int* count,
               cudaStream_t st) {
  if (!tile_max || !mask || !count || ntx < 1 || nty < 1) return 1;
  k_tile_flags<<<1, 1024, 0, st>>>(tile_max, ntx, nty, thresh, border, mask, count);
  return status();
}
int merge_tiles(const double* fine, const unsigned char* mask, int ntx, int T, int Mx, int My, double* out,
                cudaStream_t st) {
  if (!fine || !mask || !out || T < 1 || ntx < (Mx + T - 1) / T) return 1;
  if (My < 1 || Mx < 1) return 0;
  k_merge_tiles<<<dim3((Mx + kBlock - 1) / kBlock, My < 65535 ? My : 65535), kBlock, 0, st>>>(fine, mask, ntx, T, Mx,
                                                                                            My, out);
  return status();
}
int to_bf16(const float* x, __nv_bfloat16* y, long long n, cudaStream_t st) {
  if (!x || !y) return 1;
  k_to_bf16<<<grid_for(n), kBlock, 0, st>>>(x, y, n);
  return status();
}

}  // namespace nn
}  // namespace stem
