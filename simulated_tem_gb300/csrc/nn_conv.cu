// Convolution kernels of the learned corrector on the fifth-generation tensor cores.
//
// A 3 x 3 ("same" padding) or 1 x 1 convolution over NHWC BF16 activations is an
// implicit GEMM: D[p, co] = sum_k A[p, k] B[co, k] with p the output pixel, k = (tap,
// ci) and A gathered from the input on the fly (zero outside the image).  A CTA of four
// warps owns 128 pixels x BN output channels; the FP32 accumulator lives in TMEM
// (BN columns).  K advances in chunks of KC = min(64, Cin) channels of one tap: all
// threads gather the A and B chunk into shared memory (two stages, so gathering chunk
// c + 1 overlaps the MMAs of chunk c), one thread issues the tcgen05 MMAs (K = 16 each)
// and commits them to the stage's mbarrier.  The epilogue reads TMEM with tcgen05.ld,
// adds the bias, applies ReLU and stores BF16 (or FP32) NHWC.
//
// Every wait on an mbarrier is bounded; a wait that runs out records an error in
// g_nn_error, waits once more (bounded) for the MMAs in flight and still frees TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nn.h"
#include "tc_sm100.cuh"

namespace stem {
namespace nn {

__device__ int g_nn_error = 0;  // first failure code of a corrector kernel (0 = none)

namespace {

constexpr int kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 20;  // polls of an mbarrier before giving up (about a second)

struct ConvArgs {
  const __nv_bfloat16* x;     // [B][H][W][Cin]
  const __nv_bfloat16* w;     // [Cout][taps][Cin]
  const float* bias;          // [Cout] or null
  const __nv_bfloat16* mask;  // [B][H][W][Cout] or null: outputs where mask <= 0 are zeroed
  void* y;                    // [B][H][W][Cout], BF16 or FP32
  int B, H, W, Cin, Cout, taps, relu, y_fp32;
};

template <int BN, int KC>
struct Smem {
  alignas(1024) unsigned char a[2][128 * KC * 2];
  alignas(1024) unsigned char b[2][BN * KC * 2];
  alignas(8) unsigned long long mbar[2];
  uint32_t tmem;
};

// Gather chunk (tap, ci0) of A (128 pixels from p0) and B (BN output channels from n0).
template <int BN, int KC>
__device__ __forceinline__ void gather(const ConvArgs& a, int p0, int n0, int tap, int ci0, unsigned char* sa,
                                       unsigned char* sb) {
  const int t = threadIdx.x;
  const int npix = a.B * a.H * a.W;
  const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
  // A: thread t owns pixel row t; KC / 8 units of 16 bytes
  {
    const int p = p0 + t;
    const __nv_bfloat16* src = nullptr;
    if (p < npix) {
      const int xw = p % a.W;
      const int rest = p / a.W;
      const int yh = rest % a.H, b = rest / a.H;
      const int yy = yh + dy, xx = xw + dx;
      if (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
        src = a.x + (((size_t)b * a.H + yy) * a.W + xx) * a.Cin + ci0;
    }
#pragma unroll
    for (int u = 0; u < KC / 8; ++u) {
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (src) v = *reinterpret_cast<const uint4*>(src + 8 * u);
      *reinterpret_cast<uint4*>(sa + tc::tile_offset(t, 8 * u, KC)) = v;
    }
  }
  // B: BN rows of KC
#pragma unroll
  for (int r = t; r < BN; r += kThreads) {
    const int n = n0 + r;
    const __nv_bfloat16* src = n < a.Cout ? a.w + ((size_t)n * a.taps + tap) * a.Cin + ci0 : nullptr;
#pragma unroll
    for (int u = 0; u < KC / 8; ++u) {
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (src) v = *reinterpret_cast<const uint4*>(src + 8 * u);
      *reinterpret_cast<uint4*>(sb + tc::tile_offset(r, 8 * u, KC)) = v;
    }
  }
}

template <int BN, int KC>
__global__ void __launch_bounds__(kThreads) k_conv_fwd(const ConvArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Smem<BN, KC>& S = *reinterpret_cast<Smem<BN, KC>*>(
      smem_raw + ((1024 - ((uintptr_t)smem_raw & 1023)) & 1023));
  const int t = threadIdx.x, warp = t >> 5;
  const int p0 = blockIdx.x * 128, n0 = blockIdx.y * BN;

  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&S.tmem), BN < 32 ? 32 : BN);
  if (t == 0) {
    tc::mbar_init(tc::smem_addr(&S.mbar[0]), 1);
    tc::mbar_init(tc::smem_addr(&S.mbar[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;

  const int chunks_per_tap = a.Cin / KC;
  const int nchunks = a.taps * chunks_per_tap;
  constexpr uint32_t idesc = tc::make_idesc_bf16(128, BN);
  // every decision to go on is CTA-uniform (__syncthreads_and), so no thread leaves a
  // barrier or a warp-collective TMEM load behind
  bool ok = true;
  int issued = 0;  // chunks whose MMAs were issued
  for (int c = 0; c < nchunks; ++c) {
    const int st = c & 1;
    if (c >= 2) ok = tc::mbar_wait(tc::smem_addr(&S.mbar[st]), ((c - 2) >> 1) & 1, kWaitLimit);
    ok = __syncthreads_and(ok);
    if (!ok) break;
    gather<BN, KC>(a, p0, n0, c / chunks_per_tap, (c % chunks_per_tap) * KC, S.a[st], S.b[st]);
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_addr(S.a[st]), sb = tc::smem_addr(S.b[st]);
#pragma unroll
      for (int s = 0; s < KC / 16; ++s)
        tc::mma_bf16(tmem, tc::make_desc(sa + 256 * s, 128, KC * 16), tc::make_desc(sb + 256 * s, 128, KC * 16),
                     idesc, (c > 0 || s > 0) ? 1u : 0u);
      tc::mma_commit(tc::smem_addr(&S.mbar[st]));
    }
    issued = c + 1;
  }
  // the last commit covers every MMA issued before it
  if (issued > 0) {
    const int last = issued - 1;
    bool done = tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    done = __syncthreads_and(done);
    if (!done) tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    ok = ok && done;
  }
  if (!ok && t == 0) atomicCAS(&g_nn_error, 0, 1);
  tc::fence_after_sync();

  if (ok) {
    // epilogue: warp w holds TMEM lanes (pixels) 32w .. 32w + 31
    const int p = p0 + 32 * warp + (t & 31);
    const int npix = a.B * a.H * a.W;
    for (int col = 0; col < BN; col += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)col, v);
      const int n = n0 + col;
      if (p < npix && n < a.Cout) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          if (a.bias) v[i] += a.bias[n + i];
          if (a.relu) v[i] = fmaxf(v[i], 0.f);
        }
        if (a.mask) {  // gradient through the ReLU that produced this layer's input
          const uint4 mv = *reinterpret_cast<const uint4*>(a.mask + (size_t)p * a.Cout + n);
          const __nv_bfloat16* m = reinterpret_cast<const __nv_bfloat16*>(&mv);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!(__bfloat162float(m[i]) > 0.f)) v[i] = 0.f;
        }
        if (a.y_fp32) {
          float* dst = reinterpret_cast<float*>(a.y) + (size_t)p * a.Cout + n;
          *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
          *reinterpret_cast<float4*>(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
        } else {
          __align__(16) __nv_bfloat162 h[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
          *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.y) + (size_t)p * a.Cout + n) =
              *reinterpret_cast<const uint4*>(h);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, BN < 32 ? 32 : BN);
}

template <int BN, int KC>
cudaError_t launch_fwd(const ConvArgs& a, cudaStream_t st) {
  const size_t smem = sizeof(Smem<BN, KC>) + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_conv_fwd<BN, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int npix = a.B * a.H * a.W;
  dim3 grid((npix + 127) / 128, (a.Cout + BN - 1) / BN);
  k_conv_fwd<BN, KC><<<grid, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int KC>
cudaError_t launch_fwd_kc(const ConvArgs& a, cudaStream_t st) {
  if (a.Cout <= 32) return launch_fwd<32, KC>(a, st);
  if (a.Cout <= 64) return launch_fwd<64, KC>(a, st);
  return launch_fwd<128, KC>(a, st);
}

}  // namespace

int conv_fwd(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
             const float* bias, int relu, const __nv_bfloat16* mask, void* y, int y_fp32, cudaStream_t st) {
  if (!x || !w || !y || B < 1 || H < 1 || W < 1) return 1;
  if (Cin < 16 || Cin % 16 != 0 || Cout < 8 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return 1;
  if ((long long)B * H * W >= (1LL << 31)) return 1;
  ConvArgs a{x, w, bias, mask, y, B, H, W, Cin, Cout, taps, relu, y_fp32};
  cudaError_t e;
  if (Cin % 64 == 0)
    e = launch_fwd_kc<64>(a, st);
  else if (Cin % 32 == 0)
    e = launch_fwd_kc<32>(a, st);
  else
    e = launch_fwd_kc<16>(a, st);
  return e == cudaSuccess ? 0 : 2;
}

namespace {

// ---------------------------------------------------------------------------
// Weight gradient: gw[co, t, ci] += sum_p gy[p, co] x[p + d_t, ci]
// ---------------------------------------------------------------------------
// GEMM per tap with K = pixels: A[co, p] = gy[p, co], B_t[ci, p] = x[p + d_t, ci], both
// transposed while staged (K-major tiles, p along K).  A CTA owns 128 output channels x
// BN input channels x TG taps (TG x BN TMEM columns) for one range of pixels, in chunks
// of 64 pixels; the A tile of a chunk serves all TG taps.  Partial sums over the CTA's
// pixels go to the CTA's slice of a workspace (one slice per pixel split), which a second
// kernel adds to the FP32 gradient in split order: the result does not depend on the
// order in which CTAs finish (training is reproducible).
struct WgradArgs {
  const __nv_bfloat16* x;   // [B][H][W][Cin]
  const __nv_bfloat16* gy;  // [B][H][W][Cout]
  float* ws;                // [splits][Cout][taps][Cin] partial sums
  int B, H, W, Cin, Cout, taps;
  int chunks_per_cta;       // 64-pixel chunks per CTA (pixel split)
};

template <int BN, int TG>
struct WSmem {
  alignas(1024) unsigned char a[2][128 * 64 * 2];
  alignas(1024) unsigned char b[2][TG][BN * 64 * 2];
  alignas(8) unsigned long long mbar[2];
  uint32_t tmem;
};

__host__ __device__ constexpr int tmem_cols(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512; }

// Stage 8 consecutive channels of pixel p (or zeros) as column kp of rows r0 .. r0 + 7.
__device__ __forceinline__ void put_column8(unsigned char* tile, int r0, int kp, const __nv_bfloat16* src) {
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (src) v = *reinterpret_cast<const uint4*>(src);
  const unsigned short* h = reinterpret_cast<const unsigned short*>(&v);
#pragma unroll
  for (int i = 0; i < 8; ++i) *reinterpret_cast<unsigned short*>(tile + tc::tile_offset(r0 + i, kp, 64)) = h[i];
}

template <int BN, int TG>
__global__ void __launch_bounds__(kThreads) k_conv_wgrad(const WgradArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  WSmem<BN, TG>& S = *reinterpret_cast<WSmem<BN, TG>*>(smem_raw + ((1024 - ((uintptr_t)smem_raw & 1023)) & 1023));
  const int t = threadIdx.x, warp = t >> 5;
  const int m0 = blockIdx.y * 128;                    // output channels
  const int n_ctiles = (a.Cin + BN - 1) / BN;
  const int c0 = (blockIdx.z % n_ctiles) * BN;        // input channels
  const int t0 = (blockIdx.z / n_ctiles) * TG;        // first tap of the group
  const int ntap = min(TG, a.taps - t0);
  const int npix = a.B * a.H * a.W;
  const int chunk0 = blockIdx.x * a.chunks_per_cta;
  const int nchunks = max(0, min(a.chunks_per_cta, (npix + 63) / 64 - chunk0));
  constexpr int kCols = tmem_cols(TG * BN);

  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&S.tmem), kCols);
  if (t == 0) {
    tc::mbar_init(tc::smem_addr(&S.mbar[0]), 1);
    tc::mbar_init(tc::smem_addr(&S.mbar[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  constexpr uint32_t idesc = tc::make_idesc_bf16(128, BN);

  const int kp = t & 63, half = t >> 6;
  bool ok = true;
  int issued = 0;
  for (int c = 0; c < nchunks; ++c) {
    const int st = c & 1;
    if (c >= 2) ok = tc::mbar_wait(tc::smem_addr(&S.mbar[st]), ((c - 2) >> 1) & 1, kWaitLimit);
    ok = __syncthreads_and(ok);
    if (!ok) break;
    const int p = (chunk0 + c) * 64 + kp;
    int b = 0, yh = 0, xw = 0;
    if (p < npix) {
      xw = p % a.W;
      const int rest = p / a.W;
      yh = rest % a.H;
      b = rest / a.H;
    }
    // A: 128 output channels x 64 pixels
    for (int g = half; g < 16; g += 2) {
      const int co = m0 + 8 * g;
      const __nv_bfloat16* src = (p < npix && co < a.Cout) ? a.gy + (size_t)p * a.Cout + co : nullptr;
      put_column8(S.a[st], 8 * g, kp, src);
    }
    // B_t: BN input channels x 64 pixels, one tile per tap of the group
    for (int j = 0; j < TG; ++j) {
      const int tap = t0 + j;
      const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
      const int yy = yh + dy, xx = xw + dx;
      const bool in = j < ntap && p < npix && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      for (int g = half; g < BN / 8; g += 2) {
        const int ci = c0 + 8 * g;
        const __nv_bfloat16* src =
            (in && ci < a.Cin) ? a.x + (((size_t)b * a.H + yy) * a.W + xx) * a.Cin + ci : nullptr;
        put_column8(S.b[st][j], 8 * g, kp, src);
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_addr(S.a[st]);
      for (int j = 0; j < ntap; ++j) {
        const uint32_t sb = tc::smem_addr(S.b[st][j]);
#pragma unroll
        for (int s = 0; s < 4; ++s)
          tc::mma_bf16(tmem + (uint32_t)(j * BN), tc::make_desc(sa + 256 * s, 128, 64 * 16),
                       tc::make_desc(sb + 256 * s, 128, 64 * 16), idesc, (c > 0 || s > 0) ? 1u : 0u);
      }
      tc::mma_commit(tc::smem_addr(&S.mbar[st]));
    }
    issued = c + 1;
  }
  if (issued > 0) {
    const int last = issued - 1;
    bool done = tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    done = __syncthreads_and(done);
    if (!done) tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    ok = ok && done;
  }
  if (!ok && t == 0) atomicCAS(&g_nn_error, 0, 1);
  tc::fence_after_sync();

  if (ok && issued > 0) {
    const int co = m0 + 32 * warp + (t & 31);
    for (int j = 0; j < ntap; ++j) {
      for (int col = 0; col < BN; col += 8) {
        float v[8];
        tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(j * BN + col), v);
        const int ci = c0 + col;
        if (co < a.Cout && ci < a.Cin) {
          float* dst = a.ws + (size_t)blockIdx.x * a.Cout * a.taps * a.Cin + ((size_t)co * a.taps + t0 + j) * a.Cin + ci;
          reinterpret_cast<float4*>(dst)[0] = make_float4(v[0], v[1], v[2], v[3]);
          reinterpret_cast<float4*>(dst)[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// gw[i] += sum over splits s (in order) of ws[s][i]
__global__ void k_wgrad_reduce(const float* __restrict__ ws, int splits, long long n, float* __restrict__ gw) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += ws[(size_t)k * n + i];
    gw[i] += s;
  }
}

// Pixel split of a weight-gradient launch: about two waves of CTAs, at least 8 chunks per
// CTA so the partial sums amortise.
template <int BN, int TG>
void wgrad_split(int B, int H, int W, int Cin, int Cout, int taps, int& splits, int& chunks_per_cta) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int npix = B * H * W;
  const int chunks = (npix + 63) / 64;
  const int tiles = ((Cout + 127) / 128) * ((Cin + BN - 1) / BN) * ((taps + TG - 1) / TG);
  splits = (2 * sms + tiles - 1) / tiles;
  splits = max(1, min(splits, (chunks + 7) / 8));
  chunks_per_cta = (chunks + splits - 1) / splits;
  splits = (chunks + chunks_per_cta - 1) / chunks_per_cta;
}

template <int BN, int TG>
cudaError_t launch_wgrad(WgradArgs a, float* gw, size_t ws_floats, cudaStream_t st) {
  const size_t smem = sizeof(WSmem<BN, TG>) + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad<BN, TG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int splits = 1;
  wgrad_split<BN, TG>(a.B, a.H, a.W, a.Cin, a.Cout, a.taps, splits, a.chunks_per_cta);
  const long long n = (long long)a.Cout * a.taps * a.Cin;
  if ((size_t)splits * (size_t)n > ws_floats) return cudaErrorInvalidValue;
  dim3 grid(splits, (a.Cout + 127) / 128, ((a.Cin + BN - 1) / BN) * ((a.taps + TG - 1) / TG));
  k_conv_wgrad<BN, TG><<<grid, kThreads, smem, st>>>(a);
  const long long blocks = (n + 255) / 256;
  k_wgrad_reduce<<<(int)(blocks < 1024 ? blocks : 1024), 256, 0, st>>>(a.ws, splits, n, gw);
  return cudaGetLastError();
}

template <int BN, int TG>
size_t wgrad_ws(int B, int H, int W, int Cin, int Cout, int taps) {
  int splits = 1, cpc = 1;
  wgrad_split<BN, TG>(B, H, W, Cin, Cout, taps, splits, cpc);
  return (size_t)splits * Cout * taps * Cin;
}

// wt[ci][8 - t][co] = w[co][t][ci] (taps 9) or wt[ci][0][co] = w[co][0][ci]: the weights
// of the input gradient as a forward convolution of the output gradient.
__global__ void k_flip_transpose(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt, int Cout,
                                 int taps, int Cin) {
  const int n = Cout * taps * Cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % Cin;
    const int rest = i / Cin;
    const int tp = rest % taps, co = rest / taps;
    wt[((size_t)ci * taps + (taps - 1 - tp)) * Cout + co] = w[i];
  }
}

}  // namespace

bool wgrad_args_ok(int B, int H, int W, int Cin, int Cout, int taps) {
  if (B < 1 || H < 1 || W < 1) return false;
  if (Cin < 8 || Cin % 8 != 0 || Cout < 8 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return false;
  return (long long)B * H * W < (1LL << 31);
}

size_t conv_wgrad_workspace(int B, int H, int W, int Cin, int Cout, int taps) {
  if (!wgrad_args_ok(B, H, W, Cin, Cout, taps)) return 0;
  if (taps == 1)
    return Cin <= 32 ? wgrad_ws<32, 1>(B, H, W, Cin, Cout, taps)
                     : Cin <= 64 ? wgrad_ws<64, 1>(B, H, W, Cin, Cout, taps) : wgrad_ws<128, 1>(B, H, W, Cin, Cout, taps);
  return Cin <= 32 ? wgrad_ws<32, 9>(B, H, W, Cin, Cout, taps)
                   : Cin <= 64 ? wgrad_ws<64, 3>(B, H, W, Cin, Cout, taps) : wgrad_ws<128, 3>(B, H, W, Cin, Cout, taps);
}

int conv_wgrad(const __nv_bfloat16* x, const __nv_bfloat16* gy, int B, int H, int W, int Cin, int Cout, int taps,
               float* gw, float* ws, size_t ws_floats, cudaStream_t st) {
  if (!x || !gy || !gw || !ws || !wgrad_args_ok(B, H, W, Cin, Cout, taps)) return 1;
  if (ws_floats < conv_wgrad_workspace(B, H, W, Cin, Cout, taps)) return 1;
  WgradArgs a{x, gy, ws, B, H, W, Cin, Cout, taps, 1};
  cudaError_t e;
  if (taps == 1)
    e = Cin <= 32 ? launch_wgrad<32, 1>(a, gw, ws_floats, st)
                  : Cin <= 64 ? launch_wgrad<64, 1>(a, gw, ws_floats, st) : launch_wgrad<128, 1>(a, gw, ws_floats, st);
  else
    e = Cin <= 32 ? launch_wgrad<32, 9>(a, gw, ws_floats, st)
                  : Cin <= 64 ? launch_wgrad<64, 3>(a, gw, ws_floats, st) : launch_wgrad<128, 3>(a, gw, ws_floats, st);
  return e == cudaSuccess ? 0 : 2;
}

int flip_transpose(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int taps, int Cin, cudaStream_t st) {
  if (!w || !wt || Cout < 1 || Cin < 1 || (taps != 1 && taps != 9)) return 1;
  const int n = Cout * taps * Cin;
  k_flip_transpose<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(w, wt, Cout, taps, Cin);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int take_error() {
  int v = 0, zero = 0;
  cudaDeviceSynchronize();
  cudaMemcpyFromSymbol(&v, g_nn_error, sizeof v);
  cudaMemcpyToSymbol(g_nn_error, &zero, sizeof zero);
  return v;
}

}  // namespace nn
}  // namespace stem
