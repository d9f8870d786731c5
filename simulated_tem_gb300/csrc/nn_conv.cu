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
  const __nv_bfloat16* x;  // [B][H][W][Cin]
  const __nv_bfloat16* w;  // [Cout][taps][Cin]
  const float* bias;       // [Cout] or null
  void* y;                 // [B][H][W][Cout], BF16 or FP32
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
             const float* bias, int relu, void* y, int y_fp32, cudaStream_t st) {
  if (!x || !w || !y || B < 1 || H < 1 || W < 1) return 1;
  if (Cin < 16 || Cin % 16 != 0 || Cout < 8 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return 1;
  if ((long long)B * H * W >= (1LL << 31)) return 1;
  ConvArgs a{x, w, bias, y, B, H, W, Cin, Cout, taps, relu, y_fp32};
  cudaError_t e;
  if (Cin % 64 == 0)
    e = launch_fwd_kc<64>(a, st);
  else if (Cin % 32 == 0)
    e = launch_fwd_kc<32>(a, st);
  else
    e = launch_fwd_kc<16>(a, st);
  return e == cudaSuccess ? 0 : 2;
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
