// Internal declarations of the corrector's CUDA kernels (libstem_nn).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace stem {
namespace nn {

// y = act(conv(x, w) + bias) over NHWC BF16 activations; taps 9 (3 x 3, "same" padding)
// or 1.  Cin a multiple of 16, Cout a multiple of 8.  y is BF16, or FP32 when y_fp32.
// Returns 0, 1 for invalid arguments, 2 for a launch error.
// mask (same shape as y, or null): outputs where mask <= 0 are zeroed, the gradient through
// the ReLU that produced a layer's input.
int conv_fwd(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
             const float* bias, int relu, const __nv_bfloat16* mask, void* y, int y_fp32, cudaStream_t st);
// The strip-persistent kernel for Cout <= 64 and Cin <= 128 (same contract as conv_fwd, whose
// checks have passed); -1 when the layer does not fit it.
int conv_fwd_strip(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
                   const float* bias, int relu, const __nv_bfloat16* mask, void* y, int y_fp32, cudaStream_t st);

// gw[co][t][ci] += sum over pixels of gy[p][co] x[p + d_t][ci] (FP32, accumulated), the
// partial sums of the pixel split in ws (conv_wgrad_workspace floats), added in a fixed order.
size_t conv_wgrad_workspace(int B, int H, int W, int Cin, int Cout, int taps);
int conv_wgrad(const __nv_bfloat16* x, const __nv_bfloat16* gy, int B, int H, int W, int Cin, int Cout, int taps,
               float* gw, float* ws, size_t ws_floats, cudaStream_t st);

// wt[ci][taps - 1 - t][co] = w[co][t][ci]: input-gradient weights.
int flip_transpose(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int taps, int Cin, cudaStream_t st);

// Element-wise layers (nn_ops.cu); NHWC BF16 unless stated.
int avgpool2(const __nv_bfloat16* x, __nv_bfloat16* y, int B, int H, int W, int C, cudaStream_t st);
int avgpool2_bwd(const __nv_bfloat16* gy, __nv_bfloat16* gx, int B, int H, int W, int C, cudaStream_t st);
int upsample2(const __nv_bfloat16* x, __nv_bfloat16* y, int B, int H, int W, int C, cudaStream_t st);
int upsample2_bwd(const __nv_bfloat16* gy, __nv_bfloat16* gx, int B, int H, int W, int C, cudaStream_t st);
// y = concat(upsample2(d), e), H x W the full-resolution size
int upsample2_concat(const __nv_bfloat16* d, const __nv_bfloat16* e, __nv_bfloat16* y, int B, int H, int W, int Cd,
                     int Ce, cudaStream_t st);
int concat(const __nv_bfloat16* a, const __nv_bfloat16* b, __nv_bfloat16* y, long long npix, int Ca, int Cb,
           cudaStream_t st);
int split(const __nv_bfloat16* gy, __nv_bfloat16* ga, __nv_bfloat16* gb, long long npix, int Ca, int Cb,
          cudaStream_t st);
int relu_mask(__nv_bfloat16* g, const __nv_bfloat16* y, long long n, cudaStream_t st);
// gb[c] += sum over pixels of g[p][c], per-block partial sums in ws (bias_grad_workspace
// floats) added in block order.
size_t bias_grad_workspace(int C);
int bias_grad(const __nv_bfloat16* g, float* gb, long long npix, int C, float* ws, size_t ws_floats, cudaStream_t st);
int mse(const float* pred, const float* target, const float* target1, __nv_bfloat16* g, float* loss, long long npix,
        int Cp, float w1, cudaStream_t st);
int adam(float* w, float* m, float* v, const float* g, __nv_bfloat16* w16, long long n, float lr, float b1, float b2,
         float eps, int step, float wd, cudaStream_t st);
int pack(const float* planes, int nplanes, __nv_bfloat16* y, long long npix, int C, cudaStream_t st);
int to_bf16(const float* x, __nv_bfloat16* y, long long n, cudaStream_t st);
int add(__nv_bfloat16* a, const __nv_bfloat16* b, long long n, cudaStream_t st);
int image_mean(const double* img, long long n, double* mean, cudaStream_t st);
int resample_planes(const double* img2, int Mx2, int My2, int Mx8, int My8, int Wp, int Hp, float sg_value,
                    const double* mean, float contrast, float* planes, cudaStream_t st);
int apply_correction(const float* base, const float* pred, int Cp, int Mx8, int My8, int Wp, float scale, double* out,
                     cudaStream_t st);
int tile_maxabs(const float* pred, int Cp, int ch, int Mx8, int My8, int Wp, int T, float* tile_max, cudaStream_t st);
int tile_flags(const float* tile_max, int ntx, int nty, float thresh, int border, unsigned char* mask, int* count,
               cudaStream_t st);
int merge_tiles(const double* fine, const unsigned char* mask, int ntx, int T, int Mx, int My, double* out,
                cudaStream_t st);

// First failure recorded by a corrector kernel (0 = none), then cleared; synchronises.
int take_error();

}  // namespace nn
}  // namespace stem
