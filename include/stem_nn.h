/* libstem_nn: the learned corrector's kernels (BF16 tensor-core convolutions and the
 * element-wise layers around them), hand-written for sm_103a.  No counterpart in the
 * reference: the corrector maps an M = 2 voxel-grid image to M = 8 quality.
 *
 * Layouts: activations NHWC (channels innermost), BF16 unless stated; convolution
 * weights [Cout][taps][Cin] BF16 (taps 9 = a 3 x 3 kernel, row-major (dy, dx), or 1).
 * All pointers are device memory; every call is asynchronous on `stream` and returns 0,
 * or 1 for invalid arguments, 2 for a launch error. */
#ifndef STEM_NN_H
#define STEM_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y = relu?(conv(x, w) + bias): "same" padding, stride 1.  Cin a multiple of 16, Cout a
 * multiple of 8; y BF16, or FP32 when y_fp32.  bias and mask may be null; where
 * mask (BF16, y's shape) is <= 0 the output is zeroed (the gradient through a ReLU). */
int stn_conv2d_fwd(const void* x, int32_t B, int32_t H, int32_t W, int32_t Cin, const void* w, int32_t Cout,
                   int32_t taps, const float* bias, int32_t relu, const void* mask, void* y, int32_t y_fp32,
                   void* stream);

/* Weight gradient, accumulated: gw[co][t][ci] += sum over pixels of gy[p][co] x[p + d_t][ci]
 * (gw FP32; x [B][H][W][Cin], gy [B][H][W][Cout] BF16; Cin, Cout multiples of 8). */
int stn_conv2d_wgrad(const void* x, const void* gy, int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout,
                     int32_t taps, float* gw, void* stream);

/* wt[ci][taps - 1 - t][co] = w[co][t][ci]: the input gradient of a convolution is the
 * convolution of the output gradient with wt. */
int stn_weight_flip(const void* w, void* wt, int32_t Cout, int32_t taps, int32_t Cin, void* stream);

/* 2 x 2 average pooling (H, W even) and its gradient; nearest 2 x upsampling and its
 * gradient (a sum over each 2 x 2 block).  Shapes are those of the larger tensor for the
 * pooling pair and of the smaller one for the upsampling pair. */
int stn_avgpool2(const void* x, void* y, int32_t B, int32_t H, int32_t W, int32_t C, void* stream);
int stn_avgpool2_bwd(const void* gy, void* gx, int32_t B, int32_t H, int32_t W, int32_t C, void* stream);
int stn_upsample2(const void* x, void* y, int32_t B, int32_t H, int32_t W, int32_t C, void* stream);
int stn_upsample2_bwd(const void* gy, void* gx, int32_t B, int32_t H, int32_t W, int32_t C, void* stream);

/* Channel concatenation y = [a, b] and its inverse (Ca, Cb multiples of 8; ga or gb may be
 * null). */
int stn_concat(const void* a, const void* b, void* y, int64_t npix, int32_t Ca, int32_t Cb, void* stream);
int stn_split(const void* gy, void* ga, void* gb, int64_t npix, int32_t Ca, int32_t Cb, void* stream);

/* g *= (y > 0), element-wise over n values. */
int stn_relu_mask(void* g, const void* y, int64_t n, void* stream);

/* gb[c] += sum over pixels of g[p][c] (gb FP32). */
int stn_bias_grad(const void* g, float* gb, int64_t npix, int32_t C, void* stream);

/* *loss += mean over pixels of (pred[p][0] - target[p])^2 (pred FP32 [npix][Cp], target
 * FP32 [npix]); g (BF16 [npix][Cp], may be null) = the loss gradient, zero in channels >= 1. */
int stn_mse(const float* pred, const float* target, void* g, float* loss, int64_t npix, int32_t Cp, void* stream);

/* One Adam step (step >= 1) on FP32 parameters w with moments m, v and gradient g; w16
 * (BF16, may be null) receives the updated parameters.  wd: decoupled weight decay. */
int stn_adam(float* w, float* m, float* v, const float* g, void* w16, int64_t n, float lr, float beta1, float beta2,
             float eps, int32_t step, float wd, void* stream);

/* Planes [nplanes][npix] FP32 -> NHWC BF16 [npix][C] (channels >= nplanes zero); FP32 ->
 * BF16 copy. */
int stn_pack(const float* planes, int32_t nplanes, void* y, int64_t npix, int32_t C, void* stream);
int stn_to_bf16(const float* x, void* y, int64_t n, void* stream);

/* First failure recorded by a corrector kernel since the last call (0 = none; 1 = a
 * tensor-core wait ran out), then cleared.  Synchronises the device. */
int stn_last_kernel_error(void);

#ifdef __cplusplus
}
#endif

#endif
