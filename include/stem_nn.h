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
 * mask (BF16, y's shape) is <= 0 the output is zeroed (the gradient through a ReLU).
 * Layers the strip kernel does not take first copy w into a library-owned device buffer
 * in the order the kernel loads it (one buffer per device, kept and grown to the largest
 * layer: 1.2 MB for the corrector); calls from several threads or streams take turns on
 * it, in stream order. */
int stn_conv2d_fwd(const void* x, int32_t B, int32_t H, int32_t W, int32_t Cin, const void* w, int32_t Cout,
                   int32_t taps, const float* bias, int32_t relu, const void* mask, void* y, int32_t y_fp32,
                   void* stream);

/* Weight gradient, accumulated: gw[co][t][ci] += sum over pixels of gy[p][co] x[p + d_t][ci]
 * (gw FP32; x [B][H][W][Cin], gy [B][H][W][Cout] BF16; Cin, Cout multiples of 8).  ws: FP32
 * device workspace of at least stn_conv2d_wgrad_workspace(...) floats (0 = invalid
 * arguments) for the partial sums of the pixel split, which are added in a fixed order, so
 * the gradient does not depend on scheduling. */
int64_t stn_conv2d_wgrad_workspace(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, int32_t taps);
int stn_conv2d_wgrad(const void* x, const void* gy, int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout,
                     int32_t taps, float* gw, float* ws, int64_t ws_floats, void* stream);

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

/* The decoder's input in one pass: y = [upsample2(d), e] along channels, y and e of
 * B x H x W pixels, d of B x H/2 x W/2 (Cd, Ce multiples of 8); the upsampled tensor is not
 * stored. */
int stn_upsample2_concat(const void* d, const void* e, void* y, int32_t B, int32_t H, int32_t W, int32_t Cd,
                         int32_t Ce, void* stream);

/* Channel concatenation y = [a, b] and its inverse (Ca, Cb multiples of 8; ga or gb may be
 * null). */
int stn_concat(const void* a, const void* b, void* y, int64_t npix, int32_t Ca, int32_t Cb, void* stream);
int stn_split(const void* gy, void* ga, void* gb, int64_t npix, int32_t Ca, int32_t Cb, void* stream);

/* g *= (y > 0), element-wise over n values. */
int stn_relu_mask(void* g, const void* y, int64_t n, void* stream);

/* gb[c] += sum over pixels of g[p][c] (gb FP32), in a fixed order through a workspace of
 * stn_bias_grad_workspace(C) floats. */
int64_t stn_bias_grad_workspace(int32_t C);
int stn_bias_grad(const void* g, float* gb, int64_t npix, int32_t C, float* ws, int64_t ws_floats, void* stream);

/* *loss += mean over pixels of (pred[p][0] - target[p])^2 + w1 (pred[p][1] - t1[p])^2 with
 * t1 = target1[p], or |target[p]| when target1 is null (pred FP32 [npix][Cp], targets FP32
 * [npix]; the second term when w1 > 0).  g (BF16 [npix][Cp], may be null) = the loss
 * gradient, zero in the other channels. */
int stn_mse(const float* pred, const float* target, const float* target1, void* g, float* loss, int64_t npix,
            int32_t Cp, float w1, void* stream);

/* One Adam step (step >= 1) on FP32 parameters w with moments m, v and gradient g; w16
 * (BF16, may be null) receives the updated parameters.  wd: decoupled weight decay. */
int stn_adam(float* w, float* m, float* v, const float* g, void* w16, int64_t n, float lr, float beta1, float beta2,
             float eps, int32_t step, float wd, void* stream);

/* Planes [nplanes][npix] FP32 -> NHWC BF16 [npix][C] (channels >= nplanes zero); FP32 ->
 * BF16 copy. */
int stn_pack(const float* planes, int32_t nplanes, void* y, int64_t npix, int32_t C, void* stream);
int stn_to_bf16(const float* x, void* y, int64_t n, void* stream);

/* a += b (BF16, n values); memset of `bytes` bytes to zero. */
int stn_add(void* a, const void* b, int64_t n, void* stream);
int stn_fill_zero(void* p, int64_t bytes, void* stream);

/* *mean = the mean of an FP64 image of n pixels (device scalar). */
int stn_image_mean(const double* img, int64_t n, double* mean, void* stream);

/* The corrector's planes on the fine grid (Hp x Wp >= My8 x Mx8, extended by the last row
 * and column): with DF the coarse image img2 (FP64 Mx2 x My2, column-major) interpolated
 * bilinearly at the fine pixels' positions (pixel i of an N-pixel axis at i d / N, clamped
 * at the edges) and mu = *mean,
 * planes (FP32 [5][Hp][Wp]) = (DF - mu) contrast, (mu - DF) contrast, sg_value, mu, DF. */
int stn_resample_planes(const double* img2, int32_t Mx2, int32_t My2, int32_t Mx8, int32_t My8, int32_t Wp,
                        int32_t Hp, float sg_value, const double* mean, float contrast, float* planes, void* stream);

/* out (FP64 Mx8 x My8 column-major) = base + pred[..][0] * scale (base FP32 [Hp][Wp], pred
 * FP32 [Hp][Wp][Cp]). */
int stn_apply_correction(const float* base, const float* pred, int32_t Cp, int32_t Mx8, int32_t My8, int32_t Wp,
                         float scale, double* out, void* stream);

/* Per T x T tile of the Mx8 x My8 image: max |pred[..][ch]| -> tile_max [ceil(My8/T)][ceil(Mx8/T)]. */
int stn_tile_maxabs(const float* pred, int32_t Cp, int32_t ch, int32_t Mx8, int32_t My8, int32_t Wp, int32_t T,
                    float* tile_max, void* stream);

/* The fallback's tile mask, on the device: mask (uint8 [nty][ntx]) = tile_max > thresh, or
 * the tile on the grid's outer ring when border != 0; *count (device int32) = the flagged
 * tiles.  The mask feeds st_image_device_masked and stn_merge_tiles directly. */
int stn_tile_flags(const float* tile_max, int32_t ntx, int32_t nty, float thresh, int32_t border, uint8_t* mask,
                   int32_t* count, void* stream);

/* out = fine on every T x T tile whose mask byte (uint8 [ceil(My/T)][ntx]) is nonzero. */
int stn_merge_tiles(const double* fine, const uint8_t* mask, int32_t ntx, int32_t T, int32_t Mx, int32_t My,
                    double* out, void* stream);

/* First failure recorded by a corrector kernel since the last call (0 = none; 1 = a
 * tensor-core wait ran out), then cleared.  Synchronises the device. */
int stn_last_kernel_error(void);

#ifdef __cplusplus
}
#endif

#endif
