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
 * multiple of 8; y BF16, or FP32 when y_fp32.  bias may be null. */
int stn_conv2d_fwd(const void* x, int32_t B, int32_t H, int32_t W, int32_t Cin, const void* w, int32_t Cout,
                   int32_t taps, const float* bias, int32_t relu, void* y, int32_t y_fp32, void* stream);

/* First failure recorded by a corrector kernel since the last call (0 = none; 1 = a
 * tensor-core wait ran out), then cleared.  Synchronises the device. */
int stn_last_kernel_error(void);

#ifdef __cplusplus
}
#endif

#endif
