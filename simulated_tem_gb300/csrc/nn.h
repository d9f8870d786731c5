// Internal declarations of the corrector's CUDA kernels (libstem_nn).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace stem {
namespace nn {

// y = act(conv(x, w) + bias) over NHWC BF16 activations; taps 9 (3 x 3, "same" padding)
// or 1.  Cin a multiple of 16, Cout a multiple of 8.  y is BF16, or FP32 when y_fp32.
// Returns 0, 1 for invalid arguments, 2 for a launch error.
int conv_fwd(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
             const float* bias, int relu, void* y, int y_fp32, cudaStream_t st);

// First failure recorded by a corrector kernel (0 = none), then cleared; synchronises.
int take_error();

}  // namespace nn
}  // namespace stem
