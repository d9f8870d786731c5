// C ABI of libstem_nn (include/stem_nn.h).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/stem_nn.h"
#include "nn.h"

using namespace stem::nn;

extern "C" int stn_conv2d_fwd(const void* x, int32_t B, int32_t H, int32_t W, int32_t Cin, const void* w,
                              int32_t Cout, int32_t taps, const float* bias, int32_t relu, void* y, int32_t y_fp32,
                              void* stream) {
  return conv_fwd(static_cast<const __nv_bfloat16*>(x), B, H, W, Cin, static_cast<const __nv_bfloat16*>(w), Cout,
                  taps, bias, relu, y, y_fp32, (cudaStream_t)stream);
}

extern "C" int stn_last_kernel_error(void) { return take_error(); }
