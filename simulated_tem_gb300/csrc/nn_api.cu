// C ABI of libstem_nn (include/stem_nn.h).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/stem_nn.h"
#include "nn.h"

using namespace stem::nn;

namespace {
typedef __nv_bfloat16 bf16;
inline const bf16* cb(const void* p) { return static_cast<const bf16*>(p); }
inline bf16* mb(void* p) { return static_cast<bf16*>(p); }
inline cudaStream_t cs(void* s) { return (cudaStream_t)s; }
}  // namespace

extern "C" int stn_conv2d_fwd(const void* x, int32_t B, int32_t H, int32_t W, int32_t Cin, const void* w,
                              int32_t Cout, int32_t taps, const float* bias, int32_t relu, const void* mask, void* y,
                              int32_t y_fp32, void* stream) {
  return conv_fwd(cb(x), B, H, W, Cin, cb(w), Cout, taps, bias, relu, cb(mask), y, y_fp32, cs(stream));
}
extern "C" int64_t stn_conv2d_wgrad_workspace(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout,
                                              int32_t taps) {
  return (int64_t)conv_wgrad_workspace(B, H, W, Cin, Cout, taps);
}
extern "C" int stn_conv2d_wgrad(const void* x, const void* gy, int32_t B, int32_t H, int32_t W, int32_t Cin,
                                int32_t Cout, int32_t taps, float* gw, float* ws, int64_t ws_floats, void* stream) {
  if (ws_floats < 0) return 1;
  return conv_wgrad(cb(x), cb(gy), B, H, W, Cin, Cout, taps, gw, ws, (size_t)ws_floats, cs(stream));
}
extern "C" int stn_weight_flip(const void* w, void* wt, int32_t Cout, int32_t taps, int32_t Cin, void* stream) {
  return flip_transpose(cb(w), mb(wt), Cout, taps, Cin, cs(stream));
}
extern "C" int stn_avgpool2(const void* x, void* y, int32_t B, int32_t H, int32_t W, int32_t C, void* stream) {
  return avgpool2(cb(x), mb(y), B, H, W, C, cs(stream));
}
extern "C" int stn_avgpool2_bwd(const void* gy, void* gx, int32_t B, int32_t H, int32_t W, int32_t C, void* stream) {
  return avgpool2_bwd(cb(gy), mb(gx), B, H, W, C, cs(stream));
}
extern "C" int stn_upsample2(const void* x, void* y, int32_t B, int32_t H, int32_t W, int32_t C, void* stream) {
  return upsample2(cb(x), mb(y), B, H, W, C, cs(stream));
}
extern "C" int stn_upsample2_bwd(const void* gy, void* gx, int32_t B, int32_t H, int32_t W, int32_t C, void* stream) {
  return upsample2_bwd(cb(gy), mb(gx), B, H, W, C, cs(stream));
}
extern "C" int stn_upsample2_concat(const void* d, const void* e, void* y, int32_t B, int32_t H, int32_t W,
                                    int32_t Cd, int32_t Ce, void* stream) {
  return upsample2_concat(cb(d), cb(e), mb(y), B, H, W, Cd, Ce, cs(stream));
}
extern "C" int stn_concat(const void* a, const void* b, void* y, int64_t npix, int32_t Ca, int32_t Cb, void* stream) {
  return concat(cb(a), cb(b), mb(y), npix, Ca, Cb, cs(stream));
}
extern "C" int stn_split(const void* gy, void* ga, void* gb, int64_t npix, int32_t Ca, int32_t Cb, void* stream) {
  return split(cb(gy), mb(ga), mb(gb), npix, Ca, Cb, cs(stream));
}
extern "C" int stn_relu_mask(void* g, const void* y, int64_t n, void* stream) {
  return relu_mask(mb(g), cb(y), n, cs(stream));
}
extern "C" int64_t stn_bias_grad_workspace(int32_t C) { return (int64_t)bias_grad_workspace(C); }
extern "C" int stn_bias_grad(const void* g, float* gb, int64_t npix, int32_t C, float* ws, int64_t ws_floats,
                             void* stream) {
  if (ws_floats < 0) return 1;
  return bias_grad(cb(g), gb, npix, C, ws, (size_t)ws_floats, cs(stream));
}
extern "C" int stn_mse(const float* pred, const float* target, const float* target1, void* g, float* loss,
                       int64_t npix, int32_t Cp, float w1, void* stream) {
  return mse(pred, target, target1, mb(g), loss, npix, Cp, w1, cs(stream));
}
extern "C" int stn_adam(float* w, float* m, float* v, const float* g, void* w16, int64_t n, float lr, float beta1,
                        float beta2, float eps, int32_t step, float wd, void* stream) {
  return adam(w, m, v, g, mb(w16), n, lr, beta1, beta2, eps, step, wd, cs(stream));
}
extern "C" int stn_pack(const float* planes, int32_t nplanes, void* y, int64_t npix, int32_t C, void* stream) {
  return pack(planes, nplanes, mb(y), npix, C, cs(stream));
}
extern "C" int stn_to_bf16(const float* x, void* y, int64_t n, void* stream) {
  return to_bf16(x, mb(y), n, cs(stream));
}
extern "C" int stn_add(void* a, const void* b, int64_t n, void* stream) { return add(mb(a), cb(b), n, cs(stream)); }
extern "C" int stn_fill_zero(void* p, int64_t bytes, void* stream) {
  if (!p || bytes < 0) return 1;
  return cudaMemsetAsync(p, 0, (size_t)bytes, cs(stream)) == cudaSuccess ? 0 : 2;
}
extern "C" int stn_image_mean(const double* img, int64_t n, double* mean, void* stream) {
  return image_mean(img, n, mean, cs(stream));
}
extern "C" int stn_resample_planes(const double* img2, int32_t Mx2, int32_t My2, int32_t Mx8, int32_t My8,
                                   int32_t Wp, int32_t Hp, float sg_value, const double* mean, float contrast,
                                   float* planes, void* stream) {
  return resample_planes(img2, Mx2, My2, Mx8, My8, Wp, Hp, sg_value, mean, contrast, planes, cs(stream));
}
extern "C" int stn_apply_correction(const float* base, const float* pred, int32_t Cp, int32_t Mx8, int32_t My8,
                                    int32_t Wp, float scale, double* out, void* stream) {
  return apply_correction(base, pred, Cp, Mx8, My8, Wp, scale, out, cs(stream));
}
extern "C" int stn_tile_maxabs(const float* pred, int32_t Cp, int32_t ch, int32_t Mx8, int32_t My8, int32_t Wp,
                               int32_t T, float* tile_max, void* stream) {
  return tile_maxabs(pred, Cp, ch, Mx8, My8, Wp, T, tile_max, cs(stream));
}
extern "C" int stn_tile_flags(const float* tile_max, int32_t ntx, int32_t nty, float thresh, int32_t border,
                              uint8_t* mask, int32_t* count, void* stream) {
  return tile_flags(tile_max, ntx, nty, thresh, border, mask, count, cs(stream));
}
extern "C" int stn_merge_tiles(const double* fine, const uint8_t* mask, int32_t ntx, int32_t T, int32_t Mx,
                               int32_t My, double* out, void* stream) {
  return merge_tiles(fine, mask, ntx, T, Mx, My, out, cs(stream));
}
extern "C" int stn_last_kernel_error(void) { return take_error(); }
