// st_blur_noalloc: the PNG blur of d2bi without any allocation by the library.
//
// Some callers cannot let a library allocate GPU memory: a Fortran host that
// runs under an MPI or batch runtime owning the device memory pool, code that
// images inside a fixed memory budget, or a caller that must not allocate
// between steps it later replays.  This variant keeps the one intermediate it
// needs -- the x-pass image and the per-column weights w_stripe -- in a
// file-scope __device__ array of fixed size instead of memory from
// cudaMalloc.  Every GPU that loads the library holds that array until the
// process exits.
//
// Arithmetic is that of st_blur / gaussianBlurImage (src/d2bi.f90:1543-1624):
// the weights are computed on the host exactly as st_blur computes them and
// passed by value to the kernels, and the sums run in the same order, so the
// output is identical to st_blur's.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/stem.h"

namespace {

constexpr int kMaxContexts = 64;
constexpr int64_t kScratchDoubles = (int64_t)ST_BLUR_NOALLOC_MAX_PIXELS + ST_BLUR_NOALLOC_MAX_NX;

// The scratch: x-pass image (nx * ny doubles) followed by w_stripe (nx doubles).
static __device__ __align__(256) double g_blur_scratch[kScratchDoubles];

// Device addresses of g_blur_scratch, looked up once per CUDA context (the module, and so
// the array, is loaded per context).  In host code the name g_blur_scratch is only a
// host-side stand-in for the device array, so the kernels receive the looked-up address.
// The cache is keyed on the context's unique ID (cuCtxGetId), not on the device ordinal or
// the context handle: after a device reset, or under another context of the same device,
// the first call looks the address up again.
struct ScratchAddr {
  unsigned long long ctx_id;
  double* addr;
};
ScratchAddr g_scratch_addr[kMaxContexts] = {};
int g_scratch_next = 0;
std::mutex g_setup_mutex;
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// The unique ID of the calling thread's current context (driver entry points fetched through
// the runtime, so the library does not link the driver library itself); 0 on failure.
unsigned long long current_context_id() {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess)
      return 0;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

struct BlurWeights {
  int nk;
  double k[ST_BLUR_NOALLOC_MAX_NK + 1];
};

__global__ void __launch_bounds__(256) k_blur_x_fixed(const double* __restrict__ in, double* __restrict__ tmp,
                                                      int nx, int ny, const __grid_constant__ BlurWeights w) {
  const int64_t n = (int64_t)nx * ny;
  double* wstripe = tmp + n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)(i / nx);
    const int lo = max(0, ix - w.nk), hi = min(nx - 1, ix + w.nk);
    const double* row = in + (int64_t)nx * iy;
    double wf = 0.0, ws = 0.0;
    for (int jj = lo; jj <= hi; ++jj) {
      const double ww = w.k[abs(jj - ix)];
      wf = __dadd_rn(wf, __dmul_rn(ww, row[jj]));
      ws = __dadd_rn(ws, ww);
    }
    tmp[i] = wf;
    if (iy == 0) wstripe[ix] = __ddiv_rn(1.0, ws);
  }
}

__global__ void __launch_bounds__(256) k_blur_y_fixed(const double* __restrict__ tmp, double* __restrict__ out,
                                                      int nx, int ny, const __grid_constant__ BlurWeights w) {
  const int64_t n = (int64_t)nx * ny;
  const double* wstripe = tmp + n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)(i / nx);
    const int lo = max(0, iy - w.nk), hi = min(ny - 1, iy + w.nk);
    double wf = 0.0, ws = 0.0;
    for (int jj = lo; jj <= hi; ++jj) {
      const double ww = w.k[abs(jj - iy)];
      wf = __dadd_rn(wf, __dmul_rn(ww, tmp[ix + (int64_t)nx * jj]));
      ws = __dadd_rn(ws, ww);
    }
    out[i] = __ddiv_rn(__dmul_rn(wf, wstripe[ix]), ws);
  }
}

int report(char* err, int32_t err_len, int code, const char* msg) {
  if (err && err_len > 0) {
    std::strncpy(err, msg, (size_t)err_len - 1);
    err[err_len - 1] = '\0';
  }
  return code;
}

}  // namespace

extern "C" int st_blur_noalloc(const double* d_in, int32_t nx, int32_t ny, double t, double* d_out, void* stream,
                               char* err, int32_t err_len) {
  if (err && err_len > 0) err[0] = '\0';
  if (!d_in || !d_out || nx < 1 || ny < 1) return report(err, err_len, ST_ERR_ARG, "st_blur_noalloc: invalid image");
  if (nx > ST_BLUR_NOALLOC_MAX_NX || (int64_t)nx * ny > ST_BLUR_NOALLOC_MAX_PIXELS) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "st_blur_noalloc: %d x %d pixels exceeds the fixed scratch (at most %d pixels, "
                  "nx <= %d)", nx, ny, ST_BLUR_NOALLOC_MAX_PIXELS, ST_BLUR_NOALLOC_MAX_NX);
    return report(err, err_len, ST_ERR_ARG, buf);
  }
  if (!(t > 0.0)) return report(err, err_len, ST_ERR_ARG, "st_blur_noalloc: blur width t must be > 0 pixels");
  // kernel(0:Nk): Nk = max(5, ceiling(5 t)), exp(-k^2 / (2 t^2)), as st_blur computes it
  const double nkd = std::ceil(t * 5);
  if (!(nkd <= ST_BLUR_NOALLOC_MAX_NK))
    return report(err, err_len, ST_ERR_ARG, "st_blur_noalloc: blur width t exceeds the fixed weight table");
  BlurWeights w;
  w.nk = nkd < 5 ? 5 : (int)nkd;
  const double i2s2 = 1 / (2 * t * t);
  w.k[0] = 1.0;
  for (int i = 1; i <= w.nk; ++i) w.k[i] = std::exp(-(i * i * i2s2));

  cudaError_t e = cudaSuccess;
  double* scratch = nullptr;
  {
    // once per context, with it current: the device address of the scratch array (a thread
    // without a current context gets the device's primary context from this first lookup)
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = current_context_id();
    for (const ScratchAddr& a : g_scratch_addr)
      if (id != 0 && a.ctx_id == id) scratch = a.addr;
    if (!scratch) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_blur_scratch);
      if (e != cudaSuccess) return report(err, err_len, ST_ERR_CUDA, cudaGetErrorString(e));
      scratch = static_cast<double*>(p);
      if (id == 0) id = current_context_id();
      if (id == 0) return report(err, err_len, ST_ERR_CUDA, "st_blur_noalloc: no current CUDA context");
      g_scratch_addr[g_scratch_next] = ScratchAddr{id, scratch};
      g_scratch_next = (g_scratch_next + 1) % kMaxContexts;
    }
  }
  const int64_t n = (int64_t)nx * ny;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  cudaStream_t st = (cudaStream_t)stream;
  // every pixel of the x-pass image and every w_stripe entry is written before it is read
  k_blur_x_fixed<<<blocks, 256, 0, st>>>(d_in, scratch, nx, ny, w);
  k_blur_y_fixed<<<blocks, 256, 0, st>>>(scratch, d_out, nx, ny, w);
  e = cudaGetLastError();
  if (e != cudaSuccess) return report(err, err_len, ST_ERR_CUDA, cudaGetErrorString(e));
  return ST_OK;
}
