// K4: the separable Gaussian blur of d2bi's PNG output (src/d2bi.f90:1543-1624).
//
// x pass:  f_x(ix,iy) = sum_{jj=max(0,ix-Nk)}^{min(Nx-1,ix+Nk)} k(|jj-ix|) f(jj,iy),
//          w_stripe(ix) = 1 / sum of the same weights;
// y pass:  out(ix,iy) = [sum_jj k(|jj-iy|) f_x(ix,jj)] * w_stripe(ix) / (sum of those weights).
// The weights k are computed on the host exactly as the reference does; the
// sums run in ascending jj with separately rounded operations, so the result
// equals the reference's double arithmetic.  The y pass reads columns with
// consecutive ix in consecutive threads (coalesced); one launch per pass, the
// intermediate image stays in L2 for the image sizes d2bi produces.
#include <cuda_runtime.h>

#include "internal.h"

namespace stem {
namespace {

__global__ void __launch_bounds__(256) k_blur_x(const double* __restrict__ in, double* __restrict__ tmp,
                                                double* __restrict__ wstripe, int nx, int ny,
                                                const double* __restrict__ kern, int nk) {
  const int64_t n = (int64_t)nx * ny;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)(i / nx);
    const int lo = max(0, ix - nk), hi = min(nx - 1, ix + nk);
    const double* row = in + (int64_t)nx * iy;
    double wf = 0.0, ws = 0.0;
    for (int jj = lo; jj <= hi; ++jj) {
      const double ww = kern[abs(jj - ix)];
      wf = __dadd_rn(wf, __dmul_rn(ww, row[jj]));
      ws = __dadd_rn(ws, ww);
    }
    tmp[i] = wf;
    if (iy == 0) wstripe[ix] = __ddiv_rn(1.0, ws);
  }
}

__global__ void __launch_bounds__(256) k_blur_y(const double* __restrict__ tmp, const double* __restrict__ wstripe,
                                                double* __restrict__ out, int nx, int ny,
                                                const double* __restrict__ kern, int nk) {
  const int64_t n = (int64_t)nx * ny;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)(i / nx);
    const int lo = max(0, iy - nk), hi = min(ny - 1, iy + nk);
    double wf = 0.0, ws = 0.0;
    for (int jj = lo; jj <= hi; ++jj) {
      const double ww = kern[abs(jj - iy)];
      wf = __dadd_rn(wf, __dmul_rn(ww, tmp[ix + (int64_t)nx * jj]));
      ws = __dadd_rn(ws, ww);
    }
    out[i] = __ddiv_rn(__dmul_rn(wf, wstripe[ix]), ws);
  }
}

}  // namespace

// d_tmp holds nx*ny + nx doubles (the x-pass image, then w_stripe).
cudaError_t launch_blur(const double* d_in, double* d_tmp, double* d_out, int nx, int ny, const double* d_kernel,
                        int nk, cudaStream_t st) {
  const int64_t n = (int64_t)nx * ny;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  double* wstripe = d_tmp + n;
  k_blur_x<<<blocks, 256, 0, st>>>(d_in, d_tmp, wstripe, nx, ny, d_kernel, nk);
  k_blur_y<<<blocks, 256, 0, st>>>(d_tmp, wstripe, d_out, nx, ny, d_kernel, nk);
  return cudaGetLastError();
}

}  // namespace stem
