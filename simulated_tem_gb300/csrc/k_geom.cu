// Per-condition geometry over the atoms on the GPU (the O(N) parts of d2bi's set-up):
//   * wrapPBC0 (src/Lib_SimpleSupercells.f90:992-1023, applied on read at src/d2bi.f90:856-866):
//     the cell coordinates ia x, their integer parts taken modulo the supercell, back to
//     real space a xx;
//   * the atom extents behind findImageParameters' image space (src/d2bi.f90:983-991):
//     max - min of each component of U x, U the rotation to the standard frame of (k, g),
//     for several conditions in one pass over the atoms.
// Every product and sum is rounded separately in the host mirror's order
// (host_d2bi.cpp: apply(), st_wrap_pbc, st_atom_extents), so both give the same bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace stem {
namespace {

// y_i = (m(i,1) v0 + m(i,2) v1) + m(i,3) v2, m column-major
__device__ __forceinline__ double row(const double* m, int i, double v0, double v1, double v2) {
  return __dadd_rn(__dadd_rn(__dmul_rn(m[i], v0), __dmul_rn(m[i + 3], v1)), __dmul_rn(m[i + 6], v2));
}

__global__ void k_wrap_pbc(GeomWrap w, double* __restrict__ x, int64_t ldx, int64_t n) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    double* y = x + j * ldx;
    const double y0 = y[0], y1 = y[1], y2 = y[2];
    double xx[3];
    for (int d = 0; d < 3; ++d) {
      double c = row(w.ia, d, y0, y1, y2);
      int ii = (int)floor(c);
      c = __dsub_rn(c, (double)ii);
      ii = (ii + (w.N[d] << 8)) % w.N[d];
      xx[d] = __dadd_rn((double)ii, c);
    }
    y[0] = row(w.a, 0, xx[0], xx[1], xx[2]);
    y[1] = row(w.a, 1, xx[0], xx[1], xx[2]);
    y[2] = row(w.a, 2, xx[0], xx[1], xx[2]);
  }
}

// part[block][r][0..5] = min x, y, z, max x, y, z of U_r x over the block's atoms
__global__ void __launch_bounds__(256) k_extents_part(GeomRot rot, const double* __restrict__ x, int64_t ldx,
                                                      int64_t n, double* __restrict__ part) {
  __shared__ double red[8][6];
  for (int r = 0; r < rot.n; ++r) {
    const double* U = rot.U + 9 * r;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
      const double* p = x + j * ldx;
      const double v0 = p[0], v1 = p[1], v2 = p[2];
      for (int i = 0; i < 3; ++i) {
        const double yi = row(U, i, v0, v1, v2);
        lo[i] = fmin(lo[i], yi);
        hi[i] = fmax(hi[i], yi);
      }
    }
    for (int i = 0; i < 3; ++i)
      for (int o = 16; o > 0; o >>= 1) {
        lo[i] = fmin(lo[i], __shfl_xor_sync(0xffffffffu, lo[i], o));
        hi[i] = fmax(hi[i], __shfl_xor_sync(0xffffffffu, hi[i], o));
      }
    if ((threadIdx.x & 31) == 0)
      for (int i = 0; i < 3; ++i) {
        red[threadIdx.x >> 5][i] = lo[i];
        red[threadIdx.x >> 5][3 + i] = hi[i];
      }
    __syncthreads();
    if (threadIdx.x < 6) {
      double v = red[0][threadIdx.x];
      for (int w = 1; w < 8; ++w) v = threadIdx.x < 3 ? fmin(v, red[w][threadIdx.x]) : fmax(v, red[w][threadIdx.x]);
      part[((int64_t)blockIdx.x * rot.n + r) * 6 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

__global__ void k_extents_final(const double* __restrict__ part, int nblocks, int nrot, double* __restrict__ out) {
  const int t = threadIdx.x;  // (r, k) pairs
  if (t >= 6 * nrot) return;
  const int r = t / 6, k = t % 6;
  double v = part[r * 6 + k];
  for (int b = 1; b < nblocks; ++b) {
    const double u = part[((int64_t)b * nrot + r) * 6 + k];
    v = k < 3 ? fmin(v, u) : fmax(v, u);
  }
  out[t] = v;
}

int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : g > kExtentBlocks ? kExtentBlocks : g);
}

}  // namespace

cudaError_t launch_wrap_pbc(const GeomWrap& w, double* d_x, int64_t ldx, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_wrap_pbc<<<grid_for(n), 256, 0, st>>>(w, d_x, ldx, n);
  return cudaGetLastError();
}

cudaError_t launch_extents(const GeomRot& rot, const double* d_x, int64_t ldx, int64_t n, double* d_part,
                           double* d_out, cudaStream_t st) {
  const int nb = grid_for(n);
  k_extents_part<<<nb, 256, 0, st>>>(rot, d_x, ldx, n, d_part);
  k_extents_final<<<1, 6 * kMaxRot, 0, st>>>(d_part, nb, rot.n, d_out);
  return cudaGetLastError();
}

}  // namespace stem
