// FP64 arithmetic of the column integrator shared by the FP64 column kernels: the
// reference's operations in its order, each explicitly rounded (no contraction), for
// the samples x(z) and rho(z) (Lib_DynamicalTwoBeamImaging.f90:1877-1895, 1973-1994)
// and the RK4 double step of dynamicalTwoBeamIntegrationColumn_phaserho (:2316-2480).
#pragma once
#include <cuda_runtime.h>

namespace stem {
namespace fp64col {

#define DM __dmul_rn
#define DA __dadd_rn
#define DS __dsub_rn

struct Sample64 {
  double c0, ca_base, cgr, cgi;  // c0 = b0 rho; ca = b0 rho + a
};

__device__ __forceinline__ void deriv64(const Sample64& s, double a, const double* ph, double* d) {
  const double ca = DA(s.ca_base, a);
  // dphi0r = - c0*phi0i - cgi*phigr - cgr*phigi  (and so on, :2393-2396)
  d[0] = DS(DS(-DM(s.c0, ph[1]), DM(s.cgi, ph[2])), DM(s.cgr, ph[3]));
  d[1] = DS(DA(DM(s.c0, ph[0]), DM(s.cgr, ph[2])), DM(s.cgi, ph[3]));
  d[2] = DS(DS(DM(s.cgi, ph[0]), DM(s.cgr, ph[1])), DM(ca, ph[3]));
  d[3] = DA(DA(DM(s.cgr, ph[0]), DM(s.cgi, ph[1])), DM(ca, ph[2]));
}

__device__ __forceinline__ void rk4_64(const Sample64& s0, const Sample64& s1, const Sample64& s2, double a,
                                       double dz, double* ph) {
  double d[4], p1[4], p2[4], q[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) p2[i] = ph[i];
  deriv64(s0, a, ph, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    p1[i] = DA(ph[i], __ddiv_rn(DM(d[i], dz), 3.0));  // phi + dphi*dz/3
    q[i] = DA(ph[i], DM(d[i], dz));
  }
  deriv64(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = DA(p2[i], DM(d[i], dz));
    p1[i] = DA(p1[i], __ddiv_rn(DM(DM(d[i], 2.0), dz), 3.0));  // + dphi*2*dz/3
  }
  deriv64(s1, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = DA(p2[i], DM(DM(d[i], 2.0), dz));  // + dphi*2*dz
    p1[i] = DA(p1[i], __ddiv_rn(DM(DM(d[i], 2.0), dz), 3.0));
  }
  deriv64(s2, a, q, d);
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = DA(p1[i], __ddiv_rn(DM(d[i], dz), 3.0));
  double mag = DA(DA(DA(DM(ph[0], ph[0]), DM(ph[1], ph[1])), DM(ph[2], ph[2])), DM(ph[3], ph[3]));
  mag = __ddiv_rn(1.0, __dsqrt_rn(mag));
#pragma unroll
  for (int i = 0; i < 4; ++i) ph[i] = DM(ph[i], mag);
}

__device__ __forceinline__ double rho64(double r2min, double sig) {
  if (r2min < DM(sig, sig)) return 1.0;
  if (r2min > DM(DM(4.0, sig), sig)) return 0.0;
  const double xx = DS(__ddiv_rn(__dsqrt_rn(r2min), sig), 1.0);
  // 1 - xx*xx*xx*(10 - 15*xx + 6*xx*xx)
  const double poly = DA(DS(10.0, DM(15.0, xx)), DM(DM(6.0, xx), xx));
  return DS(1.0, DM(DM(DM(xx, xx), xx), poly));
}


}  // namespace fp64col
}  // namespace stem
