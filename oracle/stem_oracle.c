/*
 * ORACLE -- test infrastructure only (see stem_oracle.h).
 *
 * Plain-C restatement of simulated_tem's imaging hot path.  Every function
 * names the reference lines it follows.  Compiled with -O2 -ffp-contract=off so
 * that the left-to-right double arithmetic of the reference is kept.
 */
#include "stem_oracle.h"

#include <float.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* PI of Lib_DynamicalTwoBeamImaging.f90:55 and Lib_DiffractionConditions.f90:21. */
static const double PI = 3.141592653589790;
/* Lib_RelativisticElectrons.f90:9-14. */
static const double ME = 0.056856301036;
static const double EC = 1.0;
static const double CL = 2997.92458;
static const double HP = 4.135667696;
#define HBAR (HP / (2 * 3.14159265390))
/* huge(1.0): the default-kind (single precision) largest value. */
static const double HUGE1 = (double)FLT_MAX;

#define A(m, i, j) ((m)[((i)-1) + 3 * ((j)-1)])

/* ------------------------------------------------------------------------ */
/* small linear algebra                                                     */
/* ------------------------------------------------------------------------ */

/* gfortran's NORM2: scaled sum of squares. */
double oc_norm2(const double* v) {
  double scale = 0.0, res = 1.0;
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0.0) {
      double ax = fabs(v[i]);
      if (scale < ax) {
        double val = scale / ax;
        res = 1.0 + res * val * val;
        scale = ax;
      } else {
        double val = ax / scale;
        res += val * val;
      }
    }
  }
  return sqrt(res) * scale;
}

/* determinant3Mat (Lib_SimpleSupercells.f90:1240-1256). */
double oc_det3(const double* M) {
  double dd[9];
  dd[0] = A(M, 1, 1) * (A(M, 2, 2) * A(M, 3, 3) - A(M, 2, 3) * A(M, 3, 2));
  dd[1] = A(M, 1, 2) * (A(M, 2, 3) * A(M, 3, 1) - A(M, 2, 1) * A(M, 3, 3));
  dd[2] = A(M, 1, 3) * (A(M, 2, 1) * A(M, 3, 2) - A(M, 2, 2) * A(M, 3, 1));
  dd[3] = A(M, 2, 1) * (A(M, 3, 2) * A(M, 1, 3) - A(M, 3, 3) * A(M, 1, 2));
  dd[4] = A(M, 2, 2) * (A(M, 3, 3) * A(M, 1, 1) - A(M, 3, 1) * A(M, 1, 3));
  dd[5] = A(M, 2, 3) * (A(M, 3, 1) * A(M, 1, 2) - A(M, 3, 2) * A(M, 1, 1));
  dd[6] = A(M, 3, 1) * (A(M, 1, 2) * A(M, 2, 3) - A(M, 1, 3) * A(M, 2, 2));
  dd[7] = A(M, 3, 2) * (A(M, 1, 3) * A(M, 2, 1) - A(M, 1, 1) * A(M, 2, 3));
  dd[8] = A(M, 3, 3) * (A(M, 1, 1) * A(M, 2, 2) - A(M, 1, 2) * A(M, 2, 1));
  double s = 0.0;
  for (int i = 0; i < 9; ++i) s += dd[i];
  return (1.0 / 3.0) * s;
}

/* inverse3Mat (Lib_SimpleSupercells.f90:1205-1236). */
void oc_inv3(const double* M, double* N) {
  double idd = oc_det3(M);
  if (fabs(idd) < DBL_MIN) {
    memset(N, 0, 9 * sizeof(double));
    N[0] = N[4] = N[8] = 1.0;
    return;
  }
  idd = 1.0 / idd;
  A(N, 1, 1) = (A(M, 2, 2) * A(M, 3, 3) - A(M, 2, 3) * A(M, 3, 2)) * idd;
  A(N, 2, 1) = (A(M, 2, 3) * A(M, 3, 1) - A(M, 2, 1) * A(M, 3, 3)) * idd;
  A(N, 3, 1) = (A(M, 2, 1) * A(M, 3, 2) - A(M, 2, 2) * A(M, 3, 1)) * idd;
  A(N, 1, 2) = (A(M, 1, 3) * A(M, 3, 2) - A(M, 1, 2) * A(M, 3, 3)) * idd;
  A(N, 2, 2) = (A(M, 1, 1) * A(M, 3, 3) - A(M, 1, 3) * A(M, 3, 1)) * idd;
  A(N, 3, 2) = (A(M, 1, 2) * A(M, 3, 1) - A(M, 1, 1) * A(M, 3, 2)) * idd;
  A(N, 1, 3) = (A(M, 1, 2) * A(M, 2, 3) - A(M, 1, 3) * A(M, 2, 2)) * idd;
  A(N, 2, 3) = (A(M, 1, 3) * A(M, 2, 1) - A(M, 1, 1) * A(M, 2, 3)) * idd;
  A(N, 3, 3) = (A(M, 1, 1) * A(M, 2, 2) - A(M, 1, 2) * A(M, 2, 1)) * idd;
}

/* matmul of two 3x3 matrices, k ascending. */
static void mat_mul(const double* a, const double* b, double* c) {
  double t[9];
  for (int j = 1; j <= 3; ++j)
    for (int i = 1; i <= 3; ++i) {
      double s = 0.0;
      for (int k = 1; k <= 3; ++k) s += A(a, i, k) * A(b, k, j);
      A(t, i, j) = s;
    }
  memcpy(c, t, sizeof t);
}

static void transpose3(const double* a, double* t) {
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j) A(t, i, j) = A(a, j, i);
}

/* y(1:3) = m(1:3,1)*v(1) + m(1:3,2)*v(2) + m(1:3,3)*v(3) */
static void mat_vec(const double* m, const double* v, double* y) {
  double t[3];
  for (int i = 1; i <= 3; ++i) t[i - 1] = A(m, i, 1) * v[0] + A(m, i, 2) * v[1] + A(m, i, 3) * v[2];
  y[0] = t[0];
  y[1] = t[1];
  y[2] = t[2];
}

static void identity3(double* m) {
  memset(m, 0, 9 * sizeof(double));
  m[0] = m[4] = m[8] = 1.0;
}

static int imod(int a, int n) { /* Fortran mod: sign of a */
  return a % n;
}

/* ------------------------------------------------------------------------ */
/* SimpleSupercell                                                          */
/* ------------------------------------------------------------------------ */

/* SimpleSupercell_ctor0 (Lib_SimpleSupercells.f90:183-196). */
void oc_super_ctor(oc_super* s, const double* a, int Nx, int Ny, int Nz) {
  memcpy(s->a, a, 9 * sizeof(double));
  s->Nx = Nx;
  s->Ny = Ny;
  s->Nz = Nz;
  oc_inv3(s->a, s->ia);
}

/* cellToRealSpace2 (Lib_SimpleSupercells.f90:338-345). */
static void cell_to_real_i(const oc_super* s, int ix, int iy, int iz, double* y) {
  for (int i = 1; i <= 3; ++i)
    y[i - 1] = A(s->a, i, 1) * (double)ix + A(s->a, i, 2) * (double)iy + A(s->a, i, 3) * (double)iz;
}

/* realSpaceToCell0 (Lib_SimpleSupercells.f90:348-356). */
static void real_to_cell(const oc_super* s, const double* y, double* x) { mat_vec(s->ia, y, x); }

/* pointInSupercell0 (Lib_SimpleSupercells.f90:1063-1102). */
static int point_in_super(const oc_super* s, const double* x) {
  int ix = (int)floor(A(s->ia, 1, 1) * x[0] + A(s->ia, 1, 2) * x[1] + A(s->ia, 1, 3) * x[2]);
  int is = (ix == imod(ix + (s->Nx << 8), s->Nx));
  int iy = (int)floor(A(s->ia, 2, 1) * x[0] + A(s->ia, 2, 2) * x[1] + A(s->ia, 2, 3) * x[2]);
  is = is && (iy == imod(iy + (s->Ny << 8), s->Ny));
  int iz = (int)floor(A(s->ia, 3, 1) * x[0] + A(s->ia, 3, 2) * x[1] + A(s->ia, 3, 3) * x[2]);
  is = is && (iz == imod(iz + (s->Nz << 8), s->Nz));
  return is;
}

/* wrapPBC0 (Lib_SimpleSupercells.f90:992-1023). */
void oc_wrap_pbc(const oc_super* s, const double* y, double* yp) {
  double xx[3];
  real_to_cell(s, y, xx);
  int N[3] = {s->Nx, s->Ny, s->Nz};
  for (int d = 0; d < 3; ++d) {
    int ii = (int)floor(xx[d]);
    xx[d] = xx[d] - ii;
    ii = imod(ii + (N[d] << 8), N[d]);
    xx[d] = (ii + xx[d]);
  }
  mat_vec(s->a, xx, yp);
}

static double cell_side_length(const oc_super* s, int i) { return oc_norm2(&s->a[3 * (i - 1)]); }

/* getSuperCellSideLength0 (Lib_SimpleSupercells.f90:862-876). */
static double super_side_length(const oc_super* s, int i) {
  int N = (i == 1) ? s->Nx : (i == 2) ? s->Ny : s->Nz;
  return oc_norm2(&s->a[3 * (i - 1)]) * N;
}

/* getSuperA (Lib_SimpleSupercells.f90:851-860). */
static void super_a(const oc_super* s, double* a) {
  for (int i = 0; i < 3; ++i) {
    a[i] = s->a[i] * s->Nx;
    a[3 + i] = s->a[3 + i] * s->Ny;
    a[6 + i] = s->a[6 + i] * s->Nz;
  }
}

/* ------------------------------------------------------------------------ */
/* Lib_RelativisticElectrons / Lib_DiffractionConditions                    */
/* ------------------------------------------------------------------------ */

/* wavelength (Lib_RelativisticElectrons.f90:25-38). */
double oc_wavelength(double V) {
  if (V <= 0) return 0.0;
  double lambda = 2 * ME * EC * V * (1 + EC * V / (2 * ME * CL * CL));
  return HP / sqrt(lambda);
}

/* velocity (Lib_RelativisticElectrons.f90:40-50). */
double oc_velocity(double V) {
  double u = 1 + EC * V / (ME * CL * CL);
  return CL * sqrt(1 - 1 / (u * u));
}

/* getReciprocalLatticeVectors (Lib_DiffractionConditions.f90:1630-1640). */
static void reciprocal(const double* A_cell, double* B) {
  double t[9];
  transpose3(A_cell, t);
  oc_inv3(t, B);
  for (int i = 0; i < 9; ++i) B[i] = 2 * PI * B[i];
}

/* reflection1 (Lib_DiffractionConditions.f90:1656-1667). */
static void reflection(const double* B, const double* hkl, double* g) {
  double t[3];
  for (int i = 1; i <= 3; ++i) t[i - 1] = A(B, i, 1) * hkl[0] + A(B, i, 2) * hkl[1] + A(B, i, 3) * hkl[2];
  memcpy(g, t, sizeof t);
}

/* energyToLengthDeviationParameter (Lib_DiffractionConditions.f90:1194-1204). */
static double energy_to_length_sg(double v, double eps) { return -eps / (2 * PI * HBAR * v); }

/* energy_deviation_parameter (Lib_DiffractionConditions.f90:1265-1299). */
static double energy_deviation_parameter(double v, const double* khat, const double* g) {
  const double HBAR2ON2M = HBAR * HBAR / (2 * ME);
  double cst = 2 * ME * v / HBAR;
  double eps = khat[0] * g[0] + khat[1] * g[1] + khat[2] * g[2];
  eps = cst * eps;
  eps = eps + g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  return eps * HBAR2ON2M;
}

/* intensityAtDepthZ (Lib_DiffractionConditions.f90:1209-1259). */
double oc_intensity_at_depth(double xi0, double xig, double sg, double z) {
  double b0 = PI / xi0, bg = PI / xig, aa = 2 * PI * sg;
  double dd = sqrt(aa * aa / 4 + bg * bg);
  double l1 = (b0 + aa / 2) + dd, l2 = (b0 + aa / 2) - dd;
  double re = cos(l1 * z) - cos(l2 * z), im = sin(l1 * z) - sin(l2 * z);
  double s = bg / (2 * dd);
  re *= s;
  im *= s;
  return re * re + im * im;
}

static void cross3(const double* x, const double* y, double* z) {
  z[0] = x[1] * y[2] - x[2] * y[1];
  z[1] = x[2] * y[0] - x[0] * y[2];
  z[2] = x[0] * y[1] - x[1] * y[0];
}

/* rotateToStandardFrame0 (Lib_DiffractionConditions.f90:65-108). */
void oc_rotate_to_standard_frame(const double* z0, const double* A_cell, const double* hkl, double* U) {
  double BB[9], gg[3], zz[3], xx[3], yy[3];
  reciprocal(A_cell, BB);
  reflection(BB, hkl, gg);
  for (int i = 1; i <= 3; ++i) {
    double s = 0.0;
    for (int k = 1; k <= 3; ++k) s += A(A_cell, i, k) * z0[k - 1];
    zz[i - 1] = s;
  }
  double nz = oc_norm2(zz);
  for (int i = 0; i < 3; ++i) zz[i] = zz[i] / nz;
  double gz = 0.0;
  for (int i = 0; i < 3; ++i) gz += gg[i] * zz[i];
  for (int i = 0; i < 3; ++i) xx[i] = gg[i] - gz * zz[i];
  double nx = oc_norm2(xx);
  for (int i = 0; i < 3; ++i) xx[i] = xx[i] / nx;
  cross3(zz, xx, yy);
  for (int j = 1; j <= 3; ++j) {
    A(U, 1, j) = xx[j - 1];
    A(U, 2, j) = yy[j - 1];
    A(U, 3, j) = zz[j - 1];
  }
}

/* findTransformedSupercell (Lib_DiffractionConditions.f90:996-1189): the
 * cuboid D, the offset delta and the 27 periodic replicas. */
static void find_transformed_supercell(const double* A_super, const double* R, double* D_super, double* delta,
                                       int* uvw, int* nuvw, const double* foil) {
  double dd[3] = {foil[0], foil[1], foil[2]}, xx[3];
  memset(D_super, 0, 9 * sizeof(double));
  A(D_super, 1, 1) = dd[0];
  A(D_super, 2, 2) = dd[1];
  A(D_super, 3, 3) = dd[2];
  xx[0] = xx[1] = xx[2] = 0.5;
  mat_vec(A_super, xx, xx);
  mat_vec(R, xx, xx);
  for (int i = 0; i < 3; ++i) delta[i] = dd[i] / 2 - xx[i];
  int n = 0;
  for (int iz = -1; iz <= 1; ++iz)
    for (int iy = -1; iy <= 1; ++iy)
      for (int ix = -1; ix <= 1; ++ix) {
        uvw[3 * n + 0] = ix;
        uvw[3 * n + 1] = iy;
        uvw[3 * n + 2] = iz;
        ++n;
      }
  *nuvw = n;
}

/* ------------------------------------------------------------------------ */
/* DynamicalTwoBeamImaging                                                  */
/* ------------------------------------------------------------------------ */

/* DynamicalTwoBeamImaging_ctor0 / _null (Lib_DynamicalTwoBeamImaging.f90:125-178). */
void oc_d2bi_ctor(oc_d2bi* t, const oc_super* super, double a0, const double* k, const double* g, double E,
                  int mxy, int mzz) {
  memset(t, 0, sizeof *t);
  t->super = *super;
  double id[9];
  identity3(id);
  oc_super_ctor(&t->gksuper, id, 1, 1, 1);
  t->a0 = a0;
  t->xi0 = 103.9;
  t->xig = 207.5;
  t->useDensityField = 1;
  memcpy(t->a_cell, id, sizeof id); /* set while a0 = 1 (:131) */
  t->sg = NAN;
  t->nuvw = 1;
  identity3(t->R);
  identity3(t->U);
  t->test = 0;
  memcpy(t->k, k, 3 * sizeof(double));
  memcpy(t->g, g, 3 * sizeof(double));
  t->E = E;
  t->mxy = mxy;
  t->mzz = mzz;
}

void oc_set_conventional_unit_cell(oc_d2bi* t, const double* a_cell) { memcpy(t->a_cell, a_cell, 9 * sizeof(double)); }

/* setVoxelSupercellSize2 (Lib_DynamicalTwoBeamImaging.f90:349-430) for
 * cuboidSides with all three entries nonzero (the d2bi path). */
int oc_set_voxel_supercell_size(oc_d2bi* t, const double* cs) {
  double hkl[3] = {(double)lround(t->g[0]), (double)lround(t->g[1]), (double)lround(t->g[2])};
  oc_rotate_to_standard_frame(t->k, t->a_cell, hkl, t->U);
  if (cs[0] == 0 || cs[1] == 0 || cs[2] == 0) return OC_ERR_ARG;
  memcpy(t->voxelSupercellDimensions, cs, 3 * sizeof(double));
  return OC_OK;
}

void oc_set_deviation_parameter(oc_d2bi* t, double sg) { t->sg = sg; }
void oc_set_extinction_distances(oc_d2bi* t, double xi0, double xig) {
  t->xi0 = xi0;
  t->xig = xig;
}
void oc_set_use_density_field(oc_d2bi* t, int is) { t->useDensityField = is; }

/* getAperture (Lib_DynamicalTwoBeamImaging.f90:1137-1155). */
void oc_get_aperture(const oc_d2bi* t, const double* beamTilt, double* g) {
  double b[9], RU[9];
  reciprocal(t->a_cell, b);
  reflection(b, t->g, g);
  mat_mul(t->R, t->U, RU);
  if (beamTilt) mat_mul(beamTilt, RU, RU);
  mat_vec(RU, g, g);
}

/* getDeviationParameter (Lib_DynamicalTwoBeamImaging.f90:292-307). */
double oc_get_deviation_parameter(const oc_d2bi* t, const double* g) {
  if (!g) return t->sg;
  double modk = 2 * PI / oc_wavelength(t->E * 1000);
  double vv = HBAR * modk / ME;
  const double khat[3] = {0.0, 0.0, 1.0};
  double eps = energy_deviation_parameter(vv, khat, g);
  return energy_to_length_sg(vv, eps);
}

/* gksuper from D_super (Lib_DynamicalTwoBeamImaging.f90:775-784, 1086-1096). */
static void build_gksuper(oc_d2bi* t, double* D) {
  int Nx = t->mxy, Ny = t->mxy, Nz = t->mzz;
  int nx = (int)lround(t->mxy * A(D, 1, 1) / t->a0);
  int ny = (int)lround(t->mxy * A(D, 2, 2) / t->a0);
  int nz = (int)lround(t->mzz * A(D, 3, 3) / t->a0);
  if (nx > Nx) Nx = nx;
  if (ny > Ny) Ny = ny;
  if (nz > Nz) Nz = nz;
  A(D, 1, 1) = A(D, 1, 1) / Nx;
  A(D, 2, 2) = A(D, 2, 2) / Ny;
  A(D, 3, 3) = A(D, 3, 3) / Nz;
  oc_super_ctor(&t->gksuper, D, Nx, Ny, Nz);
}

static void tilt_about_y(double theta, double* R) {
  double c = cos(theta), s = sin(theta);
  /* reshape((/cos,0,-sin, 0,1,0, sin,0,cos/),(/3,3/)) */
  R[0] = c;
  R[1] = 0.0;
  R[2] = -s;
  R[3] = 0.0;
  R[4] = 1.0;
  R[5] = 0.0;
  R[6] = s;
  R[7] = 0.0;
  R[8] = c;
}

/* setSupercellTilt0 (Lib_DynamicalTwoBeamImaging.f90:567-792). */
void oc_set_supercell_tilt0(oc_d2bi* t) {
  double hkl[3] = {(double)lround(t->g[0]), (double)lround(t->g[1]), (double)lround(t->g[2])};
  oc_rotate_to_standard_frame(t->k, t->a_cell, hkl, t->U);
  double a_cell0[9], b_cell[9], gg[3], a_cell[9];
  mat_mul(t->U, t->a_cell, a_cell0);
  reciprocal(a_cell0, b_cell);
  reflection(b_cell, t->g, gg);
  double modg = oc_norm2(gg);
  double modk = 2 * PI / oc_wavelength(t->E * 1000);
  double vv = HBAR * modk / ME;
  const double khat[3] = {0.0, 0.0, 1.0};
  double eps = energy_deviation_parameter(vv, khat, gg);
  if (isnan(t->sg)) {
    t->sg = energy_to_length_sg(vv, eps);
    identity3(t->R);
  } else {
    double aa = 2 * PI * t->sg + HBAR * modg * modg / (2 * ME * vv);
    double cc = gg[0] * gg[0] + gg[2] * gg[2];
    double bb = cc - aa * aa;
    if (bb < 0) {
      t->sg = energy_to_length_sg(vv, eps);
      identity3(t->R);
    } else {
      bb = sqrt(bb);
      cc = 1 / cc;
      double th[4], sgs[4];
      th[0] = acos(-(gg[2] * aa + gg[0] * bb) * cc);
      th[1] = acos(-(gg[2] * aa - gg[0] * bb) * cc);
      th[2] = -th[0];
      th[3] = -th[1];
      for (int i = 0; i < 4; ++i) {
        double g2[3];
        tilt_about_y(th[i], t->R);
        mat_mul(t->R, a_cell0, a_cell);
        reciprocal(a_cell, b_cell);
        reflection(b_cell, t->g, g2);
        sgs[i] = energy_to_length_sg(vv, energy_deviation_parameter(vv, khat, g2));
      }
      for (int i = 0; i < 4; ++i)
        if (fabs(th[i]) * 2 > PI) sgs[i] = HUGE1;
      /* minloc of |sg - sg_i|: first minimum wins */
      int best = 0;
      double bestv = fabs(t->sg - sgs[0]);
      for (int i = 1; i < 4; ++i) {
        double v = fabs(t->sg - sgs[i]);
        if (v < bestv) {
          bestv = v;
          best = i;
        }
      }
      tilt_about_y(th[best], t->R);
    }
    mat_mul(t->R, a_cell0, a_cell);
    reciprocal(a_cell, b_cell);
    reflection(b_cell, t->g, gg);
    eps = energy_deviation_parameter(vv, khat, gg);
    t->sg = energy_to_length_sg(vv, eps);
  }
  double RU[9], a_sup[9], D[9];
  mat_mul(t->R, t->U, RU);
  super_a(&t->super, a_sup);
  find_transformed_supercell(a_sup, RU, D, t->delta, t->uvw, &t->nuvw, t->voxelSupercellDimensions);
  build_gksuper(t, D);
  oc_get_aperture(t, NULL, gg);
  t->sg = oc_get_deviation_parameter(t, gg);
}

/* setSupercellTilt2 (Lib_DynamicalTwoBeamImaging.f90:1048-1122). */
void oc_set_supercell_tilt2(oc_d2bi* t, const double* U, const double* R) {
  memcpy(t->U, U, 9 * sizeof(double));
  memcpy(t->R, R, 9 * sizeof(double));
  double a_sup[9], RU[9], D[9], gg[3];
  super_a(&t->super, a_sup);
  mat_mul(t->R, t->U, RU);
  find_transformed_supercell(a_sup, RU, D, t->delta, t->uvw, &t->nuvw, t->voxelSupercellDimensions);
  build_gksuper(t, D);
  oc_get_aperture(t, NULL, gg);
  t->sg = oc_get_deviation_parameter(t, gg);
}

/* findImageParameters (Lib_DynamicalTwoBeamImaging.f90:450-482). */
void oc_find_image_parameters(const oc_d2bi* t, double* aperpx, double* xmax, double* modg, int* Mx, int* My,
                              int* Mz) {
  double b[9], gg[3];
  reciprocal(t->a_cell, b);
  reflection(b, t->g, gg);
  *modg = oc_norm2(gg);
  for (int i = 1; i <= 3; ++i) xmax[i - 1] = super_side_length(&t->gksuper, i);
  *Mx = t->gksuper.Nx;
  *My = t->gksuper.Ny;
  *Mz = t->gksuper.Nz;
  *aperpx = sqrt(xmax[0] * xmax[1] / (double)((*Mx) * (*My)));
}

/* estimateMaxCountPerCell1 (Lib_LinkCell3D.f90:320-349). */
static int estimate_max_count_per_cell(double nCells, int nTotal) {
  double rho = nTotal / nCells;
  double pp = exp(-rho), psum = pp;
  for (int kk = 1; kk <= nTotal; ++kk) {
    if (psum >= 0.99) return kk;
    pp = pp * rho / kk;
    psum = psum + pp;
  }
  return nTotal;
}

/* FactoriseParallel0 for the process counts a single GPU replaces
 * (Lib_FactoriseParallel.f90:33-88). */
static int factorise_parallel(int Ai, int Bi, int N, int* C, int* D) {
  double Ad = Ai, Bd = Bi;
  switch (N) {
    case 1: *C = 1; *D = 1; return OC_OK;
    case 2: if (Ad >= Bd) { *C = 2; *D = 1; } else { *C = 1; *D = 2; } return OC_OK;
    case 3: if (Ad >= Bd) { *C = 3; *D = 1; } else { *C = 1; *D = 3; } return OC_OK;
    case 4:
      if (Ad >= 2 * Bd) { *C = 4; *D = 1; }
      else if (Bd >= 2 * Ad) { *C = 1; *D = 4; }
      else { *C = 2; *D = 2; }
      return OC_OK;
    default: return OC_ERR_ARG;
  }
}

/* Prologue of computeD2BI_img (Lib_DynamicalTwoBeamImaging.f90:1635-1852). */
int oc_image_geometry(const oc_d2bi* t, int64_t nAtoms, int nProcs, int jj, double precAngle, int nPrec,
                      oc_geom* G, double* aa) {
  memset(G, 0, sizeof *G);
  double aperpx, xmax[3], modg;
  int Mx, My, Mz;
  oc_find_image_parameters(t, &aperpx, xmax, &modg, &Mx, &My, &Mz);
  double costheta = 1.0, sintheta = 0.0;
  if (nPrec > 1) {
    costheta = cos(precAngle);
    sintheta = sin(precAngle);
  }
  double sigma = t->a0 / 2;
  G->sigma = sigma;
  G->i2s2 = 1 / (2 * sigma * sigma);
  double cmin = cell_side_length(&t->gksuper, 1), c2 = cell_side_length(&t->gksuper, 2);
  if (c2 < cmin) cmin = c2;
  int deltaM = (int)ceil(3 * sigma / cmin);
  int nMax = estimate_max_count_per_cell((double)Mx * My * Mz, (int)nAtoms) * deltaM * deltaM;
  int Cx, Cy;
  if (factorise_parallel(Mx, My, nProcs, &Cx, &Cy) != OC_OK) return OC_ERR_ARG;
  int Dx = (int)ceilf((float)Mx / (float)Cx);
  int Dy = (int)ceilf((float)My / (float)Cy);
  int Ex = (int)floorf((float)Dx / (float)deltaM + 2.0f);
  int Ey = (int)floorf((float)Dy / (float)deltaM + 2.0f);
  int Ez = (int)floorf((float)Mz / (float)deltaM);
  if (Ex < 3) Ex = 3;
  if (Ey < 3) Ey = 3;
  if (Ez < 3) Ez = 3;
  double a_col[9];
  const double* a_vox = t->gksuper.a;
  for (int i = 0; i < 3; ++i) {
    a_col[i] = (Dx + 2 * deltaM) * a_vox[i] / Ex;
    a_col[3 + i] = (Dy + 2 * deltaM) * a_vox[3 + i] / Ey;
    a_col[6 + i] = Mz * a_vox[6 + i] / Ez;
  }
  oc_super lc;
  oc_super_ctor(&lc, a_col, Ex, Ey, Ez);

  G->Mx = Mx;
  G->My = My;
  G->Mz = Mz;
  G->Ex = Ex;
  G->Ey = Ey;
  G->Ez = Ez;
  G->deltaM = deltaM;
  G->nMax0 = nMax;
  memcpy(G->a_col, lc.a, sizeof lc.a);
  memcpy(G->ia_col, lc.ia, sizeof lc.ia);
  memcpy(G->a_vox, a_vox, 9 * sizeof(double));
  G->deltaz = xmax[2] / Mz;
  G->bg = (PI / t->xig);
  G->b0 = (PI / t->xi0);
  G->cut2 = (3 * sigma) * (3 * sigma);
  G->useDensity = t->useDensityField;

  /* precession (:1805-1831); nApp = 1 and its aperture offset is zero */
  for (int prec = 1; prec <= nPrec; ++prec) {
    double gg[3];
    if (prec == 1) {
      oc_get_aperture(t, NULL, gg);
    } else {
      double phi = (prec - 1) * 2 * PI / (nPrec - 1);
      double ux = sin(phi), uy = cos(phi), BT[9];
      A(BT, 1, 1) = costheta + ux * ux * (1 - costheta);
      A(BT, 1, 2) = ux * uy * (1 - costheta);
      A(BT, 1, 3) = uy * sintheta;
      A(BT, 2, 1) = ux * uy * (1 - costheta);
      A(BT, 2, 2) = costheta + uy * uy * (1 - costheta);
      A(BT, 2, 3) = -ux * sintheta;
      A(BT, 3, 1) = -uy * sintheta;
      A(BT, 3, 2) = ux * sintheta;
      A(BT, 3, 3) = costheta;
      oc_get_aperture(t, BT, gg);
    }
    double z[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; ++i) z[i] = gg[i] + z[i];
    double sg = oc_get_deviation_parameter(t, z);
    aa[prec - 1] = (2 * PI * sg);
  }

  /* patch jj (:1843-1852) */
  int jy = jj / Cx, jx = jj - jy * Cx;
  double p0[3], p1[3];
  cell_to_real_i(&t->gksuper, jx * Dx, jy * Dy, 0, p0);
  cell_to_real_i(&lc, 1, 1, 0, p1);
  for (int i = 0; i < 3; ++i) G->lc_delta[i] = p0[i] - p1[i];
  G->ix0 = jx * Dx;
  G->ix1 = ((jx + 1) * Dx < Mx) ? (jx + 1) * Dx : Mx;
  G->iy0 = jy * Dy;
  G->iy1 = ((jy + 1) * Dy < My) ? (jy + 1) * Dy : My;

  /* findGdotR's transform (:1220-1240): RU, replicas, untilted aperture */
  mat_mul(t->R, t->U, G->RU);
  memcpy(G->delta, t->delta, sizeof t->delta);
  G->nuvw = t->nuvw;
  for (int nn = 0; nn < t->nuvw; ++nn) {
    double sv[9];
    super_a(&t->super, sv);
    for (int i = 0; i < 3; ++i)
      G->Ruvw[3 * nn + i] = t->uvw[3 * nn + 0] * sv[i] + t->uvw[3 * nn + 1] * sv[3 + i] + t->uvw[3 * nn + 2] * sv[6 + i];
  }
  oc_get_aperture(t, NULL, G->g);
  return OC_OK;
}

/* ------------------------------------------------------------------------ */
/* LinkCell3D                                                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n, cap;
  int* indx;
  double* x; /* 3 per entry */
} lc_cell;

typedef struct {
  oc_super s;
  int nMax0;
  int maxCount;
  lc_cell* c;
} lc3d;

/* LinkCell3D_ctor1 / Cell_ctor0 (Lib_LinkCell3D.f90:237-259, 288-301). */
static int lc_ctor(lc3d* L, const oc_super* s, int nMax0) {
  L->s = *s;
  L->nMax0 = nMax0;
  L->maxCount = 0;
  size_t nc = (size_t)s->Nx * s->Ny * s->Nz;
  L->c = (lc_cell*)calloc(nc, sizeof(lc_cell));
  if (!L->c) return OC_ERR_ALLOC;
  for (size_t i = 0; i < nc; ++i) {
    L->c[i].cap = nMax0;
    if (nMax0 > 0) {
      L->c[i].indx = (int*)malloc(sizeof(int) * nMax0);
      L->c[i].x = (double*)malloc(sizeof(double) * 3 * nMax0);
      if (!L->c[i].indx || !L->c[i].x) return OC_ERR_ALLOC;
    }
  }
  return OC_OK;
}

static void lc_delete(lc3d* L) {
  if (!L->c) return;
  size_t nc = (size_t)L->s.Nx * L->s.Ny * L->s.Nz;
  for (size_t i = 0; i < nc; ++i) {
    free(L->c[i].indx);
    free(L->c[i].x);
  }
  free(L->c);
  L->c = NULL;
}

/* clear0 (Lib_LinkCell3D.f90:576-590). */
static void lc_clear(lc3d* L) {
  size_t nc = (size_t)L->s.Nx * L->s.Ny * L->s.Nz;
  for (size_t i = 0; i < nc; ++i) L->c[i].n = 0;
  L->maxCount = 0;
}

static lc_cell* lc_at(lc3d* L, int ix, int iy, int iz) {
  return &L->c[(size_t)ix + (size_t)L->s.Nx * ((size_t)iy + (size_t)L->s.Ny * iz)];
}

/* add0 with doubleCell (Lib_LinkCell3D.f90:691-748, 388-410). */
static int lc_add(lc3d* L, int id, const double* x) {
  double yy[3], zz[3];
  real_to_cell(&L->s, x, yy);
  for (int i = 0; i < 3; ++i) zz[i] = yy[i] - floor(yy[i]);
  int ix = imod((int)floor(yy[0]) + (L->s.Nx << 4), L->s.Nx);
  int iy = imod((int)floor(yy[1]) + (L->s.Ny << 4), L->s.Ny);
  int iz = imod((int)floor(yy[2]) + (L->s.Nz << 4), L->s.Nz);
  lc_cell* c = lc_at(L, ix, iy, iz);
  int nn = c->n + 1;
  if (nn > c->cap) {
    if (c->cap == 16 * L->nMax0) return OC_ERR_CAPACITY;
    int nc = (c->cap == 0) ? 2 : ((2 * c->cap > 2) ? 2 * c->cap : 2);
    int* ni = (int*)realloc(c->indx, sizeof(int) * nc);
    if (!ni) return OC_ERR_ALLOC;
    c->indx = ni;
    double* nx = (double*)realloc(c->x, sizeof(double) * 3 * nc);
    if (!nx) return OC_ERR_ALLOC;
    c->x = nx;
    c->cap = nc;
  }
  c->n = nn;
  c->indx[nn - 1] = id;
  memcpy(&c->x[3 * (nn - 1)], zz, sizeof zz);
  if (nn > L->maxCount) L->maxCount = nn;
  return OC_OK;
}

/* neighbourList1b (Lib_LinkCell3D.f90:1515-1605); also returns the real-space
 * separations when dxo is non-null (the neighbourList0a layout). */
static int lc_neighbours(const lc3d* L, const double* x, double sigma, int* id, double* r2, double* dxo,
                         int64_t* ntests) {
  int Nx = L->s.Nx, Ny = L->s.Ny, Nz = L->s.Nz;
  const double* a = L->s.a;
  double zi[3];
  real_to_cell(&L->s, x, zi);
  int ix = imod((int)floor(zi[0]) + 16 * Nx, Nx);
  int iy = imod((int)floor(zi[1]) + 16 * Ny, Ny);
  int iz = imod((int)floor(zi[2]) + 16 * Nz, Nz);
  zi[0] = zi[0] - ix;
  zi[1] = zi[1] - iy;
  zi[2] = zi[2] - iz;
  int n = 0;
  int64_t tests = 0;
  for (int kz = -1; kz <= 1; ++kz) {
    int jz = imod(iz + Nz + kz, Nz);
    double dzi3 = kz - zi[2];
    for (int ky = -1; ky <= 1; ++ky) {
      int jy = imod(iy + Ny + ky, Ny);
      double dzi2 = ky - zi[1];
      for (int kx = -1; kx <= 1; ++kx) {
        int jx = imod(ix + Nx + kx, Nx);
        double dzi1 = kx - zi[0];
        const lc_cell* c = &L->c[(size_t)jx + (size_t)Nx * ((size_t)jy + (size_t)Ny * jz)];
        tests += c->n;
        for (int jk = 0; jk < c->n; ++jk) {
          double dzj1 = c->x[3 * jk + 0] + dzi1;
          double dzj2 = c->x[3 * jk + 1] + dzi2;
          double dzj3 = c->x[3 * jk + 2] + dzi3;
          double d0 = A(a, 1, 1) * dzj1 + A(a, 1, 2) * dzj2 + A(a, 1, 3) * dzj3;
          double d1 = A(a, 2, 1) * dzj1 + A(a, 2, 2) * dzj2 + A(a, 2, 3) * dzj3;
          double d2 = A(a, 3, 1) * dzj1 + A(a, 3, 2) * dzj2 + A(a, 3, 3) * dzj3;
          double dd = d0 * d0 + d1 * d1 + d2 * d2;
          if (dd <= sigma * sigma) {
            id[n] = c->indx[jk];
            r2[n] = dd;
            if (dxo) {
              dxo[3 * n + 0] = d0;
              dxo[3 * n + 1] = d1;
              dxo[3 * n + 2] = d2;
            }
            ++n;
          }
        }
      }
    }
  }
  if (ntests) *ntests += tests;
  return n;
}

static int lc_max_27(const lc3d* L) {
  /* upper bound on the neighbour count of any point: 27 x largest cell */
  size_t nc = (size_t)L->s.Nx * L->s.Ny * L->s.Nz;
  int m = 0;
  for (size_t i = 0; i < nc; ++i)
    if (L->c[i].n > m) m = L->c[i].n;
  return 27 * (m > 0 ? m : 1);
}

int oc_neighbour_list(const oc_super* lc, const double* pts, int npts, int nMax0, const double* query,
                      double cutoff, int* ids, double* dx, double* r2, int maxn, int* max_count) {
  lc3d L;
  if (lc_ctor(&L, lc, nMax0) != OC_OK) return -OC_ERR_ALLOC;
  for (int i = 0; i < npts; ++i) {
    int rc = lc_add(&L, i + 1, &pts[3 * i]);
    if (rc != OC_OK) {
      lc_delete(&L);
      return -rc;
    }
  }
  int need = lc_max_27(&L);
  int* tid = (int*)malloc(sizeof(int) * need);
  double* tr2 = (double*)malloc(sizeof(double) * need);
  double* tdx = (double*)malloc(sizeof(double) * 3 * need);
  int n = lc_neighbours(&L, query, cutoff, tid, tr2, tdx, NULL);
  for (int i = 0; i < n && i < maxn; ++i) {
    ids[i] = tid[i];
    r2[i] = tr2[i];
    memcpy(&dx[3 * i], &tdx[3 * i], 3 * sizeof(double));
  }
  if (max_count) *max_count = L.maxCount;
  free(tid);
  free(tr2);
  free(tdx);
  lc_delete(&L);
  return n;
}

/* ------------------------------------------------------------------------ */
/* findGdotR and the voxel loops                                            */
/* ------------------------------------------------------------------------ */

/* findGdotR (Lib_DynamicalTwoBeamImaging.f90:1160-1265): rotate the 27
 * replicas, keep atoms inside the link-cell box, bin them and record g.y. */
static int find_gdotr(const oc_geom* G, const double* x, int64_t ldx, int64_t nAtoms, lc3d* L, double** gdotr,
                      int64_t* nkept) {
  lc_clear(L);
  int64_t cap = (int64_t)(nAtoms * 1.5) + 1, ii = 0;
  double* gd = (double*)malloc(sizeof(double) * cap);
  if (!gd) return OC_ERR_ALLOC;
  for (int nn = 0; nn < G->nuvw; ++nn) {
    const double* Ruvw = &G->Ruvw[3 * nn];
    for (int64_t jj = 0; jj < nAtoms; ++jj) {
      double yy[3], zz[3];
      const double* xa = &x[jj * ldx];
      for (int i = 0; i < 3; ++i) yy[i] = xa[i] + Ruvw[i];
      mat_vec(G->RU, yy, yy);
      for (int i = 0; i < 3; ++i) yy[i] = yy[i] + G->delta[i];
      for (int i = 0; i < 3; ++i) zz[i] = yy[i] - G->lc_delta[i];
      if (point_in_super(&L->s, zz)) {
        ii = ii + 1;
        if (ii > cap) {
          double* ng = (double*)realloc(gd, sizeof(double) * cap * 2);
          if (!ng) {
            free(gd);
            return OC_ERR_ALLOC;
          }
          gd = ng;
          cap *= 2;
        }
        int rc = lc_add(L, (int)ii, zz);
        if (rc != OC_OK) {
          free(gd);
          return rc;
        }
        gd[ii - 1] = G->g[0] * yy[0] + G->g[1] * yy[1] + G->g[2] * yy[2];
      }
    }
  }
  *gdotr = gd;
  *nkept = ii;
  return OC_OK;
}

/* convertScaledRangeToRho (Lib_DynamicalTwoBeamImaging.f90:1973-1994). */
static double scaled_range_to_rho(double r2_min, double sig) {
  if (r2_min < sig * sig) return 1.0;
  if (r2_min > 4 * sig * sig) return 0.0;
  double xx = (sqrt(r2_min) / sig - 1.0);
  return 1 - xx * xx * xx * (10 - 15 * xx + 6 * xx * xx);
}

/* dynamicalTwoBeamIntegrationColumn_phaserho (Lib_DynamicalTwoBeamImaging.f90:2316-2480). */
double oc_integrate_column(double a, double b0, double bg, double dz, const double* x, const double* rho, int nz) {
  double phi0r = 1.0, phi0i = 0.0, phigr = 0.0, phigi = 0.0;
  for (int ii = 0; ii <= nz - 2; ii += 2) {
    double c0[3], ca[3], cgr[3], cgi[3];
    for (int s = 0; s < 3; ++s) {
      int k = ii + s;
      c0[s] = b0 * rho[k];
      ca[s] = b0 * rho[k] + a;
      cgr[s] = bg * rho[k] * x[2 * k];
      cgi[s] = bg * rho[k] * x[2 * k + 1];
    }
    double d0r, d0i, dgr, dgi;
    /* step 1 at ii */
    d0r = -c0[0] * phi0i - cgi[0] * phigr - cgr[0] * phigi;
    d0i = c0[0] * phi0r + cgr[0] * phigr - cgi[0] * phigi;
    dgr = cgi[0] * phi0r - cgr[0] * phi0i - ca[0] * phigi;
    dgi = cgr[0] * phi0r + cgi[0] * phi0i + ca[0] * phigr;
    double p0r2 = phi0r, p0i2 = phi0i, pgr2 = phigr, pgi2 = phigi;
    double p0r1 = phi0r + d0r * dz / 3, p0i1 = phi0i + d0i * dz / 3;
    double pgr1 = phigr + dgr * dz / 3, pgi1 = phigi + dgi * dz / 3;
    phi0r = phi0r + d0r * dz;
    phi0i = phi0i + d0i * dz;
    phigr = phigr + dgr * dz;
    phigi = phigi + dgi * dz;
    /* step 2 at ii+1 */
    d0r = -c0[1] * phi0i - cgi[1] * phigr - cgr[1] * phigi;
    d0i = c0[1] * phi0r + cgr[1] * phigr - cgi[1] * phigi;
    dgr = cgi[1] * phi0r - cgr[1] * phi0i - ca[1] * phigi;
    dgi = cgr[1] * phi0r + cgi[1] * phi0i + ca[1] * phigr;
    phi0r = p0r2 + d0r * dz;
    phi0i = p0i2 + d0i * dz;
    phigr = pgr2 + dgr * dz;
    phigi = pgi2 + dgi * dz;
    p0r1 = p0r1 + d0r * 2 * dz / 3;
    p0i1 = p0i1 + d0i * 2 * dz / 3;
    pgr1 = pgr1 + dgr * 2 * dz / 3;
    pgi1 = pgi1 + dgi * 2 * dz / 3;
    /* step 3 at ii+1 */
    d0r = -c0[1] * phi0i - cgi[1] * phigr - cgr[1] * phigi;
    d0i = c0[1] * phi0r + cgr[1] * phigr - cgi[1] * phigi;
    dgr = cgi[1] * phi0r - cgr[1] * phi0i - ca[1] * phigi;
    dgi = cgr[1] * phi0r + cgi[1] * phi0i + ca[1] * phigr;
    phi0r = p0r2 + d0r * 2 * dz;
    phi0i = p0i2 + d0i * 2 * dz;
    phigr = pgr2 + dgr * 2 * dz;
    phigi = pgi2 + dgi * 2 * dz;
    p0r1 = p0r1 + d0r * 2 * dz / 3;
    p0i1 = p0i1 + d0i * 2 * dz / 3;
    pgr1 = pgr1 + dgr * 2 * dz / 3;
    pgi1 = pgi1 + dgi * 2 * dz / 3;
    /* step 4 at ii+2 */
    d0r = -c0[2] * phi0i - cgi[2] * phigr - cgr[2] * phigi;
    d0i = c0[2] * phi0r + cgr[2] * phigr - cgi[2] * phigi;
    dgr = cgi[2] * phi0r - cgr[2] * phi0i - ca[2] * phigi;
    dgi = cgr[2] * phi0r + cgi[2] * phi0i + ca[2] * phigr;
    phi0r = p0r1 + d0r * dz / 3;
    phi0i = p0i1 + d0i * dz / 3;
    phigr = pgr1 + dgr * dz / 3;
    phigi = pgi1 + dgi * dz / 3;
    double phimag = phi0r * phi0r + phi0i * phi0i + phigr * phigr + phigi * phigi;
    phimag = 1 / sqrt(phimag);
    phi0r = phi0r * phimag;
    phi0i = phi0i * phimag;
    phigr = phigr * phimag;
    phigi = phigi * phimag;
  }
  return phigr * phigr + phigi * phigi;
}

/* Voxel loop of one pixel column (:1877-1900). */
static void column_field(const oc_geom* G, const lc3d* L, const double* gdotr, int ix, int iy, double* xf,
                         double* rho, int* id, double* r2, oc_stats* st) {
  oc_super gk;
  gk.Nx = G->Mx;
  gk.Ny = G->My;
  gk.Nz = G->Mz;
  memcpy(gk.a, G->a_vox, sizeof gk.a);
  for (int iz = 0; iz < G->Mz; ++iz) {
    double xx[3];
    cell_to_real_i(&gk, ix, iy, iz, xx);
    for (int i = 0; i < 3; ++i) xx[i] = xx[i] - G->lc_delta[i];
    int64_t tests = 0;
    int nn = lc_neighbours(L, xx, 3 * G->sigma, id, r2, NULL, &tests);
    double r2_min = HUGE1, sr = 0.0, si = 0.0;
    for (int kk = 0; kk < nn; ++kk) {
      if (r2[kk] < r2_min) r2_min = r2[kk];
      double w = exp(-r2[kk] * G->i2s2), s, c;
      sincos(gdotr[id[kk] - 1], &s, &c);
      sr = sr + w * c;
      si = si + w * s;
    }
    if (G->useDensity) rho[iz] = scaled_range_to_rho(r2_min, G->sigma);
    double ww = hypot(sr, si);
    ww = 1 / (1.0e-16 > ww ? 1.0e-16 : ww);
    xf[2 * iz] = sr * ww;
    xf[2 * iz + 1] = si * ww;
    if (st) {
      st->n_tests += tests;
      st->n_accepted += nn;
      st->n_voxels += 1;
    }
  }
  xf[2 * G->Mz] = xf[0];
  xf[2 * G->Mz + 1] = xf[1];
  rho[G->Mz] = rho[0];
}

int oc_patch_image_rows(const oc_geom* G, const double* aa, int nPrec, const double* x, int64_t ldx, int64_t nAtoms,
                        int iy_lo, int iy_hi, double* img, oc_stats* stats, int nthreads) {
  oc_super lcs;
  lcs.Nx = G->Ex;
  lcs.Ny = G->Ey;
  lcs.Nz = G->Ez;
  memcpy(lcs.a, G->a_col, sizeof lcs.a);
  memcpy(lcs.ia, G->ia_col, sizeof lcs.ia);
  lc3d L;
  int rc = lc_ctor(&L, &lcs, G->nMax0);
  if (rc != OC_OK) return rc;
  double* gdotr = NULL;
  int64_t nkept = 0;
  rc = find_gdotr(G, x, ldx, nAtoms, &L, &gdotr, &nkept);
  if (rc != OC_OK) {
    lc_delete(&L);
    return rc;
  }
  int need = lc_max_27(&L);
  if (iy_lo < G->iy0) iy_lo = G->iy0;
  if (iy_hi > G->iy1) iy_hi = G->iy1;
  int64_t tests = 0, acc = 0, vox = 0;
  int err = 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads) reduction(+ : tests, acc, vox)
#endif
  {
    double* xf = (double*)malloc(sizeof(double) * 2 * (G->Mz + 1));
    double* rho = (double*)malloc(sizeof(double) * (G->Mz + 1));
    int* id = (int*)malloc(sizeof(int) * need);
    double* r2 = (double*)malloc(sizeof(double) * need);
    if (!xf || !rho || !id || !r2) {
      err = 1;
    } else {
      for (int i = 0; i <= G->Mz; ++i) rho[i] = 1.0;
      oc_stats st;
      memset(&st, 0, sizeof st);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int iy = iy_lo; iy < iy_hi; ++iy) {
        for (int ix = G->ix0; ix < G->ix1; ++ix) {
          column_field(G, &L, gdotr, ix, iy, xf, rho, id, r2, &st);
          double acc_px = img[(size_t)ix + (size_t)G->Mx * iy];
          for (int p = 0; p < nPrec; ++p)
            acc_px = acc_px + oc_integrate_column(aa[p], G->b0, G->bg, G->deltaz, xf, rho, G->Mz);
          img[(size_t)ix + (size_t)G->Mx * iy] = acc_px;
        }
      }
      tests += st.n_tests;
      acc += st.n_accepted;
      vox += st.n_voxels;
    }
    free(xf);
    free(rho);
    free(id);
    free(r2);
  }
  (void)nthreads;
  if (stats) {
    stats->n_kept += nkept;
    stats->n_tests += tests;
    stats->n_accepted += acc;
    stats->n_voxels += vox;
    if (L.maxCount > stats->max_cell_count) stats->max_cell_count = L.maxCount;
  }
  free(gdotr);
  lc_delete(&L);
  return err ? OC_ERR_ALLOC : OC_OK;
}

int oc_patch_image(const oc_geom* G, const double* aa, int nPrec, const double* x, int64_t ldx, int64_t nAtoms,
                   double* img, oc_stats* stats, int nthreads) {
  return oc_patch_image_rows(G, aa, nPrec, x, ldx, nAtoms, G->iy0, G->iy1, img, stats, nthreads);
}

/* computeD2BI_img with one process (Lib_DynamicalTwoBeamImaging.f90:1563-1998). */
int oc_compute_d2bi_img(const oc_d2bi* t, const double* x, int64_t ldx, int64_t nAtoms, double precAngle, int nPrec,
                        double* img, oc_stats* stats, int nthreads) {
  if (nPrec < 1) return OC_ERR_ARG;
  oc_geom G;
  double* aa = (double*)malloc(sizeof(double) * nPrec);
  int rc = oc_image_geometry(t, nAtoms, 1, 0, precAngle, nPrec, &G, aa);
  if (rc != OC_OK) {
    free(aa);
    return rc;
  }
  memset(img, 0, sizeof(double) * (size_t)G.Mx * G.My);
  if (stats) memset(stats, 0, sizeof *stats);
  rc = oc_patch_image(&G, aa, nPrec, x, ldx, nAtoms, img, stats, nthreads);
  for (size_t i = 0; i < (size_t)G.Mx * G.My; ++i) img[i] = img[i] / (double)(1 * nPrec);
  free(aa);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* d2bi                                                                     */
/* ------------------------------------------------------------------------ */

/* src/d2bi.f90:782-789, 856-866, 983-991, 1145-1268, 1352-1381 for one
 * diffraction condition and tomography step nn. */
int oc_d2bi_setup(const oc_args* args, double* x, int64_t ldx, int64_t nAtoms, int nn, oc_d2bi* t,
                  double* aperpx_out) {
  double a0in[3] = {args->a0in, args->a0in, args->a0in};
  double a0 = (a0in[0] + a0in[1] + a0in[2]) / 3;
  const double* a_super = args->a_super;
  int Mx = (int)floor(args->M[0] * oc_norm2(&a_super[0]) / a0);
  int My = (int)floor(args->M[0] * oc_norm2(&a_super[3]) / a0);
  int Mz = (int)floor(args->M[1] * oc_norm2(&a_super[6]) / a0);
  if (Mx < 3) Mx = 3;
  if (My < 3) My = 3;
  if (Mz < 3) Mz = 3;
  double a_vox[9];
  for (int i = 0; i < 3; ++i) {
    a_vox[i] = a_super[i] / Mx;
    a_vox[3 + i] = a_super[3 + i] / My;
    a_vox[6 + i] = a_super[6 + i] / Mz;
  }
  oc_super super;
  oc_super_ctor(&super, a_vox, Mx, My, Mz);
  for (int64_t i = 0; i < nAtoms; ++i) oc_wrap_pbc(&super, &x[i * ldx], &x[i * ldx]);

  double a_cell[9];
  identity3(a_cell);
  for (int i = 0; i < 9; ++i) a_cell[i] = a0 * a_cell[i];

  double d[3];
  if (args->haveD) {
    memcpy(d, args->d0, sizeof d);
  } else {
    double rot[9], xmin[3] = {HUGE1, HUGE1, HUGE1}, xmax[3] = {-HUGE1, -HUGE1, -HUGE1};
    oc_rotate_to_standard_frame(args->k, a_cell, args->g, rot);
    for (int64_t i = 0; i < nAtoms; ++i) {
      double yy[3];
      mat_vec(rot, &x[i * ldx], yy);
      for (int k = 0; k < 3; ++k) {
        if (yy[k] < xmin[k]) xmin[k] = yy[k];
        if (yy[k] > xmax[k]) xmax[k] = yy[k];
      }
    }
    for (int k = 0; k < 3; ++k) d[k] = xmax[k] - xmin[k];
  }
  double xi0 = args->xi0, xig = args->xig;
  if (args->xifile[0]) { /* d2bi.f90:1183-1192 */
    int idat[6] = {0, 0, 0, (int)lround(args->g[0]), (int)lround(args->g[1]), (int)lround(args->g[2])};
    double dat[2];
    int symm = args->lattice == OC_LATTICE_HCP ? OC_SYM_HEX : OC_SYM_CUBIC;
    if (oc_read_extinction_distances(args->xifile, idat, 2, symm, dat) != 1) return OC_ERR_ARG;
    xi0 = dat[0];
    xig = dat[1];
  }
  oc_d2bi_ctor(t, &super, a0, args->k, args->g, args->V, args->M[0], args->M[1]);
  oc_set_conventional_unit_cell(t, a_cell);
  int rc = oc_set_voxel_supercell_size(t, d);
  if (rc != OC_OK) return rc;
  if (args->tilt_mode == 3) {
    rc = oc_set_supercell_tilt1a(t, args->ng, args->xifile, args->lattice, args->thetaMax, args->rhoMax,
                                 args->surf ? x : NULL, ldx, nAtoms, NULL);
    if (rc != OC_OK) return rc;
  } else if (args->tilt_mode == 1) {
    oc_set_deviation_parameter(t, args->sg);
    oc_set_supercell_tilt0(t);
  } else if (args->tilt_mode == 2) {
    double U[9];
    if (args->haveU)
      memcpy(U, args->U, sizeof U);
    else
      identity3(U);
    oc_set_supercell_tilt2(t, U, args->R);
  } else {
    oc_set_deviation_parameter(t, 0.0);
    oc_set_supercell_tilt0(t);
  }
  double U0[9], R0[9];
  memcpy(U0, t->U, sizeof U0);
  memcpy(R0, t->R, sizeof R0);
  oc_set_extinction_distances(t, xi0, xig);
  double aperpx, xm[3], modg;
  int mx, my, mz;
  oc_find_image_parameters(t, &aperpx, xm, &modg, &mx, &my, &mz);
  oc_set_use_density_field(t, args->useDensity);
  if (args->nTomo > 1) {
    double theta = args->tomoAngle - 2 * args->tomoAngle * nn / (args->nTomo - 1);
    theta = theta * 3.141592654 / 180.0;
    double R[9] = {1.0, 0.0, 0.0, 0.0, cos(theta), sin(theta), 0.0, -sin(theta), cos(theta)};
    mat_mul(R, R0, R);
    oc_set_supercell_tilt2(t, U0, R);
  }
  if (aperpx_out) *aperpx_out = aperpx;
  return OC_OK;
}

/* gaussianBlurImage (src/d2bi.f90:1543-1624). */
void oc_gaussian_blur(const double* f_in, int Nx, int Ny, double t, double* f_out) {
  int Nk = (int)ceil(t * 5);
  if (Nk < 5) Nk = 5;
  double* kernel = (double*)malloc(sizeof(double) * (Nk + 1));
  double i2s2 = 1 / (2 * t * t);
  kernel[0] = 1.0;
  for (int ix = 1; ix <= Nk; ++ix) kernel[ix] = exp(-(ix * ix * i2s2));
  double* f_stripe = (double*)malloc(sizeof(double) * Ny);
  double* w_stripe = (double*)malloc(sizeof(double) * Nx);
  for (int iy = 0; iy < Ny; ++iy) {
    for (int ix = 0; ix < Nx; ++ix) {
      double wf = 0.0, ws = 0.0;
      int lo = ix - Nk > 0 ? ix - Nk : 0, hi = ix + Nk < Nx - 1 ? ix + Nk : Nx - 1;
      for (int jj = lo; jj <= hi; ++jj) {
        double ww = kernel[abs(jj - ix)];
        wf = wf + ww * f_in[(size_t)jj + (size_t)Nx * iy];
        ws = ws + ww;
      }
      f_out[(size_t)ix + (size_t)Nx * iy] = wf;
      if (iy == 0) w_stripe[ix] = 1 / ws;
    }
  }
  for (int ix = 0; ix < Nx; ++ix) {
    for (int iy = 0; iy < Ny; ++iy) f_stripe[iy] = f_out[(size_t)ix + (size_t)Nx * iy];
    for (int iy = 0; iy < Ny; ++iy) {
      double wf = 0.0, ws = 0.0;
      int lo = iy - Nk > 0 ? iy - Nk : 0, hi = iy + Nk < Ny - 1 ? iy + Nk : Ny - 1;
      for (int jj = lo; jj <= hi; ++jj) {
        double ww = kernel[abs(jj - iy)];
        wf = wf + ww * f_stripe[jj];
        ws = ws + ww;
      }
      f_out[(size_t)ix + (size_t)Nx * iy] = wf * w_stripe[ix] / (ws);
    }
  }
  free(kernel);
  free(f_stripe);
  free(w_stripe);
}

/* write_greyscale_png(normalise=.true.) levels (Lib_Png.f90:117-181) and the
 * C writer's clamp and truncation (Lib_Greyscale.c:234-241). */
void oc_png_levels(const double* img, int Nx, int Ny, uint16_t* levels) {
  const double ONE = 1.0 - 1.0 / 65536;
  double mn = img[0], mx = img[0];
  for (size_t i = 0; i < (size_t)Nx * Ny; ++i) {
    if (img[i] < mn) mn = img[i];
    if (img[i] > mx) mx = img[i];
  }
  double aa, bb;
  if (mx - mn < 1.0e-16) {
    aa = 0.0;
    bb = 0.5;
  } else {
    aa = ONE / (mx - mn);
    bb = -aa * mn;
  }
  for (int y = 0; y < Ny; ++y)
    for (int x = 0; x < Nx; ++x) {
      float f = (float)(aa * img[(size_t)x + (size_t)Nx * y] + bb);
      if (f > 0.999984741) {
        f = 0.999984741f;
      } else if (f < 0.0) {
        f = 0.0f;
      }
      int i = (int)(f * 65536);
      levels[(size_t)y * Nx + x] = (uint16_t)i;
    }
}

/* outputImgAsPng, contrast mode (src/d2bi.f90:1531-1535): img = (img - lo)/(hi - lo),
 * clamped to [0, 1], then Lib_Png.f90:164-165 with aa = 1, bb = 0 and
 * Lib_Greyscale.c:230-245. */
void oc_png_levels_window(const double* img, int Nx, int Ny, double lo, double hi, uint16_t* levels) {
  for (int y = 0; y < Ny; ++y)
    for (int x = 0; x < Nx; ++x) {
      double v = (img[(size_t)x + (size_t)Nx * y] - lo) / (hi - lo);
      v = v < 1.0 ? v : 1.0;
      v = v > 0.0 ? v : 0.0;
      float f = (float)(1.0 * v + 0.0);
      if (f > 0.999984741) {
        f = 0.999984741f;
      } else if (f < 0.0) {
        f = 0.0f;
      }
      levels[(size_t)y * Nx + x] = (uint16_t)(int)(f * 65536);
    }
}

/* Fortran F12.7 of one value: C's correctly rounded %.7f of |v| (no exact ties arise at
 * 7 decimals of a binary value), '-' for negative values, right-justified, asterisks
 * when longer than 12 characters; NaN and Infinity spelled as gfortran does. */
static void f12_7(double v, char* o) {
  char s[400];
  if (isnan(v)) {
    snprintf(s, sizeof s, "NaN");
  } else if (isinf(v)) {
    snprintf(s, sizeof s, "%s", v > 0 ? "Infinity" : "-Infinity");
  } else {
    snprintf(s, sizeof s, "%s%.7f", signbit(v) ? "-" : "", fabs(v));
  }
  const size_t len = strlen(s);
  if (len > 12) {
    memset(o, '*', 12);
  } else {
    memset(o, ' ', 12 - len);
    memcpy(o + 12 - len, s, len);
  }
}

long long oc_format_f12_7(const double* v, long long n, char* out) {
  long long p = 0;
  for (long long i = 0; i < n; ++i) {
    f12_7(v[i], out + p);
    p += 12;
    if (i % 1000 == 999 || i == n - 1) out[p++] = '\n';
  }
  return p;
}

long long oc_read_lammps_atoms(const char* path, long long offset, long long n_atoms, double* x, int* types) {
  FILE* f = fopen(path, "rb");
  if (!f) return 1;
  fseek(f, offset, SEEK_SET);
  size_t cap = 1 << 16;
  char* line = (char*)malloc(cap);
  long long bad = 0;
  for (long long i = 0; i < n_atoms; ++i) {
    if (!fgets(line, (int)cap, f)) {
      bad = i + 1;
      break;
    }
    for (char* q = line; *q; ++q)
      if (*q == ',') *q = ' ';  /* list-directed reads also separate by commas */
    long long id;
    int ty;
    double a, b, c;
    if (sscanf(line, "%lld %d %lf %lf %lf", &id, &ty, &a, &b, &c) != 5) {
      bad = i + 1;
      break;
    }
    x[3 * i] = a;
    x[3 * i + 1] = b;
    x[3 * i + 2] = c;
    types[i] = ty;
  }
  free(line);
  fclose(f);
  return bad;
}


/* ------------------------------------------------------------------------ */
/* The -ng tilt search (setSupercellTilt1a / setSupercellTilt1)             */
/* ------------------------------------------------------------------------ */

/* NTHETA (Lib_DiffractionConditions.f90:22) and DEGTORAD (:26). */
#define OC_NTHETA 2000
static const double DEGTORAD = 3.141592654 / 180;

/* symmetry (Lib_ReadExtinctionDistances.f90:112-170): the standard form of a
 * reflection under cubic or hexagonal symmetry. */
static void xi_symmetry(const int* in, int symm, int* out) {
  int hh = abs(in[0]), kk = abs(in[1]), ll = abs(in[2]);
  if (symm == OC_SYM_CUBIC) {
    if (hh >= (kk > ll ? kk : ll)) {
      if (kk >= ll) { out[0] = hh; out[1] = kk; out[2] = ll; }
      else { out[0] = hh; out[1] = ll; out[2] = kk; }
    } else if (kk >= (hh > ll ? hh : ll)) {
      if (hh >= ll) { out[0] = kk; out[1] = hh; out[2] = ll; }
      else { out[0] = kk; out[1] = ll; out[2] = hh; }
    } else {
      if (hh >= kk) { out[0] = ll; out[1] = hh; out[2] = kk; }
      else { out[0] = ll; out[1] = kk; out[2] = hh; }
    }
  } else {
    if (in[0] * in[1] >= 0) {
      if (hh >= kk) { out[0] = hh; out[1] = kk; out[2] = ll; }
      else { out[0] = kk; out[1] = hh; out[2] = ll; }
    } else {
      if (hh >= kk) { out[0] = hh; out[1] = -kk; out[2] = ll; }
      else { out[0] = kk; out[1] = -hh; out[2] = ll; }
    }
  }
}

/* One list-directed READ of `dummy, idat(3), rdat(5)`: a new record per READ,
 * items separated by blanks or commas and continued over records as needed.
 * Returns 0, or -1 at the end of the file or on an item of the wrong form. */
static int read_xi_record(FILE* f, int* idat, double* rdat) {
  char line[4096];
  int got = 0;
  while (got < 9) {
    if (!fgets(line, sizeof line, f)) return -1;
    char* p = line;
    while (got < 9) {
      while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r' || *p == '\n') ++p;
      if (!*p) break;
      char* s = p;
      while (*p && *p != ' ' && *p != '\t' && *p != ',' && *p != '\r' && *p != '\n') ++p;
      char tok[256];
      size_t len = (size_t)(p - s) < sizeof tok - 1 ? (size_t)(p - s) : sizeof tok - 1;
      memcpy(tok, s, len);
      tok[len] = 0;
      if (got == 0) {
        /* the element name: any token */
      } else if (got <= 3) {
        char* e;
        long v = strtol(tok, &e, 10);
        if (e == tok || *e) return -1;
        idat[got - 1] = (int)v;
      } else {
        for (char* q = tok; *q; ++q)
          if (*q == 'd' || *q == 'D') *q = 'E';
        char* e;
        double v = strtod(tok, &e);
        if (e == tok || *e) return -1;
        rdat[got - 4] = v;
      }
      ++got;
    }
  }
  return 0;
}

/* readExtinctionDistance (Lib_ReadExtinctionDistances.f90:29-109). */
int oc_read_extinction_distances(const char* path, const int* hkl, int n, int symm, double* xi_g) {
  for (int j = 0; j < n; ++j) xi_g[j] = HUGE1;
  FILE* f = fopen(path, "r");
  if (!f) return -1;
  int* hs = (int*)malloc(sizeof(int) * 3 * (n > 0 ? n : 1));
  char* found = (char*)calloc(n > 0 ? n : 1, 1);
  for (int j = 0; j < n; ++j) xi_symmetry(&hkl[3 * j], symm, &hs[3 * j]);
  char line[4096];
  int bad = !fgets(line, sizeof line, f);
  bad = !fgets(line, sizeof line, f); /* only the second read's status is checked */
  if (bad) {
    free(hs);
    free(found);
    fclose(f);
    return -1;
  }
  for (int ii = 1; ii <= 1000; ++ii) {
    int idat[3], is[3];
    double rdat[5];
    if (read_xi_record(f, idat, rdat) != 0) break;
    xi_symmetry(idat, symm, is);
    int all = 1;
    for (int j = 0; j < n; ++j) {
      if (is[0] == hs[3 * j] && is[1] == hs[3 * j + 1] && is[2] == hs[3 * j + 2]) {
        found[j] = 1;
        xi_g[j] = rdat[4];
      }
      all = all && found[j];
    }
    if (all) break;
  }
  int ok = 1;
  for (int j = 0; j < n; ++j) ok = ok && found[j];
  free(hs);
  free(found);
  fclose(f);
  return ok;
}

/* permittedReflections (Lib_Lattices.f90:678-735): the reflections with
 * |hkl|^2 <= rho^2 allowed by the lattice, l outermost, h innermost. */
int oc_permitted_reflections(int latt, double rho, int* hkl, int cap) {
  int mm = (int)ceil(rho + 1.0e-12);
  int n = 0;
  for (int lp = -mm; lp <= mm; ++lp)
    for (int kp = -mm; kp <= mm; ++kp)
      for (int hp = -mm; hp <= mm; ++hp) {
        int rr = lp * lp + kp * kp + hp * hp, ok;
        if (latt == OC_LATTICE_HCP) {
          rr = (int)floor((double)((hp + kp) * (hp + kp) + (hp - kp) * (hp - kp) / 3) + lp * lp * 0.375);
          if (rr > rho * rho + 1.0e-6) continue;
          ok = !((imod(hp + 2 * kp, 3) == 0) && (imod(abs(lp), 2) == 1));
        } else {
          if (rr > rho * rho + 1.0e-6) continue;
          if (latt == OC_LATTICE_FCC) {
            int hx = imod(hp, 2), kx = imod(kp, 2), lx = imod(lp, 2);
            ok = (hx * hx + kx * kx + lx * lx) - (hx * kx + kx * lx + lx * hx) == 0;
          } else if (latt == OC_LATTICE_BCC) {
            ok = imod(hp + kp + lp, 2) == 0;
          } else {
            ok = 1;
          }
        }
        if (ok) {
          if (hkl && n < cap) {
            hkl[3 * n] = hp;
            hkl[3 * n + 1] = kp;
            hkl[3 * n + 2] = lp;
          }
          ++n;
        }
      }
  return n;
}

/* find_gvectors_permittedReflections (Lib_DiffractionConditions.f90:1727-1790),
 * including its second swap, which exchanges hklp(:,1) (not hklp(:,2)) with
 * hklp(:,ihkl) while ghkl(:,2) is exchanged with ghkl(:,ihkl). */
static int gvectors_permitted(int latt, const double* B, const int* hkl, double rho, double** ghkl_out,
                              int** hklp_out) {
  int n = oc_permitted_reflections(latt, rho, NULL, 0);
  int* hklp = (int*)malloc(sizeof(int) * 3 * (n > 0 ? n : 1));
  double* ghkl = (double*)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
  oc_permitted_reflections(latt, rho, hklp, n);
  int i000 = 0, ihkl = 0;
  for (int ii = 1; ii <= n; ++ii) {
    int* h = &hklp[3 * (ii - 1)];
    if (h[0] * h[0] + h[1] * h[1] + h[2] * h[2] == 0) i000 = ii;
    int d0 = h[0] - hkl[0], d1 = h[1] - hkl[1], d2 = h[2] - hkl[2];
    if (d0 * d0 + d1 * d1 + d2 * d2 == 0) ihkl = ii;
    double hd[3] = {(double)h[0], (double)h[1], (double)h[2]};
    reflection(B, hd, &ghkl[3 * (ii - 1)]);
  }
  if (i000 != 0) {
    for (int c = 0; c < 3; ++c) {
      double t = ghkl[c];
      ghkl[c] = ghkl[3 * (i000 - 1) + c];
      ghkl[3 * (i000 - 1) + c] = t;
      int u = hklp[c];
      hklp[c] = hklp[3 * (i000 - 1) + c];
      hklp[3 * (i000 - 1) + c] = u;
    }
  }
  if (ihkl != 0) {
    for (int c = 0; c < 3; ++c) {
      double t = ghkl[3 + c];
      ghkl[3 + c] = ghkl[3 * (ihkl - 1) + c];
      ghkl[3 * (ihkl - 1) + c] = t;
      int u = hklp[c];
      hklp[c] = hklp[3 * (ihkl - 1) + c];
      hklp[3 * (ihkl - 1) + c] = u;
    }
  }
  *ghkl_out = ghkl;
  *hklp_out = hklp;
  return n;
}

/* findRotationsForBraggCondition2 (Lib_DiffractionConditions.f90:1382-1515).
 * mode 0: nolimitPhi absent (|phi - phi0| <= THETA_MAX degrees); 1: present and
 * true (no limit); 2: present and false (2 THETA_MAX degrees). */
static int bragg_rotations(double v, const double* g, double cosq, double sinq, double phi0, double theta_max_deg,
                           int mode, double* phi) {
  int nphi = 0;
  double xx = g[1] * sinq + g[2] * cosq;
  double aa = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  aa = -aa * HBAR / (2 * ME * v);
  double uu = g[0] * g[0] + xx * xx;
  double vv = uu - aa * aa;
  if (vv < 0) return 0;
  uu = 1 / uu;
  vv = sqrt(vv) * g[0] * uu;
  uu = aa * xx * uu;
  double lim = mode == 2 ? 2 * theta_max_deg * DEGTORAD : theta_max_deg * DEGTORAD;
  for (int branch = 0; branch < 2; ++branch) {
    double c = branch == 0 ? uu + vv : uu - vv;
    if (fabs(c) <= 1) {
      double pp = acos(c);
      long jj = lround((pp - phi0) / (2 * PI));
      pp = pp - 2 * jj * PI;
      if (mode == 1 || fabs(pp - phi0) <= lim) {
        phi[nphi] = pp;
        phi[nphi + 1] = -pp;
        nphi += 2;
      }
    }
  }
  return nphi;
}

/* findAllEulerAngles (Lib_DiffractionConditions.f90:1565-1625): khat(3, 4 NTHETA). */
static int find_all_euler_angles(double v, const double* g, double theta0, double phi0, double theta_max,
                                 double theta_max_deg, int mode, double* khat) {
  double theta_min = theta0 - theta_max / 2;
  if (!(theta_min > 0.0)) theta_min = 0.0;
  int nk = 0;
  for (int ii = 1; ii <= OC_NTHETA; ++ii) {
    double theta = theta_min + theta_max * ii / OC_NTHETA;
    double cost = cos(theta), sint = sin(theta), phi[4];
    int nphi = bragg_rotations(v, g, cost, sint, phi0, theta_max_deg, mode, phi);
    for (int jj = 0; jj < nphi; ++jj) {
      double pp = phi[jj], cosp = cos(pp), sinp = sin(pp);
      khat[3 * (nk + jj)] = -sinp;
      khat[3 * (nk + jj) + 1] = sint * cosp;
      khat[3 * (nk + jj) + 2] = cost * cosp;
    }
    nk += nphi;
  }
  return nk;
}

/* intensityAtDepthZ (Lib_DiffractionConditions.f90:1209-1259) in the
 * reference's order of operations: (phig * bg) / (2 dd), then |phig|^2. */
static double intensity_exact(double xi0, double xig, double sg, double z) {
  double b0 = PI / xi0, bg = PI / xig, aa = 2 * PI * sg;
  double dd = sqrt(aa * aa / 4 + bg * bg);
  double l1 = (b0 + aa / 2) + dd, l2 = (b0 + aa / 2) - dd;
  double re = cos(l1 * z) - cos(l2 * z), im = sin(l1 * z) - sin(l2 * z);
  re = re * bg / (2 * dd);
  im = im * bg / (2 * dd);
  return re * re + im * im;
}

/* scoreForIncidentVector1 (Lib_DiffractionConditions.f90:1835-1867). */
double oc_score_incident_vector(double v, const double* khat, const double* ghkl, const double* xi_g, int nn,
                                double foil) {
  double s = 0;
  for (int ii = 3; ii <= nn; ++ii) {
    const double* g = &ghkl[3 * (ii - 1)];
    double eps = energy_deviation_parameter(v, khat, g);
    double sg = energy_to_length_sg(v, eps);
    s = s + intensity_exact(xi_g[0], xi_g[ii - 1], sg, foil);
  }
  return s;
}

static int lattice_symmetry(int latt) {
  if (latt == OC_LATTICE_HCP) return OC_SYM_HEX;
  if (latt >= OC_LATTICE_SC && latt <= OC_LATTICE_FCC) return OC_SYM_CUBIC;
  return -1;
}

/* findBestRotationMatrix (Lib_DiffractionConditions.f90:129-357) without the
 * optional near-Bragg list.  scores (optional) receives every incident
 * vector's score, khat (optional) the incident vectors: both 4 NTHETA long. */
int oc_find_best_rotation(double v, const double* z0, const double* A_cell, int latt, const int* hkl,
                          const char* xifile, double foil, double theta_max_deg, double rho_max, double* U,
                          double* R, oc_tilt_info* info, double* scores, double* khat_out) {
  int symm = lattice_symmetry(latt);
  if (symm < 0) return OC_ERR_ARG;
  double BB[9], gg[3], ghkl0[3], hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]};
  reciprocal(A_cell, BB);
  reflection(BB, hd, gg);
  oc_rotate_to_standard_frame(z0, A_cell, hd, U);
  mat_vec(U, gg, ghkl0);
  double* ghkl;
  int* hklp;
  int nn = gvectors_permitted(latt, BB, hkl, rho_max, &ghkl, &hklp);
  double* xi_g = (double*)malloc(sizeof(double) * (nn > 0 ? nn : 1));
  int xi_ok = oc_read_extinction_distances(xifile, hklp, nn, symm, xi_g);
  double* khat = (double*)malloc(sizeof(double) * 3 * 4 * OC_NTHETA);
  int nk = find_all_euler_angles(v, ghkl0, 0.0, 0.0, theta_max_deg * DEGTORAD, theta_max_deg, 0, khat);
  int attempt = 1;
  if (nk == 0) {
    attempt = 2;
    nk = find_all_euler_angles(v, ghkl0, 0.0, 0.0, 2 * theta_max_deg * DEGTORAD, theta_max_deg, 0, khat);
    if (nk == 0) {
      attempt = 3;
      nk = find_all_euler_angles(v, ghkl0, 0.0, 0.0, theta_max_deg * DEGTORAD, theta_max_deg, 1, khat);
    }
  }
  if (nk == 0) {
    free(ghkl);
    free(hklp);
    free(xi_g);
    free(khat);
    return OC_ERR_ARG;
  }
  double ss_best = HUGE1;
  int ii_best = 0;
  for (int ii = 1; ii <= nk; ++ii) {
    double ss = oc_score_incident_vector(v, &khat[3 * (ii - 1)], ghkl, xi_g, nn, foil);
    if (scores) scores[ii - 1] = ss;
    if (ss < ss_best) {
      ss_best = ss;
      ii_best = ii;
    }
  }
  const double* kb = &khat[3 * (ii_best - 1)];
  double phi = -asin(kb[0]);
  double theta = acos(kb[2] / cos(phi));
  A(R, 1, 1) = cos(phi);
  A(R, 1, 2) = sin(theta) * sin(phi);
  A(R, 1, 3) = cos(theta) * sin(phi);
  A(R, 2, 1) = 0.0;
  A(R, 2, 2) = cos(theta);
  A(R, 2, 3) = -sin(theta);
  A(R, 3, 1) = -sin(phi);
  A(R, 3, 2) = sin(theta) * cos(phi);
  A(R, 3, 3) = cos(theta) * cos(phi);
  if (A(R, 3, 3) < 0) {
    for (int i = 1; i <= 3; ++i) {
      A(R, i, 3) = -A(R, i, 3);
      A(R, i, 2) = -A(R, i, 2);
    }
  }
  if (khat_out) memcpy(khat_out, khat, sizeof(double) * 3 * nk);
  if (info) {
    info->nk = nk;
    info->nn = nn;
    info->ii_best = ii_best;
    info->attempt = attempt;
    info->xi_ok = xi_ok;
    info->ss_best = ss_best;
    info->theta = theta;
    info->phi = phi;
  }
  free(ghkl);
  free(hklp);
  free(xi_g);
  free(khat);
  return OC_OK;
}

/* The scoring inputs of findBestRotationMatrix: the permitted g-vectors after both swaps
 * and their extinction distances (Lib_DiffractionConditions.f90:204-214).  Returns nn;
 * the first cap go to ghkl(3, cap) and xi_g(cap). */
int oc_tilt_reflections(int latt, const double* A_cell, const int* hkl, double rho, const char* xifile,
                        double* ghkl_out, double* xi_out, int cap) {
  int symm = lattice_symmetry(latt);
  if (symm < 0) return -1;
  double BB[9];
  reciprocal(A_cell, BB);
  double* ghkl;
  int* hklp;
  int nn = gvectors_permitted(latt, BB, hkl, rho, &ghkl, &hklp);
  double* xi_g = (double*)malloc(sizeof(double) * (nn > 0 ? nn : 1));
  oc_read_extinction_distances(xifile, hklp, nn, symm, xi_g);
  for (int i = 0; i < nn && i < cap; ++i) {
    memcpy(&ghkl_out[3 * i], &ghkl[3 * i], 3 * sizeof(double));
    xi_out[i] = xi_g[i];
  }
  free(ghkl);
  free(hklp);
  free(xi_g);
  return nn;
}

/* GoldenSection (Lib_GoldenSection.f90:41-52, 126-150, 152-264, 266-306, 308-381). */
typedef struct {
  double x1, x2, x3, y1, y2, y3;
  int bounded, step;
  double xtol, ytol;
} oc_gold;

static const double GOLD_TOL = 1.0e-6, GOLD_MINSTEP = 50, GOLD_BOUNDSTEP = 10;

static double gold_ratio(void) { return (1 + sqrt(5.0)) / 2; }

static void gold_ctor(oc_gold* g, double x1, double x3, double y1, double y3) {
  if (x1 < x3) {
    g->x1 = x1; g->x3 = x3; g->y1 = y1; g->y3 = y3;
  } else {
    g->x3 = x3; g->x1 = x1; g->y3 = y3; g->y1 = y1;
  }
  g->x2 = 0.0;
  g->y2 = HUGE1;
  g->step = 0;
  g->bounded = 0;
  g->xtol = (g->x3 - g->x1) * GOLD_TOL;
  double dy = fabs(g->y3 - g->y1);
  g->ytol = (GOLD_TOL > dy ? GOLD_TOL : dy) * GOLD_TOL;
}

static void gold_check_bounds(oc_gold* g, double xt, double yt) {
  if (g->step == 1) {
    double m = g->y1 < g->y3 ? g->y1 : g->y3;
    if (yt < m) {
      g->bounded = 1; g->x2 = xt; g->y2 = yt;
    } else if (yt > g->y1 && g->y1 > g->y3) {
      g->bounded = 0; g->x1 = xt; g->y1 = yt;
    } else if (yt > g->y3 && g->y3 > g->y1) {
      g->bounded = 0; g->x3 = xt; g->y3 = yt;
    } else if (g->y1 > yt && yt > g->y3) {
      g->bounded = 0; g->x1 = xt; g->y1 = yt;
    } else if (g->y3 > yt && yt > g->y1) {
      g->bounded = 0; g->x3 = xt; g->y3 = yt;
    }
    return;
  }
  if (g->y1 < g->y3) {
    g->bounded = !(yt < g->y1);
    g->x2 = g->x1; g->x1 = xt; g->y2 = g->y1; g->y1 = yt;
  } else {
    g->bounded = !(yt < g->y3);
    g->x2 = g->x3; g->x3 = xt; g->y2 = g->y3; g->y3 = yt;
  }
}

static double gold_next_point(const oc_gold* g) {
  const double GOLD = gold_ratio();
  if (!g->bounded) {
    if (g->step == 0) return g->x1 + (g->x3 - g->x1) * (GOLD - 1);
    if (g->y1 < g->y3) return g->x1 - (g->x3 - g->x1) / GOLD;
    return g->x3 + (g->x3 - g->x1) / GOLD;
  }
  return g->x1 + (g->x3 - g->x2);
}

static void gold_minimise(oc_gold* g, double* xt, double* yt, int* is, int* ok) {
  g->step = g->step + 1;
  if (!g->bounded) {
    gold_check_bounds(g, *xt, *yt);
    *is = 0;
    *ok = g->bounded || (g->step <= GOLD_BOUNDSTEP);
    return;
  }
  *is = 0;
  *ok = g->step <= GOLD_MINSTEP;
  if (!*ok) return;
  if (*yt < g->y2) {
    if (*xt < g->x2) {
      g->x3 = g->x2; g->y3 = g->y2; g->x2 = *xt; g->y2 = *yt;
    } else {
      g->x1 = g->x2; g->y1 = g->y2; g->x2 = *xt; g->y2 = *yt;
    }
  } else {
    if (*xt > g->x2) {
      g->x3 = *xt; g->y3 = *yt;
    } else {
      g->x1 = *xt; g->y1 = *yt;
    }
  }
  double ym = g->y1 > g->y3 ? g->y1 : g->y3;
  *is = (fabs(g->x3 - g->x1) < g->xtol) || (fabs(g->y2 - ym) < g->ytol);
  if (*is) {
    *xt = g->x2;
    *yt = g->y2;
  }
}

/* The search loop of tiltToDarkField / testLib_GoldenSection.f90 on any function:
 * nextPoint, f, minimise until converged or out of steps; returns the number of steps. */
int oc_golden_minimise(double x1, double x3, double (*f)(double, void*), void* arg, double* xt, double* yt) {
  oc_gold gold;
  gold_ctor(&gold, x1, x3, f(x1, arg), f(x3, arg));
  double x2 = 0.0, y2 = 0.0;
  int conv = 0, ok = 1;
  while (1) {
    x2 = gold_next_point(&gold);
    y2 = f(x2, arg);
    gold_minimise(&gold, &x2, &y2, &conv, &ok);
    if (conv || !ok) break;
  }
  *xt = x2;
  *yt = y2;
  return conv ? gold.step : -gold.step;
}

/* |phi_g(L')|^2 after a tilt x about y (Lib_DiffractionConditions.f90:831-859). */
static double dark_field_intensity(double x, const double* gg, double bg, double foil) {
  double cost = cos(x), sint = sin(x);
  double Lp = foil / cost;
  double sgp = (sint * gg[0] - cost * gg[2]) / (2 * PI);
  double s = bg * sin(PI * sqrt(sgp * sgp + bg * bg) * Lp);
  return s * s / (sgp * sgp + bg * bg);
}

/* tiltToDarkField (Lib_DiffractionConditions.f90:751-927): R <- Ry(theta) R. */
int oc_tilt_to_dark_field(double v, const double* A_cell, const int* hkl, double xi0, double xig, double foil,
                          double theta_max_deg, const double* U, double* R, double* theta_out) {
  (void)xi0;
  double BB[9], kk[3], RU[9], gg[3], hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]};
  reciprocal(A_cell, BB);
  reflection(BB, hd, kk);
  mat_mul(R, U, RU);
  mat_vec(RU, kk, gg);
  double bg = 1 / xig;
  const double kz[3] = {0.0, 0.0, 1.0};
  double uu = energy_deviation_parameter(v, kz, gg);
  double sg = energy_to_length_sg(v, uu);
  double s0 = bg * sin(PI * sqrt(sg * sg + bg * bg) * foil);
  double phiL2 = s0 * s0 / (sg * sg + bg * bg);
  double x1 = -(theta_max_deg * 0.01 * DEGTORAD), x3 = +(theta_max_deg * 0.01 * DEGTORAD);
  double y1 = dark_field_intensity(x1, gg, bg, foil), y3 = dark_field_intensity(x3, gg, bg, foil);
  oc_gold gold;
  gold_ctor(&gold, x1, x3, y1, y3);
  double x2, y2;
  for (;;) {
    x2 = gold_next_point(&gold);
    y2 = dark_field_intensity(x2, gg, bg, foil);
    int conv, ok;
    gold_minimise(&gold, &x2, &y2, &conv, &ok);
    if (conv) break;
    if (!ok) break;
  }
  double theta, cost, sint;
  if (y2 < phiL2) {
    theta = x2; cost = cos(x2); sint = sin(x2);
  } else {
    theta = 0.0; cost = 1.0; sint = 0.0;
  }
  double RR[9];
  A(RR, 1, 1) = cost; A(RR, 1, 2) = 0.0; A(RR, 1, 3) = sint;
  A(RR, 2, 1) = 0.0;  A(RR, 2, 2) = 1.0; A(RR, 2, 3) = 0.0;
  A(RR, 3, 1) = -sint; A(RR, 3, 2) = 0.0; A(RR, 3, 3) = cost;
  mat_mul(RR, R, R);
  if (theta_out) *theta_out = theta;
  return OC_OK;
}

/* The eigenvector of the largest eigenvalue of a symmetric 4x4 matrix by cyclic
 * Jacobi rotations.  RotMatToQuaternion calls LAPACK DSYEV for this step; the
 * largest eigenvalue of its K matrix is isolated (3 against -1, -1, -1 for a
 * rotation), so any accurate method gives the same unit vector up to sign and
 * rounding. */
static void top_eigenvector4(const double* K_in, double* vec) {
  double a[16], V[16];
  memcpy(a, K_in, sizeof a);
  for (int i = 0; i < 16; ++i) V[i] = (i % 5 == 0) ? 1.0 : 0.0;
#define M4(m, i, j) ((m)[(i) + 4 * (j)])
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) off += M4(a, p, q) * M4(a, p, q);
    if (off == 0.0) break;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) {
        double apq = M4(a, p, q);
        if (apq == 0.0) continue;
        double th = (M4(a, q, q) - M4(a, p, p)) / (2 * apq);
        double t = fabs(th) > 1.0e150 ? 0.5 / th : (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 4; ++k) {
          double akp = M4(a, k, p), akq = M4(a, k, q);
          M4(a, k, p) = c * akp - s * akq;
          M4(a, k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          double apk = M4(a, p, k), aqk = M4(a, q, k);
          M4(a, p, k) = c * apk - s * aqk;
          M4(a, q, k) = s * apk + c * aqk;
        }
        M4(a, p, q) = 0.0;
        M4(a, q, p) = 0.0;
        for (int k = 0; k < 4; ++k) {
          double vkp = M4(V, k, p), vkq = M4(V, k, q);
          M4(V, k, p) = c * vkp - s * vkq;
          M4(V, k, q) = s * vkp + c * vkq;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < 4; ++i)
    if (M4(a, i, i) >= M4(a, best, best)) best = i;
  for (int k = 0; k < 4; ++k) vec[k] = M4(V, k, best);
#undef M4
}

/* RotMatToQuaternion (Lib_Quaternions.f90:246-288): q = (w, x, y, z). */
void oc_rotmat_to_quaternion(const double* R, double* q) {
  double K[16] = {0};
#define K4(i, j) K[((i)-1) + 4 * ((j)-1)]
  K4(1, 1) = A(R, 1, 1) - A(R, 2, 2) - A(R, 3, 3);
  K4(2, 1) = A(R, 2, 1) + A(R, 1, 2);
  K4(3, 1) = A(R, 3, 1) + A(R, 1, 3);
  K4(4, 1) = A(R, 2, 3) - A(R, 3, 2);
  K4(2, 2) = A(R, 2, 2) - A(R, 1, 1) - A(R, 3, 3);
  K4(3, 2) = A(R, 3, 2) + A(R, 2, 3);
  K4(4, 2) = A(R, 3, 1) - A(R, 1, 3);
  K4(3, 3) = A(R, 3, 3) - A(R, 1, 1) - A(R, 2, 2);
  K4(4, 3) = A(R, 1, 2) - A(R, 2, 1);
  K4(4, 4) = A(R, 1, 1) + A(R, 2, 2) + A(R, 3, 3);
  for (int j = 1; j <= 4; ++j)
    for (int i = 1; i < j; ++i) K4(i, j) = K4(j, i); /* DSYEV reads the lower triangle */
#undef K4
  double v[4];
  top_eigenvector4(K, v);
  if (v[3] > 0)
    for (int k = 0; k < 4; ++k) v[k] = -v[k];
  q[1] = v[0];
  q[2] = v[1];
  q[3] = v[2];
  q[0] = -v[3];
}

/* quaternionToRotMat (Lib_Quaternions.f90:290-321). */
void oc_quaternion_to_rotmat(const double* q, double* R) {
  double w = q[0], x = q[1], y = q[2], z = q[3];
  double ss = (x * x + y * y + z * z + w * w) / 2;
  A(R, 1, 1) = ss - (y * y + z * z);
  A(R, 2, 1) = (x * y + z * w);
  A(R, 3, 1) = (x * z - y * w);
  A(R, 1, 2) = (x * y - z * w);
  A(R, 2, 2) = ss - (x * x + z * z);
  A(R, 3, 2) = (y * z + x * w);
  A(R, 1, 3) = (x * z + y * w);
  A(R, 2, 3) = (y * z - x * w);
  A(R, 3, 3) = ss - (x * x + y * y);
  ss = 1 / ss;
  for (int i = 0; i < 9; ++i) R[i] = R[i] * ss;
}

/* normalise0 (Lib_Quaternions.f90:203-219). */
static void quaternion_normalise(double* q) {
  double tt = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (tt == 0) {
    q[0] = 1.0;
    q[1] = q[2] = q[3] = 0.0;
    return;
  }
  tt = 1 / sqrt(tt);
  for (int k = 0; k < 4; ++k) q[k] = q[k] * tt;
}

/* slerp (Lib_Quaternions.f90:526-564) with midpoint (:504-524). */
void oc_slerp(const double* q1, const double* q2, double x, double* qx) {
  double x1 = q1[0] * q2[0] + q1[1] * q2[1] + q1[2] * q2[2] + q1[3] * q2[3];
  if (x1 >= 1.0) {
    memcpy(qx, q1, 4 * sizeof(double));
    return;
  }
  if (x1 <= -1.0) {
    for (int k = 0; k < 4; ++k) qx[k] = q1[k] + q2[k];
    double dd = qx[0] * qx[0] + qx[1] * qx[1] + qx[2] * qx[2] + qx[3] * qx[3];
    if (dd > 0) {
      dd = 1 / sqrt(dd);
      for (int k = 0; k < 4; ++k) qx[k] = qx[k] * dd;
    }
    return;
  }
  double x2 = 2 * x1 * x1 - 1;
  double omega = acos(x2);
  x2 = 1 / sin(omega);
  x1 = sin((1 - x) * omega) * x2;
  x2 = sin(x * omega) * x2;
  for (int k = 0; k < 4; ++k) qx[k] = x1 * q1[k] + x2 * q2[k];
  quaternion_normalise(qx);
}

/* findFoilThickness (Lib_DynamicalTwoBeamImaging.f90:486-564): the mean and
 * spread of the foil thickness over columns of about 3 a0.  Returns the
 * number of columns holding atoms; d receives the cuboid sides. */
static int find_foil_thickness(oc_d2bi* t, const double* x, int64_t ldx, int64_t nAtoms, const double* RU,
                               double* d, double* zbar_out, double* zsig_out, int* Nx_out, int* Ny_out) {
  double dd[3], D[9], a_sup[9];
  memcpy(dd, t->voxelSupercellDimensions, sizeof dd);
  super_a(&t->super, a_sup);
  find_transformed_supercell(a_sup, RU, D, t->delta, t->uvw, &t->nuvw, dd);
  dd[0] = A(D, 1, 1);
  dd[1] = A(D, 2, 2);
  dd[2] = A(D, 3, 3);
  memcpy(d, dd, sizeof dd);
  int Nx = (int)lround(dd[0] / (3 * t->a0)), Ny = (int)lround(dd[1] / (3 * t->a0));
  if (Nx < 1) Nx = 1;
  if (Ny < 1) Ny = 1;
  dd[0] = Nx / dd[0];
  dd[1] = Ny / dd[1];
  double id3 = 1 / dd[2];
  double* top = (double*)malloc(sizeof(double) * Nx * Ny);
  double* thick = (double*)malloc(sizeof(double) * Nx * Ny);
  for (int i = 0; i < Nx * Ny; ++i) {
    top[i] = HUGE1;
    thick[i] = -HUGE1;
  }
  for (int nn = 0; nn < t->nuvw; ++nn) {
    double Ruvw[3];
    for (int i = 1; i <= 3; ++i)
      Ruvw[i - 1] = t->uvw[3 * nn] * (A(t->super.a, i, 1) * t->super.Nx) +
                    t->uvw[3 * nn + 1] * (A(t->super.a, i, 2) * t->super.Ny) +
                    t->uvw[3 * nn + 2] * (A(t->super.a, i, 3) * t->super.Nz);
    for (int64_t ii = 0; ii < nAtoms; ++ii) {
      double xx[3];
      for (int c = 0; c < 3; ++c) xx[c] = x[ii * ldx + c] + Ruvw[c];
      mat_vec(RU, xx, xx);
      for (int c = 0; c < 3; ++c) xx[c] = xx[c] + t->delta[c];
      int ix = (int)floor(dd[0] * xx[0]);
      if ((long long)ix * (Nx - 1 - ix) < 0) continue;
      int iy = (int)floor(dd[1] * xx[1]);
      if ((long long)iy * (Ny - 1 - iy) < 0) continue;
      int iz = (int)floor(id3 * xx[2]);
      if (iz != 0) continue;
      size_t c = (size_t)ix + (size_t)Nx * iy;
      if (xx[2] < top[c]) top[c] = xx[2];
      if (xx[2] > thick[c]) thick[c] = xx[2];
    }
  }
  double zbar = 0.0, z2bar = 0.0;
  int nn = 0;
  for (int iy = 0; iy < Ny; ++iy)
    for (int ix = 0; ix < Nx; ++ix) {
      size_t c = (size_t)ix + (size_t)Nx * iy;
      double th = thick[c] > top[c] ? thick[c] - top[c] : 0.0;
      if (th == 0) continue;
      zbar = zbar + th;
      z2bar = z2bar + th * th;
      nn = nn + 1;
    }
  zbar = zbar / nn;
  z2bar = z2bar / nn;
  z2bar = z2bar - zbar * zbar;
  z2bar = sqrt(z2bar > 0.0 ? z2bar : 0.0);
  *zbar_out = zbar;
  *zsig_out = z2bar;
  *Nx_out = Nx;
  *Ny_out = Ny;
  free(top);
  free(thick);
  return nn;
}

/* setSupercellTilt1 (Lib_DynamicalTwoBeamImaging.f90:795-939) for integer ng;
 * x may be NULL (foil thickness from the box). */
static int set_supercell_tilt1(oc_d2bi* t, int ng, const char* xifile, int latt, double theta_max_deg,
                               double rho_max, const double* x, int64_t ldx, int64_t nAtoms, oc_tilt_info* info) {
  int hkl[3];
  for (int i = 0; i < 3; ++i) hkl[i] = (int)lround(ng * t->g[i]);
  double zbar;
  if (x) {
    double hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]}, dd[3], zsig;
    int Nx, Ny;
    oc_rotate_to_standard_frame(t->k, t->a_cell, hd, t->U);
    find_foil_thickness(t, x, ldx, nAtoms, t->U, dd, &zbar, &zsig, &Nx, &Ny);
    if (zbar + 2 * t->a0 > dd[2]) zbar = dd[2];
    if (info) info->foil_sigma = zsig;
  } else {
    zbar = t->voxelSupercellDimensions[2];
  }
  t->foilThickness = zbar;
  double vv = oc_velocity(t->E * 1000);
  double z = fabs(t->foilThickness);
  int rc = oc_find_best_rotation(vv, t->k, t->a_cell, latt, hkl, xifile, z, theta_max_deg, rho_max, t->U, t->R,
                                 info, NULL, NULL);
  if (rc != OC_OK) return rc;
  z = fabs(t->foilThickness / A(t->R, 3, 3));
  int g_int[3] = {(int)lround(t->g[0]), (int)lround(t->g[1]), (int)lround(t->g[2])};
  double theta;
  oc_tilt_to_dark_field(oc_velocity(t->E * 1000), t->a_cell, g_int, t->xi0, t->xig, z, theta_max_deg, t->U, t->R,
                        &theta);
  if (info) {
    info->foil = t->foilThickness;
    info->dark_theta = theta;
  }
  t->voxelSupercellDimensions[2] = fabs(t->voxelSupercellDimensions[2] / A(t->R, 3, 3));
  double RU[9], a_sup[9], D[9], gg[3];
  mat_mul(t->R, t->U, RU);
  super_a(&t->super, a_sup);
  find_transformed_supercell(a_sup, RU, D, t->delta, t->uvw, &t->nuvw, t->voxelSupercellDimensions);
  build_gksuper(t, D);
  oc_get_aperture(t, NULL, gg);
  t->sg = oc_get_deviation_parameter(t, gg);
  return OC_OK;
}

/* setSupercellTilt1a (Lib_DynamicalTwoBeamImaging.f90:943-1045). */
int oc_set_supercell_tilt1a(oc_d2bi* t, double ng, const char* xifile, int latt, double theta_max_deg,
                            double rho_max, const double* x, int64_t ldx, int64_t nAtoms, oc_tilt_info* info) {
  double dd[3], q1[4], q2[4], q[4];
  memcpy(dd, t->voxelSupercellDimensions, sizeof dd);
  int rc = set_supercell_tilt1(t, (int)floor(ng), xifile, latt, theta_max_deg, rho_max, x, ldx, nAtoms, info);
  if (rc != OC_OK) return rc;
  oc_rotmat_to_quaternion(t->R, q1);
  if (ng - floor(ng) > 1.0e-4) {
    memcpy(t->voxelSupercellDimensions, dd, sizeof dd);
    rc = set_supercell_tilt1(t, (int)ceil(ng), xifile, latt, theta_max_deg, rho_max, x, ldx, nAtoms, NULL);
    if (rc != OC_OK) return rc;
    oc_rotmat_to_quaternion(t->R, q2);
  } else {
    memcpy(q2, q1, sizeof q1);
  }
  oc_slerp(q1, q2, ng - floor(ng), q);
  oc_quaternion_to_rotmat(q, t->R);
  t->voxelSupercellDimensions[2] = fabs(dd[2] / A(t->R, 3, 3));
  double RU[9], a_sup[9], D[9], gg[3];
  mat_mul(t->R, t->U, RU);
  super_a(&t->super, a_sup);
  find_transformed_supercell(a_sup, RU, D, t->delta, t->uvw, &t->nuvw, t->voxelSupercellDimensions);
  build_gksuper(t, D);
  oc_get_aperture(t, NULL, gg);
  t->sg = oc_get_deviation_parameter(t, gg);
  return OC_OK;
}

/* ------------------------------------------------------------------------ */
/* The .xyz reader (Lib_XYZFiles.f90 readHeader, getSupercell0, input0)       */
/* ------------------------------------------------------------------------ */

/* gfortran's real ** integer (libgcc __powidf2). */
static double oc_powi(double x, int m) {
  unsigned n = m < 0 ? 0u - (unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1 / y : y;
}

static int is_number_char(char c) { return (c >= '0' && c <= '9') || (c && strchr(".+-eEdD", c) != NULL); }

/* Fortran s(a:b) of a C string of length n into out (cap 33): empty when b < a;
 * character(len=32) keeps 32. */
static void fort_substr(const char* s, int n, int a, int b, char* out) {
  int k = 0;
  if (a < 1) a = 1;
  if (b > n) b = n;
  for (int i = a; i <= b && k < 32; ++i) out[k++] = s[i - 1];
  out[k] = 0;
}

/* ParseReal (NBAX_StringTokenizers.f90:303-420) of text[0..len). */
int oc_fortran_parse_real(const char* text, int len, double* r) {
  char str[65];
  int n = 0, in_num = 0;
  for (int i = 0; i < len; ++i) {
    char c = text[i];
    if (!in_num && c == ' ') continue;
    if (!is_number_char(c)) break;
    in_num = 1;
    str[n++] = c;
    if (n == 64) break;
  }
  str[n] = 0;
  if (n == 0) return 0;
  for (int i = 0; i < n; ++i)
    if (str[i] == 'd' || str[i] == 'D' || str[i] == 'E') str[i] = 'e';
  char* pd = strchr(str, '.');
  char* pe = strchr(str, 'e');
  int ii = pd ? (int)(pd - str) + 1 : 0, jj = pe ? (int)(pe - str) + 1 : 0;
  char a[33] = "0", b[33] = "0", c[33] = "0";
  if (ii == 1) {
    if (jj > 1) {
      fort_substr(str, n, 2, jj - 1, b);
      fort_substr(str, n, jj + 1, n, c);
    } else {
      fort_substr(str, n, 2, n, b);
    }
  } else if (ii > 1) {
    fort_substr(str, n, 1, ii - 1, a);
    if (jj > 1) {
      fort_substr(str, n, ii + 1, jj - 1, b);
      fort_substr(str, n, jj + 1, n, c);
    } else {
      fort_substr(str, n, ii + 1, n, b);
    }
  } else {
    if (jj > 1) {
      fort_substr(str, n, 1, jj - 1, a);
      fort_substr(str, n, jj + 1, n, c);
    } else {
      fort_substr(str, n, 1, n, a);
    }
  }
  double xa = 0.0;
  for (char* q = a; *q; ++q) {
    int d = *q - '0';
    if (d >= 0 && d <= 9) xa = xa * 10 + d;
  }
  int ic = 0;
  for (char* q = c; *q; ++q) {
    int d = *q - '0';
    if (d >= 0 && d <= 9) ic = ic * 10 + d;
  }
  if (c[0] == '-') ic = -ic;
  double xx = 1.0, xb = 0.0;
  for (char* q = b; *q; ++q) {
    xx = xx * 0.1;
    xb = xb + xx * (*q - '0');
  }
  double rr = (xa + xb) * oc_powi(10.0, ic);
  if (a[0] == '-') rr = -rr;
  if (fabs(rr) == 0) rr = 0;
  *r = rr;
  return 1;
}

static int ltrim_len(const char* s) { /* len_trim */
  int k = (int)strlen(s);
  while (k > 0 && s[k - 1] == ' ') --k;
  return k;
}

/* StringTokenizer over buf (modified in place; blank padded to its length kk). */
typedef struct {
  char buf[1025];
  const char* delims;
  int ndelims;
  int max_tok;
} oc_tok;

static void tok_init(oc_tok* t, const char* s, const char* delims, int ndelims, int max_tok) {
  int n = ltrim_len(s);
  if (n > 1024) n = 1024;
  memcpy(t->buf, s, (size_t)n);
  t->buf[n] = 0;
  t->delims = delims;
  t->ndelims = ndelims;
  t->max_tok = max_tok;
}

static int tok_more(const oc_tok* t) { return ltrim_len(t->buf) > 0; }

static int is_delim(const oc_tok* t, char c) {
  for (int i = 0; i < t->ndelims; ++i)
    if (t->delims[i] == c) return 1;
  return 0;
}

static void tok_next(oc_tok* t, char* out) {
  for (;;) {
    int kk = ltrim_len(t->buf);
    out[0] = 0;
    if (kk == 0) return;
    int jj = kk + 1;
    for (int p = 0; p < kk; ++p)
      if (is_delim(t, t->buf[p])) {
        jj = p + 1;
        break;
      }
    int i = jj - 1 < t->max_tok ? jj - 1 : t->max_tok;
    if (i < 0) i = 0;
    memcpy(out, t->buf, (size_t)i);
    out[i] = 0;
    char rest[1025];
    int m = 0;
    for (int p = jj; p < kk; ++p) rest[m++] = t->buf[p];
    while (m < kk) rest[m++] = ' ';
    rest[kk] = 0;
    memcpy(t->buf, rest, (size_t)kk + 1);
    if (i > 0) return;
  }
}

/* ParseRealArray1 (NBAX_StringTokenizers.f90:273-300). */
static int parse_real_array(const char* s, double* ra, int cap) {
  static const char delims[6] = {' ', ',', ';', '\t', '\r', '\0'};
  oc_tok t;
  char tmp[1025];
  int n = ltrim_len(s);
  if (n > 1024) n = 1024;
  memcpy(tmp, s, (size_t)n);
  tmp[n] = 0;
  tok_init(&t, tmp, delims, 6, 32);
  int cnt = 0;
  for (int k = 0; k < 1000000 && tok_more(&t); ++k) {
    char tok[33];
    tok_next(&t, tok);
    double r;
    if (oc_fortran_parse_real(tok, (int)strlen(tok), &r)) {
      ra[cnt++] = r;
      if (cnt == cap) break;
    }
  }
  return cnt;
}

/* parseInt (NBAX_StringTokenizers.f90:534-564). */
static int fortran_parse_int(const char* s, long long* v) {
  long long ii = 0;
  int started = 0, neg = 0;
  int n = ltrim_len(s);
  for (int k = 0; k < n; ++k) {
    char c = s[k];
    if (c >= '0' && c <= '9') {
      ii = ii * 10 + (c - '0');
      started = 1;
    } else if (started) {
      break;
    } else if (c == '-') {
      neg = 1;
    }
  }
  if (started) *v = neg ? -ii : ii;
  return started;
}

/* one record of at most cap - 1 characters (the rest of a longer line is skipped),
 * without its newline or a trailing CR; offset advanced by the bytes consumed */
static int read_record(FILE* f, char* out, int cap, long long* offset) {
  int c, n = 0, any = 0;
  while ((c = fgetc(f)) != EOF) {
    any = 1;
    ++*offset;
    if (c == '\n') break;
    if (n < cap - 1) out[n++] = (char)c;
  }
  if (n > 0 && out[n - 1] == '\r') --n;
  out[n] = 0;
  return any;
}

static const char* skip_spaces(const char* s) {
  while (*s == ' ') ++s;
  return s;
}

/* readHeader (Lib_XYZFiles.f90:507-626) and getSupercell0 (:905-1058) for a non-LAMMPS file. */
int oc_xyz_header(const char* path, oc_xyz_info* info) {
  memset(info, 0, sizeof *info);
  for (int i = 0; i < 9; ++i) info->a_super[i] = (i % 4 == 0) ? 1.0 : 0.0;
  info->repeats[0] = info->repeats[1] = info->repeats[2] = 1;
  info->n_read = -1;
  FILE* f = fopen(path, "rb");
  if (!f) return OC_ERR_ARG;
  static char line[4097];
  long long off = 0;
  if (!read_record(f, line, 257, &off)) {
    fclose(f);
    return OC_ERR_ARG;
  }
  if (strncmp(skip_spaces(line), "LAMMPS", 6) == 0) {
    fclose(f);
    info->lammps = 1;
    return OC_OK;
  }
  rewind(f);
  off = 0;
  char count[257] = "";
  int found = 0, nh = 0;
  for (int ii = 0; ii < 1000 && read_record(f, line, 257, &off); ++ii) {
    const char* d = skip_spaces(line);
    if (*d == '#' || *d == '%' || *d == '!') {
      ++nh;
      continue;
    }
    size_t nd = strlen(d) < sizeof count - 1 ? strlen(d) : sizeof count - 1;
    memcpy(count, d, nd);
    count[nd] = 0;
    found = 1;
    break;
  }
  char desc[257] = "";
  int ok = found && read_record(f, desc, 257, &off);
  info->data_offset = off;
  ok = ok && read_record(f, line, 4097, &off);
  fseek(f, 0, SEEK_END);
  info->file_bytes = ftell(f);
  if (!ok) {
    fclose(f);
    return OC_ERR_ARG;
  }
  /* the count: the first blank-delimited token through parseInt */
  oc_tok ct;
  char tok[1025];
  tok_init(&ct, count, " ", 1, 256);
  tok_next(&ct, tok);
  long long na;
  if (!fortran_parse_int(tok, &na)) {
    fclose(f);
    return OC_ERR_ARG;
  }
  /* input0's list-directed integer read of the same line */
  {
    const char* p = count;
    while (*p == ' ' || *p == '\t') ++p;
    const char* q = p;
    while (*q && *q != ' ' && *q != '\t' && *q != ',' && *q != '/') ++q;
    int good = q > p;
    const char* d = p;
    if (good && (*d == '+' || *d == '-')) ++d;
    good = good && d < q;
    for (const char* e = d; e < q && good; ++e) good = *e >= '0' && *e <= '9';
    info->n_read = good ? strtoll(p, NULL, 10) : -1;
  }
  /* the first atom line: the species, then the numbers of the rest */
  oc_tok ft;
  tok_init(&ft, line, " ", 1, 256);
  tok_next(&ft, tok);
  double dat[1000];
  int nc = parse_real_array(ft.buf, dat, 1000);
  if (nc < 3) {
    fclose(f);
    return OC_ERR_ARG;
  }
  info->n_atoms = na;
  info->n_columns = nc;
  info->n_header_lines = nh;
  snprintf(info->column_description, sizeof info->column_description, "%s", desc);
  /* getSupercell0 */
  double* a = info->a_super;
  double v[9];
  char dt[257];
  snprintf(dt, sizeof dt, "%s", desc);
  dt[ltrim_len(dt)] = 0;
  const char* p;
  if ((p = strstr(dt, "Lattice=\"")) != NULL) {
    info->supercell_kind = 1;
    int n = parse_real_array(desc + (p - dt) + 9, v, 9);
    if (n == 3) {
      a[0] = v[0];
      a[4] = v[1];
      a[8] = v[2];
      info->supercell_ok = 1;
    } else if (n == 9) {
      memcpy(a, v, sizeof v);
      info->supercell_ok = 1;
    }
  } else if ((p = strstr(dt, "boxsize")) != NULL) {
    info->supercell_kind = 2;
    int n = parse_real_array(desc + (p - dt) + 8, v, 9);
    if (n >= 3) {
      a[0] = v[0];
      a[4] = v[1];
      a[8] = v[2];
      info->supercell_ok = 1;
    }
  } else {
    rewind(f);
    off = 0;
    for (int ii = 0; ii < nh; ++ii) {
      char d[257];
      read_record(f, d, 257, &off);
      const char* j1 = strstr(d, "supercell");
      const char* j2 = strstr(d, "super cell");
      long long jj1 = j1 ? (j1 - d) + 1 : 0, jj2 = j2 ? (j2 - d) + 1 : 0;
      long long jj = jj1 > jj2 ? jj1 : jj2;
      if (jj == 0) continue;
      info->supercell_kind = 3;
      double xm[3] = {1.0, 1.0, 1.0};
      int n = (long long)strlen(d) >= jj + 8 ? parse_real_array(d + jj + 8, v, 9) : 0;
      if (n == 3) {
        xm[0] = v[0];
        xm[1] = v[1];
        xm[2] = v[2];
      }
      int rp[3];
      for (int k = 0; k < 3; ++k) rp[k] = (int)lround(xm[k]);
      for (int kk = 0; kk < 3; ++kk) {
        char v3[257];
        read_record(f, v3, 257, &off);
        int m = strlen(v3) > 2 ? parse_real_array(v3 + 2, v, 9) : 0;
        if (m == 3) {
          for (int j = 0; j < 3; ++j) a[kk + 3 * j] = v[j];
          if (kk == 2) {
            info->supercell_ok = 1;
            break;
          }
        } else if (m == 9) {
          memcpy(a, v, sizeof v);
          info->supercell_ok = 1;
          break;
        } else {
          break;
        }
      }
      if (info->supercell_ok)
        for (int j = 0; j < 3; ++j) {
          for (int i = 0; i < 3; ++i) a[i + 3 * j] = a[i + 3 * j] * rp[j];
          info->repeats[j] = rp[j];
        }
      break;
    }
  }
  fclose(f);
  return OC_OK;
}

/* input0 (Lib_XYZFiles.f90:756-892): n lines from byte offset `offset`, each read as
 * `atom, dat(1:ncols)` (strtod-rounded); x(ldx, n) receives the first min(ldx, ncols)
 * values; types the species numbers in order of first appearance; names (6 characters
 * each, blank padded, cap names) the species.  Returns the number of species, or
 * -(1 + the 0-based line) that does not read. */
long long oc_read_xyz_atoms(const char* path, long long offset, long long n, int ncols, double* x, int ldx,
                            int* types, char* names, int cap) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  fseek(f, offset, SEEK_SET);
  size_t lcap = 1 << 16;
  char* line = (char*)malloc(lcap);
  char (*tab)[7] = (char (*)[7])calloc(1001, 7);
  int ns = 0;
  long long rc = 0;
  int ncopy = ldx < ncols ? ldx : ncols;
  for (long long i = 0; i < n; ++i) {
    if (!fgets(line, (int)lcap, f)) {
      rc = -(i + 1);
      break;
    }
    char* p = line;
    while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r') ++p;
    char* q = p;
    while (*q && *q != ' ' && *q != '\t' && *q != ',' && *q != '\r' && *q != '\n' && *q != '/') ++q;
    if (q == p || *p == '\'' || *p == '"') {
      rc = -(i + 1);
      break;
    }
    char name[7] = "      ";
    for (int k = 0; k < 6 && p + k < q; ++k) name[k] = p[k];
    p = q;
    int bad = 0;
    for (int c = 0; c < ncols; ++c) {
      while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r') ++p;
      char* e;
      char buf[128];
      int m = 0;
      while (p[m] && p[m] != ' ' && p[m] != '\t' && p[m] != ',' && p[m] != '\r' && p[m] != '\n' && m < 127) {
        buf[m] = (p[m] == 'd' || p[m] == 'D') ? 'E' : p[m];
        ++m;
      }
      buf[m] = 0;
      double v = strtod(buf, &e);
      if (m == 0 || *e) {
        bad = 1;
        break;
      }
      if (c < ncopy) x[i * ldx + c] = v;
      p += m;
    }
    if (bad) {
      rc = -(i + 1);
      break;
    }
    int id = -1;
    for (int k = 0; k < ns; ++k)
      if (memcmp(tab[k], name, 6) == 0) {
        id = k;
        break;
      }
    if (id < 0) {
      if (ns == 1000) {
        rc = -(i + 1);
        break;
      }
      memcpy(tab[ns], name, 7);
      id = ns++;
    }
    if (types) types[i] = id + 1;
  }
  if (rc == 0) {
    rc = ns;
    for (int k = 0; k < ns && k < cap; ++k) memcpy(names + 6 * k, tab[k], 6);
  }
  free(line);
  free(tab);
  fclose(f);
  return rc;
}
