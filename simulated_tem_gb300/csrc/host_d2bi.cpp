// Host mirror of the reference's Fortran set-up of one image.
//
// C++ restatement of the DynamicalTwoBeamImaging type (src/
// Lib_DynamicalTwoBeamImaging.f90) and the helpers it uses from
// Lib_SimpleSupercells.f90, Lib_DiffractionConditions.f90 and
// Lib_RelativisticElectrons.f90.  Compiled with -ffp-contract=off: every
// expression keeps the reference's left-to-right double arithmetic, so the
// geometry handed to st_image (cell sizes, offsets, rotations) is the
// reference's to the last bit.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>

#include "../../include/stem_host.h"
#include "internal.h"

#include "host_geom.h"

using namespace stem_geom;

namespace {

int estimate_max_count_per_cell(double n_cells, int n_total) {  // Lib_LinkCell3D.f90:320-349
  const double rho = n_total / n_cells;
  double pp = std::exp(-rho), psum = pp;
  for (int kk = 1; kk <= n_total; ++kk) {
    if (psum >= 0.99) return kk;
    pp = pp * rho / kk;
    psum = psum + pp;
  }
  return n_total;
}

// FactoriseParallel0 for one to four processes (Lib_FactoriseParallel.f90:33-88)
bool factorise_parallel(int A, int B, int N, int& C, int& D) {
  const double a = A, b = B;
  switch (N) {
    case 1: C = 1; D = 1; return true;
    case 2: if (a >= b) { C = 2; D = 1; } else { C = 1; D = 2; } return true;
    case 3: if (a >= b) { C = 3; D = 1; } else { C = 1; D = 3; } return true;
    case 4:
      if (a >= 2 * b) { C = 4; D = 1; }
      else if (b >= 2 * a) { C = 1; D = 4; }
      else { C = 2; D = 2; }
      return true;
    default: return false;
  }
}

}  // namespace

extern "C" {

int st_d2bi_create(st_d2bi** h, const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double a0, const double* k,
                   const double* g, double E, int32_t mxy, int32_t mzz) {
  if (!h || !a_vox || !k || !g || Nx < 1 || Ny < 1 || Nz < 1 || !(a0 > 0) || mxy < 1 || mzz < 1) return ST_ERR_ARG;
  st_d2bi* t = new (std::nothrow) st_d2bi();
  if (!t) return ST_ERR_ALLOC;
  t->super = Supercell::make(Mat3::from(a_vox), Nx, Ny, Nz);
  t->a0 = a0;  // the constructor leaves a_cell = 1.0 * identity (a0 = 1 when it is set, :131)
  std::memcpy(t->k, k, sizeof t->k);
  std::memcpy(t->g, g, sizeof t->g);
  t->E = E;
  t->mxy = mxy;
  t->mzz = mzz;
  *h = t;
  return ST_OK;
}

void st_d2bi_destroy(st_d2bi* h) { delete h; }

int st_d2bi_set_conventional_unit_cell(st_d2bi* h, const double* a_cell) {
  if (!h || !a_cell) return ST_ERR_ARG;
  h->a_cell = Mat3::from(a_cell);
  return ST_OK;
}

int st_d2bi_set_voxel_supercell_size(st_d2bi* h, const double* cs) {
  if (!h || !cs) return ST_ERR_ARG;
  const double hkl[3] = {(double)std::lround(h->g[0]), (double)std::lround(h->g[1]), (double)std::lround(h->g[2])};
  h->U = rotate_to_standard_frame(h->k, h->a_cell, hkl);
  if (cs[0] == 0 || cs[1] == 0 || cs[2] == 0) return ST_ERR_ARG;  // sizes from the oriented supercell: not mirrored
  std::memcpy(h->vsd, cs, sizeof h->vsd);
  return ST_OK;
}

int st_d2bi_set_deviation_parameter(st_d2bi* h, double sg) {
  if (!h) return ST_ERR_ARG;
  h->sg = sg;
  return ST_OK;
}

int st_d2bi_set_supercell_tilt0(st_d2bi* t) {
  if (!t) return ST_ERR_ARG;
  const double hkl[3] = {(double)std::lround(t->g[0]), (double)std::lround(t->g[1]), (double)std::lround(t->g[2])};
  t->U = rotate_to_standard_frame(t->k, t->a_cell, hkl);
  const Mat3 a_cell0 = mul(t->U, t->a_cell);
  Vec3 gg = reflection(reciprocal(a_cell0), t->g);
  const double modg = norm2(gg.v);
  const double modk = 2 * kPi / wavelength(t->E * 1000);
  const double vv = kHbar * modk / kMe;
  const Vec3 khat{{0.0, 0.0, 1.0}};
  double eps = energy_deviation(vv, khat, gg);
  if (std::isnan(t->sg)) {
    t->sg = length_sg(vv, eps);
    t->R = Mat3::identity();
  } else {
    const double aa = 2 * kPi * t->sg + kHbar * modg * modg / (2 * kMe * vv);
    double cc = gg[0] * gg[0] + gg[2] * gg[2];
    double bb = cc - aa * aa;
    if (bb < 0) {
      t->sg = length_sg(vv, eps);
      t->R = Mat3::identity();
    } else {
      bb = std::sqrt(bb);
      cc = 1 / cc;
      double th[4], sgs[4];
      th[0] = std::acos(-(gg[2] * aa + gg[0] * bb) * cc);
      th[1] = std::acos(-(gg[2] * aa - gg[0] * bb) * cc);
      th[2] = -th[0];
      th[3] = -th[1];
      for (int i = 0; i < 4; ++i) {
        const Mat3 Ri = tilt_about_y(th[i]);
        const Vec3 g2 = reflection(reciprocal(mul(Ri, a_cell0)), t->g);
        sgs[i] = length_sg(vv, energy_deviation(vv, khat, g2));
      }
      for (int i = 0; i < 4; ++i)
        if (std::fabs(th[i]) * 2 > kPi) sgs[i] = kHuge1;
      int best = 0;
      double bestv = std::fabs(t->sg - sgs[0]);
      for (int i = 1; i < 4; ++i) {
        const double v = std::fabs(t->sg - sgs[i]);
        if (v < bestv) {
          bestv = v;
          best = i;
        }
      }
      t->R = tilt_about_y(th[best]);
    }
    gg = reflection(reciprocal(mul(t->R, a_cell0)), t->g);
    eps = energy_deviation(vv, khat, gg);
    t->sg = length_sg(vv, eps);
  }
  t->transformed_supercell();
  t->sg = t->deviation(t->aperture(nullptr));
  return ST_OK;
}

int st_d2bi_set_supercell_tilt2(st_d2bi* t, const double* U, const double* R) {
  if (!t || !U || !R) return ST_ERR_ARG;
  t->U = Mat3::from(U);
  t->R = Mat3::from(R);
  t->transformed_supercell();
  t->sg = t->deviation(t->aperture(nullptr));
  return ST_OK;
}

int st_d2bi_set_extinction_distances(st_d2bi* h, double xi0, double xig) {
  if (!h || !(xi0 != 0) || !(xig != 0)) return ST_ERR_ARG;
  h->xi0 = xi0;
  h->xig = xig;
  return ST_OK;
}

int st_d2bi_set_use_density_field(st_d2bi* h, int32_t use) {
  if (!h) return ST_ERR_ARG;
  h->useDensityField = use != 0;
  return ST_OK;
}

int st_d2bi_find_image_parameters(const st_d2bi* t, double* aperpx, double* xmax, double* modg, int32_t* Mx,
                                  int32_t* My, int32_t* Mz) {
  if (!t) return ST_ERR_ARG;
  const Vec3 gg = reflection(reciprocal(t->a_cell), t->g);
  double xm[3];
  for (int i = 1; i <= 3; ++i) xm[i - 1] = t->gksuper.super_side(i);
  const int mx = t->gksuper.Nx, my = t->gksuper.Ny, mz = t->gksuper.Nz;
  if (aperpx) *aperpx = std::sqrt(xm[0] * xm[1] / (double)(mx * my));
  if (xmax) std::memcpy(xmax, xm, sizeof xm);
  if (modg) *modg = norm2(gg.v);
  if (Mx) *Mx = mx;
  if (My) *My = my;
  if (Mz) *Mz = mz;
  return ST_OK;
}

int st_d2bi_get_rotation(const st_d2bi* h, double* U, double* R) {
  if (!h) return ST_ERR_ARG;
  if (U) std::memcpy(U, h->U.m, sizeof h->U.m);
  if (R) std::memcpy(R, h->R.m, sizeof h->R.m);
  return ST_OK;
}

double st_d2bi_get_deviation_parameter(const st_d2bi* h) { return h ? h->sg : NAN; }

namespace {

// The geometry of the pixel window [ix0, ix0 + Dx) x [iy0, iy0 + Dy) (clipped to the
// image): the patch set-up of computeD2BI_img (:1714-1760, 1843-1852) with the patch
// origin jx Dx, jy Dy replaced by (ix0, iy0).
int window_geometry(const st_d2bi* t, int64_t nAtoms, int ix0, int iy0, int Dx, int Dy, double precAngle,
                    int32_t nPrec, st_geom* G, double* aa) {
  std::memset(G, 0, sizeof *G);
  double xmax[3];
  int Mx, My, Mz;
  st_d2bi_find_image_parameters(t, nullptr, xmax, nullptr, &Mx, &My, &Mz);
  if (ix0 < 0 || iy0 < 0 || ix0 >= Mx || iy0 >= My || Dx < 1 || Dy < 1) return ST_ERR_ARG;
  double costheta = 1.0, sintheta = 0.0;
  if (nPrec > 1) {
    costheta = std::cos(precAngle);
    sintheta = std::sin(precAngle);
  }
  const double sigma = t->a0 / 2;
  const double cmin = std::min(t->gksuper.cell_side(1), t->gksuper.cell_side(2));
  const int deltaM = (int)std::ceil(3 * sigma / cmin);
  const int nMax = estimate_max_count_per_cell((double)Mx * My * Mz, (int)nAtoms) * deltaM * deltaM;
  // real(Dx)/deltaM + 2 is default-kind (single precision) in the reference
  const int Ex = std::max(3, (int)std::floor((float)Dx / (float)deltaM + 2.0f));
  const int Ey = std::max(3, (int)std::floor((float)Dy / (float)deltaM + 2.0f));
  const int Ez = std::max(3, (int)std::floor((float)Mz / (float)deltaM));
  const Mat3& a_vox = t->gksuper.a;
  Mat3 a_col;
  for (int i = 1; i <= 3; ++i) {
    a_col(i, 1) = (Dx + 2 * deltaM) * a_vox(i, 1) / Ex;
    a_col(i, 2) = (Dy + 2 * deltaM) * a_vox(i, 2) / Ey;
    a_col(i, 3) = Mz * a_vox(i, 3) / Ez;
  }
  const Supercell lc = Supercell::make(a_col, Ex, Ey, Ez);

  for (int prec = 1; prec <= nPrec; ++prec) {  // :1805-1831
    Vec3 gg;
    if (prec == 1) {
      gg = t->aperture(nullptr);
    } else {
      const double phi = (prec - 1) * 2 * kPi / (nPrec - 1);
      const double ux = std::sin(phi), uy = std::cos(phi);
      Mat3 BT;
      BT(1, 1) = costheta + ux * ux * (1 - costheta);
      BT(1, 2) = ux * uy * (1 - costheta);
      BT(1, 3) = uy * sintheta;
      BT(2, 1) = ux * uy * (1 - costheta);
      BT(2, 2) = costheta + uy * uy * (1 - costheta);
      BT(2, 3) = -ux * sintheta;
      BT(3, 1) = -uy * sintheta;
      BT(3, 2) = ux * sintheta;
      BT(3, 3) = costheta;
      gg = t->aperture(&BT);
    }
    Vec3 z{{0.0, 0.0, 0.0}};
    for (int i = 0; i < 3; ++i) z[i] = gg[i] + z[i];  // + dgAperturePoint (zero for one aperture point)
    aa[prec - 1] = (2 * kPi * t->deviation(z));
  }

  const Vec3 p0 = t->gksuper.cell_to_real(ix0, iy0, 0);  // :1843-1852
  const Vec3 p1 = lc.cell_to_real(1, 1, 0);
  for (int i = 0; i < 3; ++i) G->lc_delta[i] = p0[i] - p1[i];
  G->Mx = Mx;
  G->My = My;
  G->Mz = Mz;
  G->ix0 = ix0;
  G->ix1 = std::min(ix0 + Dx, Mx);
  G->iy0 = iy0;
  G->iy1 = std::min(iy0 + Dy, My);
  G->Ex = Ex;
  G->Ey = Ey;
  G->Ez = Ez;
  G->nMax0 = nMax;
  std::memcpy(G->a_col, lc.a.m, sizeof G->a_col);
  std::memcpy(G->ia_col, lc.ia.m, sizeof G->ia_col);
  std::memcpy(G->a_vox, a_vox.m, sizeof G->a_vox);
  const Mat3 RU = mul(t->R, t->U);
  std::memcpy(G->RU, RU.m, sizeof G->RU);
  std::memcpy(G->delta, t->delta, sizeof G->delta);
  G->nuvw = t->nuvw;
  const Mat3 sv = t->super.super_a();  // getSuperVector(this%super, i) = a(:,i) N_i
  for (int n = 0; n < t->nuvw; ++n)
    for (int i = 1; i <= 3; ++i)
      G->Ruvw[3 * n + i - 1] = t->uvw[3 * n] * sv(i, 1) + t->uvw[3 * n + 1] * sv(i, 2) + t->uvw[3 * n + 2] * sv(i, 3);
  const Vec3 g0 = t->aperture(nullptr);
  std::memcpy(G->g, g0.v, sizeof G->g);
  G->useDensity = t->useDensityField ? 1 : 0;
  G->sigma = sigma;
  G->deltaz = xmax[2] / Mz;
  G->b0 = (kPi / t->xi0);
  G->bg = (kPi / t->xig);
  return ST_OK;
}

}  // namespace

int st_d2bi_image_geometry(const st_d2bi* t, int64_t nAtoms, int32_t nprocs, int32_t jj, double precAngle,
                           int32_t nPrec, st_geom* G, double* aa) {
  if (!t || !G || !aa || nPrec < 1 || nAtoms < 0) return ST_ERR_ARG;
  double xmax[3];
  int Mx, My, Mz;
  st_d2bi_find_image_parameters(t, nullptr, xmax, nullptr, &Mx, &My, &Mz);
  int Cx, Cy;
  if (!factorise_parallel(Mx, My, nprocs, Cx, Cy)) return ST_ERR_ARG;
  if (jj < 0 || jj >= Cx * Cy) return ST_ERR_ARG;
  // real(Mx)/Cx is default-kind (single precision) in the reference
  const int Dx = (int)std::ceil((float)Mx / (float)Cx);
  const int Dy = (int)std::ceil((float)My / (float)Cy);
  const int jy = jj / Cx, jx = jj - jy * Cx;
  return window_geometry(t, nAtoms, jx * Dx, jy * Dy, Dx, Dy, precAngle, nPrec, G, aa);
}

int st_d2bi_window_geometry(const st_d2bi* t, int64_t nAtoms, int32_t ix0, int32_t iy0, int32_t Dx, int32_t Dy,
                            double precAngle, int32_t nPrec, st_geom* G, double* aa) {
  if (!t || !G || !aa || nPrec < 1 || nAtoms < 0) return ST_ERR_ARG;
  return window_geometry(t, nAtoms, ix0, iy0, Dx, Dy, precAngle, nPrec, G, aa);
}

int st_d2bi_compute_img(const st_d2bi* t, st_ctx* ctx, const double* x, int64_t ldx, int64_t nAtoms,
                        double precAngle, int32_t nPrec, int32_t flags, double* img) {
  if (!t || !ctx || nPrec < 1) return ST_ERR_ARG;
  st_geom G;
  double* aa = new (std::nothrow) double[nPrec];
  if (!aa) return ST_ERR_ALLOC;
  int rc = st_d2bi_image_geometry(t, nAtoms, 1, 0, precAngle, nPrec, &G, aa);
  if (rc == ST_OK) rc = st_image(ctx, &G, x, ldx, nAtoms, aa, nPrec, flags | ST_FLAG_AVERAGE, img);
  delete[] aa;
  return rc;
}

int st_wrap_pbc(const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double* x, int64_t ldx, int64_t n) {
  if (!a_vox || !x || ldx < 3 || n < 0 || Nx < 1 || Ny < 1 || Nz < 1) return ST_ERR_ARG;
  const Supercell s = Supercell::make(Mat3::from(a_vox), Nx, Ny, Nz);
  const int N[3] = {Nx, Ny, Nz};
  for (int64_t j = 0; j < n; ++j) {  // wrapPBC0 (Lib_SimpleSupercells.f90:992-1023)
    double* y = x + j * ldx;
    Vec3 xx = apply(s.ia, Vec3{{y[0], y[1], y[2]}});
    for (int d = 0; d < 3; ++d) {
      int ii = (int)std::floor(xx[d]);
      xx[d] = xx[d] - ii;
      ii = (ii + (N[d] << 8)) % N[d];
      xx[d] = (ii + xx[d]);
    }
    const Vec3 yp = apply(s.a, xx);
    y[0] = yp[0];
    y[1] = yp[1];
    y[2] = yp[2];
  }
  return ST_OK;
}

int st_atom_extents(const double* k, const double* g, const double* a_cell, const double* x, int64_t ldx, int64_t n,
                    double* d) {
  if (!k || !g || !a_cell || !d || (n > 0 && !x) || ldx < 3) return ST_ERR_ARG;
  const Mat3 rot = rotate_to_standard_frame(k, Mat3::from(a_cell), g);
  double lo[3] = {kHuge1, kHuge1, kHuge1}, hi[3] = {-kHuge1, -kHuge1, -kHuge1};
  for (int64_t j = 0; j < n; ++j) {
    const Vec3 y = apply(rot, Vec3{{x[j * ldx], x[j * ldx + 1], x[j * ldx + 2]}});
    for (int i = 0; i < 3; ++i) {
      lo[i] = std::min(lo[i], y[i]);
      hi[i] = std::max(hi[i], y[i]);
    }
  }
  for (int i = 0; i < 3; ++i) d[i] = hi[i] - lo[i];
  return ST_OK;
}

// ---- the same two passes over the atoms on the GPU (k_geom.cu), bit for bit

int st_wrap_pbc_device(st_ctx* ctx, const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double* d_x,
                       int64_t ldx, int64_t n, void* stream) {
  if (!ctx) return ST_ERR_ARG;
  if (!a_vox || !d_x || ldx < 3 || n < 0 || Nx < 1 || Ny < 1 || Nz < 1)
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid wrap arguments");
  const Supercell s = Supercell::make(Mat3::from(a_vox), Nx, Ny, Nz);
  stem::GeomWrap w;
  std::memcpy(w.a, s.a.m, sizeof w.a);
  std::memcpy(w.ia, s.ia.m, sizeof w.ia);
  w.N[0] = Nx;
  w.N[1] = Ny;
  w.N[2] = Nz;
  const cudaStream_t st = stem::ctx_stream(ctx, stream);
  const cudaError_t e = stem::launch_wrap_pbc(w, d_x, ldx, n, st);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "wrap");
  return ST_OK;
}

int st_atom_extents_device(st_ctx* ctx, int32_t n_cond, const double* k, const double* g, const double* a_cell,
                           const double* d_x, int64_t ldx, int64_t n, double* d) {
  if (!ctx) return ST_ERR_ARG;
  if (n_cond < 1 || n_cond > stem::kMaxRot || !k || !g || !a_cell || !d || (n > 0 && !d_x) || ldx < 3 || n < 1)
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid extents arguments (1 to 32 conditions, n >= 1)");
  stem::GeomRot rot;
  rot.n = n_cond;
  for (int r = 0; r < n_cond; ++r) {
    const Mat3 U = rotate_to_standard_frame(k + 3 * r, Mat3::from(a_cell), g + 3 * r);
    std::memcpy(rot.U + 9 * r, U.m, sizeof U.m);
  }
  const cudaStream_t st = stem::ctx_stream(ctx, nullptr);
  double *part = nullptr, *out = nullptr;
  cudaError_t e = stem::ctx_geom_scratch(ctx, &part, &out);
  if (e == cudaSuccess) e = stem::launch_extents(rot, d_x, ldx, n, part, out, st);
  double mm[6 * stem::kMaxRot];
  if (e == cudaSuccess) e = cudaMemcpyAsync(mm, out, 6 * n_cond * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "atom extents");
  for (int r = 0; r < n_cond; ++r)
    for (int i = 0; i < 3; ++i) d[3 * r + i] = mm[6 * r + 3 + i] - mm[6 * r + i];
  return ST_OK;
}

int st_tomography_tilt(double tomoAngle, int32_t nn, int32_t nTomo, const double* R0, double* Rout) {
  if (!R0 || !Rout || nTomo < 2 || nn < 0 || nn >= nTomo) return ST_ERR_ARG;
  double theta = tomoAngle - 2 * tomoAngle * nn / (nTomo - 1);
  theta = theta * 3.141592654 / 180.0;
  Mat3 R;
  const double v[9] = {1.0, 0.0, 0.0, 0.0, std::cos(theta), std::sin(theta), 0.0, -std::sin(theta), std::cos(theta)};
  std::memcpy(R.m, v, sizeof v);
  const Mat3 out = mul(R, Mat3::from(R0));
  std::memcpy(Rout, out.m, sizeof out.m);
  return ST_OK;
}

}  // extern "C"
