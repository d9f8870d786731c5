// Shared host types of the reference's set-up mirror: 3x3 column-major
// matrices, SimpleSupercell, and the state of type(DynamicalTwoBeamImaging).
// Included by the host translation units, which are compiled with
// -ffp-contract=off so that every expression keeps the reference's
// left-to-right double arithmetic.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace stem_geom {

constexpr double kPi = 3.141592653589790;  // PI of the reference modules
constexpr double kMe = 0.056856301036;     // Lib_RelativisticElectrons.f90:9-14
constexpr double kE = 1.0;
constexpr double kC = 2997.92458;
constexpr double kH = 4.135667696;
const double kHbar = kH / (2 * 3.14159265390);
const double kHuge1 = (double)FLT_MAX;  // huge(1.0)

struct Mat3 {
  double m[9];  // column-major
  double& operator()(int i, int j) { return m[(i - 1) + 3 * (j - 1)]; }
  double operator()(int i, int j) const { return m[(i - 1) + 3 * (j - 1)]; }
  static Mat3 identity() {
    Mat3 r{};
    r(1, 1) = r(2, 2) = r(3, 3) = 1.0;
    return r;
  }
  static Mat3 from(const double* p) {
    Mat3 r;
    std::memcpy(r.m, p, sizeof r.m);
    return r;
  }
};

struct Vec3 {
  double v[3];
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};

// gfortran NORM2: scaled sum of squares
inline double norm2(const double* v) {
  double scale = 0.0, res = 1.0;
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0.0) {
      const double ax = std::fabs(v[i]);
      if (scale < ax) {
        const double val = scale / ax;
        res = 1.0 + res * val * val;
        scale = ax;
      } else {
        const double val = ax / scale;
        res += val * val;
      }
    }
  }
  return std::sqrt(res) * scale;
}

// determinant3Mat (Lib_SimpleSupercells.f90:1240-1256)
inline double det3(const Mat3& M) {
  const double dd[9] = {M(1, 1) * (M(2, 2) * M(3, 3) - M(2, 3) * M(3, 2)),
                        M(1, 2) * (M(2, 3) * M(3, 1) - M(2, 1) * M(3, 3)),
                        M(1, 3) * (M(2, 1) * M(3, 2) - M(2, 2) * M(3, 1)),
                        M(2, 1) * (M(3, 2) * M(1, 3) - M(3, 3) * M(1, 2)),
                        M(2, 2) * (M(3, 3) * M(1, 1) - M(3, 1) * M(1, 3)),
                        M(2, 3) * (M(3, 1) * M(1, 2) - M(3, 2) * M(1, 1)),
                        M(3, 1) * (M(1, 2) * M(2, 3) - M(1, 3) * M(2, 2)),
                        M(3, 2) * (M(1, 3) * M(2, 1) - M(1, 1) * M(2, 3)),
                        M(3, 3) * (M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1))};
  double s = 0.0;
  for (double d : dd) s += d;
  return (1.0 / 3.0) * s;
}

// inverse3Mat (Lib_SimpleSupercells.f90:1205-1236)
inline Mat3 inv3(const Mat3& M) {
  double idd = det3(M);
  if (std::fabs(idd) < DBL_MIN) return Mat3::identity();
  idd = 1.0 / idd;
  Mat3 N;
  N(1, 1) = (M(2, 2) * M(3, 3) - M(2, 3) * M(3, 2)) * idd;
  N(2, 1) = (M(2, 3) * M(3, 1) - M(2, 1) * M(3, 3)) * idd;
  N(3, 1) = (M(2, 1) * M(3, 2) - M(2, 2) * M(3, 1)) * idd;
  N(1, 2) = (M(1, 3) * M(3, 2) - M(1, 2) * M(3, 3)) * idd;
  N(2, 2) = (M(1, 1) * M(3, 3) - M(1, 3) * M(3, 1)) * idd;
  N(3, 2) = (M(1, 2) * M(3, 1) - M(1, 1) * M(3, 2)) * idd;
  N(1, 3) = (M(1, 2) * M(2, 3) - M(1, 3) * M(2, 2)) * idd;
  N(2, 3) = (M(1, 3) * M(2, 1) - M(1, 1) * M(2, 3)) * idd;
  N(3, 3) = (M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1)) * idd;
  return N;
}

// matmul, k ascending
inline Mat3 mul(const Mat3& a, const Mat3& b) {
  Mat3 c;
  for (int j = 1; j <= 3; ++j)
    for (int i = 1; i <= 3; ++i) {
      double s = 0.0;
      for (int k = 1; k <= 3; ++k) s += a(i, k) * b(k, j);
      c(i, j) = s;
    }
  return c;
}

// y = m(:,1)*v(1) + m(:,2)*v(2) + m(:,3)*v(3)
inline Vec3 apply(const Mat3& m, const Vec3& v) {
  Vec3 y;
  for (int i = 1; i <= 3; ++i) y[i - 1] = m(i, 1) * v[0] + m(i, 2) * v[1] + m(i, 3) * v[2];
  return y;
}

inline Mat3 transpose(const Mat3& a) {
  Mat3 t;
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j) t(i, j) = a(j, i);
  return t;
}

// SimpleSupercell (Lib_SimpleSupercells.f90:51-55, 183-196)
struct Supercell {
  int Nx = 1, Ny = 1, Nz = 1;
  Mat3 a = Mat3::identity(), ia = Mat3::identity();
  static Supercell make(const Mat3& a, int nx, int ny, int nz) {
    Supercell s;
    s.a = a;
    s.Nx = nx;
    s.Ny = ny;
    s.Nz = nz;
    s.ia = inv3(a);
    return s;
  }
  int n(int i) const { return i == 1 ? Nx : (i == 2 ? Ny : Nz); }
  Vec3 col(int i) const { return Vec3{{a(1, i), a(2, i), a(3, i)}}; }
  // getSuperA (:851-860)
  Mat3 super_a() const {
    Mat3 s;
    for (int i = 1; i <= 3; ++i) {
      s(i, 1) = a(i, 1) * Nx;
      s(i, 2) = a(i, 2) * Ny;
      s(i, 3) = a(i, 3) * Nz;
    }
    return s;
  }
  double cell_side(int i) const {
    const Vec3 c = col(i);
    return norm2(c.v);
  }
  double super_side(int i) const { return cell_side(i) * n(i); }
  // cellToRealSpace2 (:338-345)
  Vec3 cell_to_real(int ix, int iy, int iz) const {
    Vec3 y;
    for (int i = 1; i <= 3; ++i) y[i - 1] = a(i, 1) * (double)ix + a(i, 2) * (double)iy + a(i, 3) * (double)iz;
    return y;
  }
};

inline double wavelength(double V) {  // Lib_RelativisticElectrons.f90:25-38
  if (V <= 0) return 0.0;
  const double lambda = 2 * kMe * kE * V * (1 + kE * V / (2 * kMe * kC * kC));
  return kH / std::sqrt(lambda);
}

inline double velocity(double V) {  // Lib_RelativisticElectrons.f90:40-50
  double u = 1 + kE * V / (kMe * kC * kC);
  return kC * std::sqrt(1 - 1 / (u * u));
}

inline Mat3 reciprocal(const Mat3& a_cell) {  // Lib_DiffractionConditions.f90:1630-1640
  Mat3 b = inv3(transpose(a_cell));
  for (double& v : b.m) v = 2 * kPi * v;
  return b;
}

inline Vec3 reflection(const Mat3& B, const double* hkl) {  // :1656-1667
  Vec3 g;
  for (int i = 1; i <= 3; ++i) g[i - 1] = B(i, 1) * hkl[0] + B(i, 2) * hkl[1] + B(i, 3) * hkl[2];
  return g;
}

inline double length_sg(double v, double eps) { return -eps / (2 * kPi * kHbar * v); }  // :1194-1204

inline double energy_deviation(double v, const Vec3& khat, const Vec3& g) {  // :1265-1299
  const double hbar2on2m = kHbar * kHbar / (2 * kMe);
  const double cst = 2 * kMe * v / kHbar;
  double eps = khat[0] * g[0] + khat[1] * g[1] + khat[2] * g[2];
  eps = cst * eps;
  eps = eps + g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  return eps * hbar2on2m;
}

// rotateToStandardFrame0 (Lib_DiffractionConditions.f90:65-108)
inline Mat3 rotate_to_standard_frame(const double* z0, const Mat3& A_cell, const double* hkl) {
  const Mat3 BB = reciprocal(A_cell);
  const Vec3 gg = reflection(BB, hkl);
  Vec3 zz;
  for (int i = 1; i <= 3; ++i) {
    double s = 0.0;
    for (int k = 1; k <= 3; ++k) s += A_cell(i, k) * z0[k - 1];
    zz[i - 1] = s;
  }
  const double nz = norm2(zz.v);
  for (int i = 0; i < 3; ++i) zz[i] = zz[i] / nz;
  double gz = 0.0;
  for (int i = 0; i < 3; ++i) gz += gg[i] * zz[i];
  Vec3 xx;
  for (int i = 0; i < 3; ++i) xx[i] = gg[i] - gz * zz[i];
  const double nx = norm2(xx.v);
  for (int i = 0; i < 3; ++i) xx[i] = xx[i] / nx;
  const Vec3 yy{{zz[1] * xx[2] - zz[2] * xx[1], zz[2] * xx[0] - zz[0] * xx[2], zz[0] * xx[1] - zz[1] * xx[0]}};
  Mat3 U;
  for (int j = 1; j <= 3; ++j) {
    U(1, j) = xx[j - 1];
    U(2, j) = yy[j - 1];
    U(3, j) = zz[j - 1];
  }
  return U;
}

inline Mat3 tilt_about_y(double th) {
  const double c = std::cos(th), s = std::sin(th);
  Mat3 R;
  const double v[9] = {c, 0.0, -s, 0.0, 1.0, 0.0, s, 0.0, c};
  std::memcpy(R.m, v, sizeof v);
  return R;
}

}  // namespace stem_geom

// type(DynamicalTwoBeamImaging) (Lib_DynamicalTwoBeamImaging.f90:59-84)
struct st_d2bi {
  using Mat3 = stem_geom::Mat3;
  using Vec3 = stem_geom::Vec3;
  using Supercell = stem_geom::Supercell;
  double k[3], g[3];
  double a0;
  Supercell super;
  double sg = NAN;
  int mxy = 0, mzz = 0;
  double xi0 = 103.9, xig = 207.5;
  double E = 150.0;
  bool useDensityField = true;
  Supercell gksuper;
  double delta[3] = {0, 0, 0};
  double vsd[3] = {0, 0, 0};  // voxelSupercellDimensions
  int nuvw = 1;
  int uvw[3 * 27] = {0};
  Mat3 a_cell = Mat3::identity(), U = Mat3::identity(), R = Mat3::identity();
  int latt = 2;                 // type(Lattice): LATTICE_BCC unless set (Lib_Lattices.f90:65-69)
  double foilThickness = 0.0;   // set by the -ng tilt search

  Vec3 aperture(const Mat3* beam_tilt) const {  // getAperture (:1137-1155)
    using namespace stem_geom;
    const Mat3 b = reciprocal(a_cell);
    Vec3 gv = reflection(b, g);
    Mat3 RU = mul(R, U);
    if (beam_tilt) RU = mul(*beam_tilt, RU);
    return apply(RU, gv);
  }
  double deviation(const Vec3& gv) const {  // getDeviationParameter (:292-307)
    using namespace stem_geom;
    const double modk = 2 * kPi / wavelength(E * 1000);
    const double vv = kHbar * modk / kMe;
    return length_sg(vv, energy_deviation(vv, Vec3{{0.0, 0.0, 1.0}}, gv));
  }
  // findTransformedSupercell (Lib_DiffractionConditions.f90:996-1189) and the
  // gksuper built from it (:775-784, :1086-1096)
  void transformed_supercell() {
    using namespace stem_geom;
    transformed_supercell_with(mul(R, U));
    Mat3 D{};
    D(1, 1) = vsd[0];
    D(2, 2) = vsd[1];
    D(3, 3) = vsd[2];
    const int nx = std::max(mxy, (int)std::lround(mxy * D(1, 1) / a0));
    const int ny = std::max(mxy, (int)std::lround(mxy * D(2, 2) / a0));
    const int nz = std::max(mzz, (int)std::lround(mzz * D(3, 3) / a0));
    D(1, 1) = D(1, 1) / nx;
    D(2, 2) = D(2, 2) / ny;
    D(3, 3) = D(3, 3) / nz;
    gksuper = Supercell::make(D, nx, ny, nz);
  }
  // the offset delta and the 27 replicas of findTransformedSupercell under rotation RU
  void transformed_supercell_with(const Mat3& RU) {
    using namespace stem_geom;
    const Mat3 A = super.super_a();
    Vec3 xx{{0.5, 0.5, 0.5}};
    xx = apply(A, xx);
    xx = apply(RU, xx);
    for (int i = 0; i < 3; ++i) delta[i] = vsd[i] / 2 - xx[i];
    int n = 0;
    for (int iz = -1; iz <= 1; ++iz)
      for (int iy = -1; iy <= 1; ++iy)
        for (int ix = -1; ix <= 1; ++ix) {
          uvw[3 * n] = ix;
          uvw[3 * n + 1] = iy;
          uvw[3 * n + 2] = iz;
          ++n;
        }
    nuvw = n;
  }
};

