// The -ng tilt search: setSupercellTilt1a / setSupercellTilt1
// (src/Lib_DynamicalTwoBeamImaging.f90:795-1045) with findBestRotationMatrix and
// tiltToDarkField (src/Lib_DiffractionConditions.f90:129-357, 751-927), the
// extinction-distance table reader (src/Lib_ReadExtinctionDistances.f90:29-170), the
// permitted reflections of a lattice (src/Lib_Lattices.f90:678-735), the golden-section
// search (src/Lib_GoldenSection.f90) and the quaternion slerp (src/Lib_Quaternions.f90).
//
// The work that grows with the problem, the scores of every candidate beam direction
// against every permitted reflection (4,000 x 2,100 terms for a bcc crystal within the
// default radius) and, with atoms given, the foil-thickness pass over 27 replicas of
// every atom, runs on the GPU (k_tilt.cu).  The host keeps the scalar steps and makes
// the final choice: the GPU scores differ from the reference's arithmetic only through
// the sine and cosine of two phases per term and the order of the sum, both bounded,
// and every candidate within twice that bound of the best is re-scored here in the
// reference's own arithmetic.  The direction chosen is the one the reference's
// arithmetic chooses; the rest of the chain is the reference's scalar code.
//
// Reference behaviours kept: find_gvectors_permittedReflections swaps hklp(:,1) rather
// than hklp(:,2) with hklp(:,ihkl) (:1779-1786), so the xi_0 of every score term is the
// table's xi of [hkl]; tiltToDarkField runs with the imaging object's xi_0, xi_g as set
// at that point (d2bi sets them from the table only after the tilt, src/d2bi.f90:1266),
// i.e. the constructor's 103.9 and 207.5 A.  RotMatToQuaternion's eigenvector comes from
// LAPACK DSYEV in the reference; it is restated here as a cyclic Jacobi eigen-solve
// (the eigenvalue is isolated: 3 against -1, -1, -1), equal to DSYEV's up to rounding.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/stem_host.h"
#include "host_geom.h"
#include "internal.h"

using namespace stem_geom;

namespace {

constexpr int kNTheta = 2000;                   // NTHETA (Lib_DiffractionConditions.f90:22)
const double kDegToRad = 3.141592654 / 180;     // DEGTORAD (:26)
constexpr int kMaxIncident = 4 * kNTheta;       // size(khat, 2)

// ---- extinction distances ------------------------------------------------------

// symmetry (Lib_ReadExtinctionDistances.f90:112-170)
void standard_form(const int* in, int symm, int* out) {
  const int hh = std::abs(in[0]), kk = std::abs(in[1]), ll = std::abs(in[2]);
  auto set = [out](int a, int b, int c) {
    out[0] = a;
    out[1] = b;
    out[2] = c;
  };
  if (symm == ST_SYMMETRY_CUBIC) {
    if (hh >= std::max(kk, ll)) {
      if (kk >= ll) set(hh, kk, ll);
      else set(hh, ll, kk);
    } else if (kk >= std::max(hh, ll)) {
      if (hh >= ll) set(kk, hh, ll);
      else set(kk, ll, hh);
    } else {
      if (hh >= kk) set(ll, hh, kk);
      else set(ll, kk, hh);
    }
  } else {
    if (in[0] * in[1] >= 0) {
      if (hh >= kk) set(hh, kk, ll);
      else set(kk, hh, ll);
    } else {
      if (hh >= kk) set(hh, -kk, ll);
      else set(kk, -hh, ll);
    }
  }
}

bool separator(char c) { return c == ' ' || c == '\t' || c == ',' || c == '\r' || c == '\n'; }

// One list-directed READ of `dummy, idat(3), rdat(5)`: starts at a new record and
// continues over records until the nine items are read.  false at the end of the
// file or on an item of the wrong form (iostat /= 0).
bool read_table_record(FILE* f, int* idat, double* rdat) {
  char line[4096];
  int got = 0;
  while (got < 9) {
    if (!std::fgets(line, sizeof line, f)) return false;
    const char* p = line;
    while (got < 9) {
      while (*p && separator(*p)) ++p;
      if (!*p) break;
      const char* s = p;
      while (*p && !separator(*p)) ++p;
      char tok[256];
      const size_t len = std::min((size_t)(p - s), sizeof tok - 1);
      std::memcpy(tok, s, len);
      tok[len] = 0;
      if (got >= 1 && got <= 3) {
        char* e;
        const long v = std::strtol(tok, &e, 10);
        if (e == tok || *e) return false;
        idat[got - 1] = (int)v;
      } else if (got >= 4) {
        for (char* q = tok; *q; ++q)
          if (*q == 'd' || *q == 'D') *q = 'E';  // Fortran double-precision exponent
        char* e;
        const double v = std::strtod(tok, &e);
        if (e == tok || *e) return false;
        rdat[got - 4] = v;
      }
      ++got;
    }
  }
  return true;
}

// readExtinctionDistance: 1 all found, 0 some missing, -1 no file / no header
int read_extinction_distances(const char* path, int n, const int* hkl, int symm, double* xi_g) {
  for (int j = 0; j < n; ++j) xi_g[j] = kHuge1;
  FILE* f = path ? std::fopen(path, "r") : nullptr;
  if (!f) return -1;
  std::vector<int> hs(3 * (size_t)std::max(n, 1));
  std::vector<char> found((size_t)std::max(n, 1), 0);
  for (int j = 0; j < n; ++j) standard_form(hkl + 3 * j, symm, &hs[3 * j]);
  char line[4096];
  bool header = std::fgets(line, sizeof line, f) != nullptr;
  header = std::fgets(line, sizeof line, f) != nullptr;  // only the second read's status is checked
  if (!header) {
    std::fclose(f);
    return -1;
  }
  for (int ii = 1; ii <= 1000; ++ii) {
    int idat[3], is[3];
    double rdat[5];
    if (!read_table_record(f, idat, rdat)) break;
    standard_form(idat, symm, is);
    bool all = true;
    for (int j = 0; j < n; ++j) {
      if (is[0] == hs[3 * j] && is[1] == hs[3 * j + 1] && is[2] == hs[3 * j + 2]) {
        found[j] = 1;
        xi_g[j] = rdat[4];
      }
      all = all && found[j];
    }
    if (all) break;
  }
  std::fclose(f);
  for (int j = 0; j < n; ++j)
    if (!found[j]) return 0;
  return 1;
}

int table_symmetry(int latt) {
  if (latt == ST_LATTICE_HCP) return ST_SYMMETRY_HEXAGONAL;
  if (latt >= ST_LATTICE_SC && latt <= ST_LATTICE_FCC) return ST_SYMMETRY_CUBIC;
  return -1;
}

// ---- reflections and candidate directions ------------------------------------------

// permittedReflections: l outermost, h innermost
int permitted_reflections(int latt, double rho, int* hkl, int cap) {
  const int mm = (int)std::ceil(rho + 1.0e-12);
  int n = 0;
  for (int lp = -mm; lp <= mm; ++lp)
    for (int kp = -mm; kp <= mm; ++kp)
      for (int hp = -mm; hp <= mm; ++hp) {
        int rr = lp * lp + kp * kp + hp * hp;
        bool ok;
        if (latt == ST_LATTICE_HCP) {
          rr = (int)std::floor((double)((hp + kp) * (hp + kp) + (hp - kp) * (hp - kp) / 3) + lp * lp * 0.375);
          if (rr > rho * rho + 1.0e-6) continue;
          ok = !(((hp + 2 * kp) % 3 == 0) && (std::abs(lp) % 2 == 1));
        } else {
          if (rr > rho * rho + 1.0e-6) continue;
          if (latt == ST_LATTICE_FCC) {
            const int hx = hp % 2, kx = kp % 2, lx = lp % 2;  // Fortran mod: sign of the dividend
            ok = (hx * hx + kx * kx + lx * lx) - (hx * kx + kx * lx + lx * hx) == 0;
          } else if (latt == ST_LATTICE_BCC) {
            ok = (hp + kp + lp) % 2 == 0;
          } else {
            ok = true;
          }
        }
        if (!ok) continue;
        if (hkl && n < cap) {
          hkl[3 * n] = hp;
          hkl[3 * n + 1] = kp;
          hkl[3 * n + 2] = lp;
        }
        ++n;
      }
  return n;
}

// find_gvectors_permittedReflections, both swaps as the reference makes them
void gvectors_permitted(int latt, const Mat3& B, const int* hkl, double rho, std::vector<double>& ghkl,
                        std::vector<int>& hklp) {
  const int n = permitted_reflections(latt, rho, nullptr, 0);
  hklp.assign(3 * (size_t)n, 0);
  ghkl.assign(3 * (size_t)n, 0.0);
  permitted_reflections(latt, rho, hklp.data(), n);
  int i000 = 0, ihkl = 0;
  for (int ii = 1; ii <= n; ++ii) {
    const int* h = &hklp[3 * (ii - 1)];
    if (h[0] * h[0] + h[1] * h[1] + h[2] * h[2] == 0) i000 = ii;
    const int d0 = h[0] - hkl[0], d1 = h[1] - hkl[1], d2 = h[2] - hkl[2];
    if (d0 * d0 + d1 * d1 + d2 * d2 == 0) ihkl = ii;
    const double hd[3] = {(double)h[0], (double)h[1], (double)h[2]};
    const Vec3 g = reflection(B, hd);
    for (int c = 0; c < 3; ++c) ghkl[3 * (ii - 1) + c] = g[c];
  }
  if (i000 != 0)
    for (int c = 0; c < 3; ++c) {
      std::swap(ghkl[c], ghkl[3 * (i000 - 1) + c]);
      std::swap(hklp[c], hklp[3 * (i000 - 1) + c]);
    }
  if (ihkl != 0)
    for (int c = 0; c < 3; ++c) {
      std::swap(ghkl[3 + c], ghkl[3 * (ihkl - 1) + c]);
      std::swap(hklp[c], hklp[3 * (ihkl - 1) + c]);  // hklp(:,1), as the reference does
    }
}

// findRotationsForBraggCondition2 (:1382-1515).  mode 0: nolimitPhi absent; 1: present
// and true; 2: present and false.
int bragg_rotations(double v, const Vec3& g, double cosq, double sinq, double phi0, double theta_max_deg, int mode,
                    double* phi) {
  int nphi = 0;
  const double xx = g[1] * sinq + g[2] * cosq;
  double aa = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  aa = -aa * kHbar / (2 * kMe * v);
  double uu = g[0] * g[0] + xx * xx;
  double vv = uu - aa * aa;
  if (vv < 0) return 0;
  uu = 1 / uu;
  vv = std::sqrt(vv) * g[0] * uu;
  uu = aa * xx * uu;
  const double lim = mode == 2 ? 2 * theta_max_deg * kDegToRad : theta_max_deg * kDegToRad;
  for (int branch = 0; branch < 2; ++branch) {
    const double c = branch == 0 ? uu + vv : uu - vv;
    if (!(std::fabs(c) <= 1)) continue;
    double pp = std::acos(c);
    const long jj = std::lround((pp - phi0) / (2 * kPi));
    pp = pp - 2 * jj * kPi;
    if (mode == 1 || std::fabs(pp - phi0) <= lim) {
      phi[nphi] = pp;
      phi[nphi + 1] = -pp;
      nphi += 2;
    }
  }
  return nphi;
}

// findAllEulerAngles (:1565-1625)
int all_euler_angles(double v, const Vec3& g, double theta0, double phi0, double theta_max, double theta_max_deg,
                     int mode, double* khat) {
  double theta_min = theta0 - theta_max / 2;
  if (!(theta_min > 0.0)) theta_min = 0.0;
  int nk = 0;
  for (int ii = 1; ii <= kNTheta; ++ii) {
    const double theta = theta_min + theta_max * ii / kNTheta;
    const double cost = std::cos(theta), sint = std::sin(theta);
    double phi[4];
    const int nphi = bragg_rotations(v, g, cost, sint, phi0, theta_max_deg, mode, phi);
    for (int jj = 0; jj < nphi; ++jj) {
      const double pp = phi[jj], cosp = std::cos(pp), sinp = std::sin(pp);
      khat[3 * (nk + jj)] = -sinp;
      khat[3 * (nk + jj) + 1] = sint * cosp;
      khat[3 * (nk + jj) + 2] = cost * cosp;
    }
    nk += nphi;
  }
  return nk;
}

// intensityAtDepthZ (:1209-1259), the reference's order: (phig bg) / (2 dd), |phig|^2
double intensity_at_depth(double xi0, double xig, double sg, double z) {
  const double b0 = kPi / xi0, bg = kPi / xig, aa = 2 * kPi * sg;
  const double dd = std::sqrt(aa * aa / 4 + bg * bg);
  const double l1 = (b0 + aa / 2) + dd, l2 = (b0 + aa / 2) - dd;
  double re = std::cos(l1 * z) - std::cos(l2 * z), im = std::sin(l1 * z) - std::sin(l2 * z);
  re = re * bg / (2 * dd);
  im = im * bg / (2 * dd);
  return re * re + im * im;
}

// scoreForIncidentVector1 (:1835-1867) in the reference's arithmetic
double score_exact(double v, const double* khat, const std::vector<double>& ghkl, const std::vector<double>& xi_g,
                   double foil) {
  const int nn = (int)xi_g.size();
  const Vec3 k{{khat[0], khat[1], khat[2]}};
  double s = 0;
  for (int ii = 3; ii <= nn; ++ii) {
    const Vec3 g{{ghkl[3 * (ii - 1)], ghkl[3 * (ii - 1) + 1], ghkl[3 * (ii - 1) + 2]}};
    const double sg = length_sg(v, energy_deviation(v, k, g));
    s = s + intensity_at_depth(xi_g[0], xi_g[ii - 1], sg, foil);
  }
  return s;
}

// ---- GPU scores and the exact choice -----------------------------------------------

int gpu_scores(st_ctx* ctx, double v, const double* khat, int nk, const double* ghkl, const double* xi_g, int nn,
               double foil, double* scores, double* ms) {
  const cudaStream_t st = stem::ctx_stream(ctx, nullptr);
  std::vector<double> bg((size_t)std::max(nn, 1));
  for (int j = 0; j < nn; ++j) bg[j] = kPi / xi_g[j];
  const size_t n_khat = 3 * (size_t)nk, n_g = 3 * (size_t)nn;
  const int ns = stem::tilt_slices(nn);
  const size_t n_part = (size_t)nk * ns;
  double* d = nullptr;
  cudaError_t e = stem::ctx_tilt_scratch(ctx, n_khat + n_g + nn + n_part, &d);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "tilt scratch");
  double *d_khat = d, *d_g = d + n_khat, *d_bg = d_g + n_g, *d_s = d_bg + nn;
  stem::TiltScores p;
  p.cst = 2 * kMe * v / kHbar;
  p.hbar2on2m = kHbar * kHbar / (2 * kMe);
  p.den = 2 * kPi * kHbar * v;
  p.twopi = 2 * kPi;
  p.b0 = kPi / xi_g[0];
  p.foil = foil;
  p.nk = nk;
  p.nn = nn;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_khat, khat, n_khat * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_g, ghkl, n_g * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_bg, bg.data(), nn * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], st);
  if (e == cudaSuccess) e = stem::launch_tilt_scores(p, d_khat, d_g, d_bg, d_s, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
  std::vector<double> part(n_part);
  if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_s, n_part * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (int i = 0; i < nk && e == cudaSuccess; ++i) {  // the slices of each score, in order
    double s = 0.0;
    for (int k = 0; k < ns; ++k) s += part[(size_t)i * ns + k];
    scores[i] = s;
  }
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "tilt scores");
  if (ms) *ms = t;
  return ST_OK;
}

// The FP32 screen of every direction: scores and bounds on their errors (summed over the
// slices in FP64; the warp's FP32 sum of a slice adds a few ulps of it).
int gpu_screen(st_ctx* ctx, double v, const double* khat, int nk, const double* ghkl, const double* xi_g, int nn,
               double foil, std::vector<double>& s32, std::vector<double>& b32, double* ms) {
  const cudaStream_t st = stem::ctx_stream(ctx, nullptr);
  // FP32 copies of the inputs (the conversions would otherwise run on the FP64 pipe per term)
  const size_t n_khat = 3 * (size_t)nk, n_g = 3 * (size_t)nn;
  std::vector<float> in(n_khat + n_g + (size_t)nn);
  for (size_t i = 0; i < n_khat; ++i) in[i] = (float)khat[i];
  for (size_t i = 0; i < n_g; ++i) in[n_khat + i] = (float)ghkl[i];
  for (int j = 0; j < nn; ++j) in[n_khat + n_g + j] = (float)(kPi / xi_g[j]);
  const int ns = stem::tilt_slices(nn);
  const size_t n_part = (size_t)nk * ns;  // float pairs: n_part doubles of room
  double* d = nullptr;
  cudaError_t e = stem::ctx_tilt_scratch(ctx, (in.size() + 1) / 2 + n_part + 1, &d);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "tilt scratch");
  float* d_khat = reinterpret_cast<float*>(d);
  float *d_g = d_khat + n_khat, *d_bg = d_g + n_g;
  float* d_p = reinterpret_cast<float*>(d + (in.size() + 1) / 2 + 1);
  stem::TiltScores p;
  p.cst = 2 * kMe * v / kHbar;
  p.hbar2on2m = kHbar * kHbar / (2 * kMe);
  p.den = 2 * kPi * kHbar * v;
  p.twopi = 2 * kPi;
  p.b0 = kPi / xi_g[0];
  p.foil = foil;
  p.nk = nk;
  p.nn = nn;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_khat, in.data(), in.size() * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], st);
  if (e == cudaSuccess) e = stem::launch_tilt_screen(p, d_khat, d_g, d_bg, d_p, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
  std::vector<float> part(2 * n_part);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), d_p, 2 * n_part * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "tilt screen");
  s32.assign((size_t)nk, 0.0);
  b32.assign((size_t)nk, 0.0);
  for (int i = 0; i < nk; ++i) {
    double s = 0.0, b = 0.0;
    for (int k = 0; k < ns; ++k) {
      s += part[2 * ((size_t)i * ns + k)];
      b += part[2 * ((size_t)i * ns + k) + 1];
    }
    s32[i] = s;
    b32[i] = b + 4.0e-6 * std::fabs(s) + 1e-12;
  }
  if (ms) *ms = t;
  return ST_OK;
}

// The reference's argmin (first strictly smaller score) from the GPU scores: every
// candidate whose score can lie within the scores' error bound of the best is re-scored
// in the reference's arithmetic.  The bound per score: 4e-15 per term for the sine and
// cosine of the two phases (at most a few ulp of values of modulus <= 1, after factors
// <= 1), plus the rounding of two different summation orders, nn * 2^-52 * score.
int choose_best(const double* khat, int nk, const double* gpu, const std::vector<double>& ghkl,
                const std::vector<double>& xi_g, double v, double foil, double* ss_best, int* n_recheck) {
  const double nn = (double)xi_g.size();
  auto bound = [nn](double s) { return 8.0 * (nn * 4.0e-15 + nn * 2.3e-16 * std::fabs(s)); };
  double lim = kHuge1;
  for (int i = 0; i < nk; ++i) lim = std::min(lim, gpu[i] + bound(gpu[i]));
  int best = -1, n = 0;
  double sb = kHuge1;
  for (int i = 0; i < nk; ++i) {
    if (!(gpu[i] - bound(gpu[i]) <= lim)) continue;
    ++n;
    const double s = score_exact(v, khat + 3 * i, ghkl, xi_g, foil);
    if (s < sb) {
      sb = s;
      best = i;
    }
  }
  *ss_best = sb;
  *n_recheck = n;
  return best;
}

// ---- golden section (Lib_GoldenSection.f90) ----------------------------------------

struct Golden {
  double x1 = 0, x2 = 0, x3 = 0, y1 = 0, y2 = 0, y3 = 0;
  bool bounded = false;
  int step = 0;
  double xtol = 0, ytol = 0;
  static constexpr double kTol = 1.0e-6, kMinStep = 50, kBoundStep = 10;
  static double ratio() { return (1 + std::sqrt(5.0)) / 2; }

  Golden(double a1, double a3, double b1, double b3) {  // GoldenSection_ctor0 (:126-150)
    if (a1 < a3) {
      x1 = a1, x3 = a3, y1 = b1, y3 = b3;
    } else {
      x3 = a3, x1 = a1, y3 = b3, y1 = b1;
    }
    x2 = 0.0;
    y2 = kHuge1;
    xtol = (x3 - x1) * kTol;
    ytol = std::max(kTol, std::fabs(y3 - y1)) * kTol;
  }
  void check_bounds(double xt, double yt) {  // checkBounds0 (:152-264)
    if (step == 1) {
      if (yt < std::min(y1, y3)) {
        bounded = true, x2 = xt, y2 = yt;
      } else if (yt > y1 && y1 > y3) {
        bounded = false, x1 = xt, y1 = yt;
      } else if (yt > y3 && y3 > y1) {
        bounded = false, x3 = xt, y3 = yt;
      } else if (y1 > yt && yt > y3) {
        bounded = false, x1 = xt, y1 = yt;
      } else if (y3 > yt && yt > y1) {
        bounded = false, x3 = xt, y3 = yt;
      }
      return;
    }
    if (y1 < y3) {
      bounded = !(yt < y1);
      x2 = x1, x1 = xt, y2 = y1, y1 = yt;
    } else {
      bounded = !(yt < y3);
      x2 = x3, x3 = xt, y2 = y3, y3 = yt;
    }
  }
  double next_point() const {  // nextPoint0 (:266-306)
    const double G = ratio();
    if (!bounded) {
      if (step == 0) return x1 + (x3 - x1) * (G - 1);
      if (y1 < y3) return x1 - (x3 - x1) / G;
      return x3 + (x3 - x1) / G;
    }
    return x1 + (x3 - x2);
  }
  void minimise(double& xt, double& yt, bool& is, bool& ok) {  // minimise0 (:308-381)
    step = step + 1;
    if (!bounded) {
      check_bounds(xt, yt);
      is = false;
      ok = bounded || (step <= kBoundStep);
      return;
    }
    is = false;
    ok = step <= kMinStep;
    if (!ok) return;
    if (yt < y2) {
      if (xt < x2) {
        x3 = x2, y3 = y2, x2 = xt, y2 = yt;
      } else {
        x1 = x2, y1 = y2, x2 = xt, y2 = yt;
      }
    } else {
      if (xt > x2) x3 = xt, y3 = yt;
      else x1 = xt, y1 = yt;
    }
    is = (std::fabs(x3 - x1) < xtol) || (std::fabs(y2 - std::max(y1, y3)) < ytol);
    if (is) xt = x2, yt = y2;
  }
};

// |phi_g(L')|^2 after a tilt x about y (Lib_DiffractionConditions.f90:831-859)
double dark_field_intensity(double x, const Vec3& gg, double bg, double foil) {
  const double cost = std::cos(x), sint = std::sin(x);
  const double Lp = foil / cost;
  const double sgp = (sint * gg[0] - cost * gg[2]) / (2 * kPi);
  const double s = bg * std::sin(kPi * std::sqrt(sgp * sgp + bg * bg) * Lp);
  return s * s / (sgp * sgp + bg * bg);
}

// tiltToDarkField (:751-927): R <- Ry(theta) R
double tilt_to_dark_field(double v, const Mat3& a_cell, const int* hkl, double xig, double foil,
                          double theta_max_deg, const Mat3& U, Mat3& R) {
  const double hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]};
  const Vec3 kk = reflection(reciprocal(a_cell), hd);
  const Vec3 gg = apply(mul(R, U), kk);
  const double bg = 1 / xig;
  const double sg = length_sg(v, energy_deviation(v, Vec3{{0.0, 0.0, 1.0}}, gg));
  const double s0 = bg * std::sin(kPi * std::sqrt(sg * sg + bg * bg) * foil);
  const double phiL2 = s0 * s0 / (sg * sg + bg * bg);
  const double x1 = -(theta_max_deg * 0.01 * kDegToRad), x3 = +(theta_max_deg * 0.01 * kDegToRad);
  Golden gold(x1, x3, dark_field_intensity(x1, gg, bg, foil), dark_field_intensity(x3, gg, bg, foil));
  double x2, y2;
  for (;;) {
    x2 = gold.next_point();
    y2 = dark_field_intensity(x2, gg, bg, foil);
    bool conv, ok;
    gold.minimise(x2, y2, conv, ok);
    if (conv || !ok) break;
  }
  double theta = 0.0, cost = 1.0, sint = 0.0;
  if (y2 < phiL2) theta = x2, cost = std::cos(x2), sint = std::sin(x2);
  Mat3 RR{};
  RR(1, 1) = cost, RR(1, 3) = sint, RR(2, 2) = 1.0, RR(3, 1) = -sint, RR(3, 3) = cost;
  R = mul(RR, R);
  return theta;
}

// ---- quaternions (Lib_Quaternions.f90) ---------------------------------------------

struct Quat {
  double w, x, y, z;
};

// the unit eigenvector of the largest eigenvalue of a symmetric 4x4 matrix (column-major),
// by cyclic Jacobi rotations until the off-diagonal part vanishes
void dominant_eigenvector(const double* K, double* vec) {
  double a[16], V[16];
  std::memcpy(a, K, sizeof a);
  for (int i = 0; i < 16; ++i) V[i] = (i % 5 == 0) ? 1.0 : 0.0;
  auto at = [](double* m, int i, int j) -> double& { return m[i + 4 * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) off += at(a, p, q) * at(a, p, q);
    if (off == 0.0) break;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) {
        const double apq = at(a, p, q);
        if (apq == 0.0) continue;
        const double th = (at(a, q, q) - at(a, p, p)) / (2 * apq);
        const double t =
            std::fabs(th) > 1.0e150 ? 0.5 / th : (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 4; ++k) {
          const double akp = at(a, k, p), akq = at(a, k, q);
          at(a, k, p) = c * akp - s * akq;
          at(a, k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          const double apk = at(a, p, k), aqk = at(a, q, k);
          at(a, p, k) = c * apk - s * aqk;
          at(a, q, k) = s * apk + c * aqk;
        }
        at(a, p, q) = 0.0;
        at(a, q, p) = 0.0;
        for (int k = 0; k < 4; ++k) {
          const double vkp = at(V, k, p), vkq = at(V, k, q);
          at(V, k, p) = c * vkp - s * vkq;
          at(V, k, q) = s * vkp + c * vkq;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < 4; ++i)
    if (at(a, i, i) >= at(a, best, best)) best = i;
  for (int k = 0; k < 4; ++k) vec[k] = at(V, k, best);
}

Quat rotmat_to_quaternion(const Mat3& R) {  // RotMatToQuaternion (:246-288)
  double K[16] = {0};
  auto k4 = [&K](int i, int j) -> double& { return K[(i - 1) + 4 * (j - 1)]; };
  k4(1, 1) = R(1, 1) - R(2, 2) - R(3, 3);
  k4(2, 1) = R(2, 1) + R(1, 2);
  k4(3, 1) = R(3, 1) + R(1, 3);
  k4(4, 1) = R(2, 3) - R(3, 2);
  k4(2, 2) = R(2, 2) - R(1, 1) - R(3, 3);
  k4(3, 2) = R(3, 2) + R(2, 3);
  k4(4, 2) = R(3, 1) - R(1, 3);
  k4(3, 3) = R(3, 3) - R(1, 1) - R(2, 2);
  k4(4, 3) = R(1, 2) - R(2, 1);
  k4(4, 4) = R(1, 1) + R(2, 2) + R(3, 3);
  for (int j = 1; j <= 4; ++j)
    for (int i = 1; i < j; ++i) k4(i, j) = k4(j, i);  // DSYEV("V", "L"): the lower triangle
  double v[4];
  dominant_eigenvector(K, v);
  if (v[3] > 0)
    for (double& c : v) c = -c;
  return Quat{-v[3], v[0], v[1], v[2]};
}

Mat3 quaternion_to_rotmat(const Quat& q) {  // quaternionToRotMat (:290-321)
  double ss = (q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w) / 2;
  Mat3 R;
  R(1, 1) = ss - (q.y * q.y + q.z * q.z);
  R(2, 1) = (q.x * q.y + q.z * q.w);
  R(3, 1) = (q.x * q.z - q.y * q.w);
  R(1, 2) = (q.x * q.y - q.z * q.w);
  R(2, 2) = ss - (q.x * q.x + q.z * q.z);
  R(3, 2) = (q.y * q.z + q.x * q.w);
  R(1, 3) = (q.x * q.z + q.y * q.w);
  R(2, 3) = (q.y * q.z - q.x * q.w);
  R(3, 3) = ss - (q.x * q.x + q.y * q.y);
  ss = 1 / ss;
  for (double& m : R.m) m = m * ss;
  return R;
}

Quat slerp(const Quat& q1, const Quat& q2, double x) {  // slerp (:526-564), midpoint (:504-524)
  double x1 = q1.w * q2.w + q1.x * q2.x + q1.y * q2.y + q1.z * q2.z;
  if (x1 >= 1.0) return q1;
  if (x1 <= -1.0) {
    Quat m{q1.w + q2.w, q1.x + q2.x, q1.y + q2.y, q1.z + q2.z};
    double dd = m.w * m.w + m.x * m.x + m.y * m.y + m.z * m.z;
    if (dd > 0) {
      dd = 1 / std::sqrt(dd);
      m = Quat{m.w * dd, m.x * dd, m.y * dd, m.z * dd};
    }
    return m;
  }
  double x2 = 2 * x1 * x1 - 1;
  const double omega = std::acos(x2);
  x2 = 1 / std::sin(omega);
  x1 = std::sin((1 - x) * omega) * x2;
  x2 = std::sin(x * omega) * x2;
  Quat q{x1 * q1.w + x2 * q2.w, x1 * q1.x + x2 * q2.x, x1 * q1.y + x2 * q2.y, x1 * q1.z + x2 * q2.z};
  double tt = q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z;  // normalise0 (:203-219)
  if (tt == 0) return Quat{1.0, 0.0, 0.0, 0.0};
  tt = 1 / std::sqrt(tt);
  return Quat{q.w * tt, q.x * tt, q.y * tt, q.z * tt};
}

// ---- findBestRotationMatrix ---------------------------------------------------------

int best_rotation(st_ctx* ctx, double v, const double* z0, const Mat3& A_cell, int latt, const int* hkl,
                  const char* xifile, double foil, double theta_max_deg, double rho_max, Mat3& U, Mat3& R,
                  st_tilt_info* info) {
  const int symm = table_symmetry(latt);
  if (symm < 0) return stem::ctx_fail(ctx, ST_ERR_ARG, "tilt search: lattice must be sc, bcc, fcc or hcp");
  const double hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]};
  const Mat3 BB = reciprocal(A_cell);
  const Vec3 gg = reflection(BB, hd);
  U = rotate_to_standard_frame(z0, A_cell, hd);
  const Vec3 ghkl0 = apply(U, gg);
  std::vector<double> ghkl;
  std::vector<int> hklp;
  gvectors_permitted(latt, BB, hkl, rho_max, ghkl, hklp);
  const int nn = (int)(hklp.size() / 3);
  if (nn < 2) return stem::ctx_fail(ctx, ST_ERR_ARG, "tilt search: fewer than two permitted reflections");
  std::vector<double> xi_g((size_t)nn);
  const int xi_status = read_extinction_distances(xifile, nn, hklp.data(), symm, xi_g.data());
  std::vector<double> khat(3 * (size_t)kMaxIncident);
  int attempt = 1;
  int nk = all_euler_angles(v, ghkl0, 0.0, 0.0, theta_max_deg * kDegToRad, theta_max_deg, 0, khat.data());
  if (nk == 0) {
    attempt = 2;
    nk = all_euler_angles(v, ghkl0, 0.0, 0.0, 2 * theta_max_deg * kDegToRad, theta_max_deg, 0, khat.data());
    if (nk == 0) {
      attempt = 3;
      nk = all_euler_angles(v, ghkl0, 0.0, 0.0, theta_max_deg * kDegToRad, theta_max_deg, 1, khat.data());
    }
  }
  if (nk == 0) return stem::ctx_fail(ctx, ST_ERR_ARG, "tilt search: no tilt meets the Bragg condition");
  // FP32 screen of every direction, then the reference's FP64 arithmetic on the directions
  // whose screened score can be within its error bound of the best
  std::vector<double> s32, b32;
  double ms_screen = 0.0, ms = 0.0;
  int rc = gpu_screen(ctx, v, khat.data(), nk, ghkl.data(), xi_g.data(), nn, foil, s32, b32, &ms_screen);
  if (rc != ST_OK) return rc;
  double lim = kHuge1;
  for (int i = 0; i < nk; ++i) lim = std::min(lim, s32[i] + b32[i]);
  std::vector<int> cand;
  for (int i = 0; i < nk; ++i)
    if (s32[i] - b32[i] <= lim) cand.push_back(i);
  if (cand.empty() || cand.size() * 4 > (size_t)nk) {  // a flat landscape: score every direction in FP64
    cand.resize((size_t)nk);
    for (int i = 0; i < nk; ++i) cand[i] = i;
  }
  const int nc = (int)cand.size();
  std::vector<double> kc(3 * (size_t)nc);
  for (int c = 0; c < nc; ++c)
    for (int d = 0; d < 3; ++d) kc[3 * (size_t)c + d] = khat[3 * (size_t)cand[c] + d];
  std::vector<double> scores((size_t)nc);
  rc = gpu_scores(ctx, v, kc.data(), nc, ghkl.data(), xi_g.data(), nn, foil, scores.data(), &ms);
  if (rc != ST_OK) return rc;
  double ss_best;
  int n_recheck;
  const int icb = choose_best(kc.data(), nc, scores.data(), ghkl, xi_g, v, foil, &ss_best, &n_recheck);
  if (icb < 0) return stem::ctx_fail(ctx, ST_ERR_ARG, "tilt search: no finite score");
  const int ib = cand[icb];
  const double* kb = &khat[3 * (size_t)ib];
  const double phi = -std::asin(kb[0]);
  const double theta = std::acos(kb[2] / std::cos(phi));
  R(1, 1) = std::cos(phi), R(1, 2) = std::sin(theta) * std::sin(phi), R(1, 3) = std::cos(theta) * std::sin(phi);
  R(2, 1) = 0.0, R(2, 2) = std::cos(theta), R(2, 3) = -std::sin(theta);
  R(3, 1) = -std::sin(phi), R(3, 2) = std::sin(theta) * std::cos(phi), R(3, 3) = std::cos(theta) * std::cos(phi);
  if (R(3, 3) < 0)
    for (int i = 1; i <= 3; ++i) {
      R(i, 3) = -R(i, 3);
      R(i, 2) = -R(i, 2);
    }
  if (info) {
    info->nk = nk;
    info->nn = nn;
    info->ii_best = ib + 1;
    info->attempt = attempt;
    info->xi_status = xi_status;
    info->n_recheck = n_recheck;
    info->ss_best = ss_best;
    info->theta = theta;
    info->phi = phi;
    info->scan_ms = ms_screen + ms;
    info->screen_ms = ms_screen;
    info->n_fp64 = nc;
  }
  return ST_OK;
}

// ---- findFoilThickness (Lib_DynamicalTwoBeamImaging.f90:486-564) on the GPU -------------

int foil_thickness(st_d2bi* t, st_ctx* ctx, const double* d_x, int64_t ldx, int64_t n, const Mat3& RU, double* d,
                   double* zbar, double* zsig, double* ms) {
  t->transformed_supercell_with(RU);  // delta and the replicas under RU; d = the cuboid sides
  double dd[3] = {t->vsd[0], t->vsd[1], t->vsd[2]};
  std::memcpy(d, dd, sizeof dd);
  const double cx = std::max(1.0, std::round(dd[0] / (3 * t->a0))), cy = std::max(1.0, std::round(dd[1] / (3 * t->a0)));
  if (!(cx * cy <= (double)(1 << 24))) return stem::ctx_fail(ctx, ST_ERR_ARG, "foil thickness: column grid too large");
  const int Nx = (int)cx, Ny = (int)cy;
  stem::FoilGrid f;
  std::memcpy(f.RU, RU.m, sizeof f.RU);
  std::memcpy(f.delta, t->delta, sizeof f.delta);
  const Mat3 A = t->super.super_a();
  for (int nn = 0; nn < t->nuvw; ++nn)
    for (int i = 1; i <= 3; ++i)
      f.Ruvw[3 * nn + i - 1] = t->uvw[3 * nn] * A(i, 1) + t->uvw[3 * nn + 1] * A(i, 2) + t->uvw[3 * nn + 2] * A(i, 3);
  f.ddx = Nx / dd[0];
  f.ddy = Ny / dd[1];
  f.id3 = 1 / dd[2];
  f.Nx = Nx;
  f.Ny = Ny;
  f.nuvw = t->nuvw;
  const size_t cells = (size_t)Nx * Ny;
  double* scratch = nullptr;
  cudaError_t e = stem::ctx_tilt_scratch(ctx, 2 * cells, &scratch);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "foil scratch");
  auto* d_top = reinterpret_cast<unsigned long long*>(scratch);
  auto* d_thick = d_top + cells;
  const cudaStream_t st = stem::ctx_stream(ctx, nullptr);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], st);
  if (e == cudaSuccess) e = stem::launch_foil_thickness(f, d_x, ldx, n, d_top, d_thick, kHuge1, -kHuge1, st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
  std::vector<unsigned long long> top(cells), thick(cells);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(top.data(), d_top, cells * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(thick.data(), d_thick, cells * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float t_ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t_ms, ev[0], ev[1]);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return stem::ctx_cuda_fail(ctx, e, "foil thickness");
  if (ms) *ms = t_ms;
  double zb = 0.0, z2 = 0.0;
  int nn = 0;
  for (size_t c = 0; c < cells; ++c) {  // ix fastest, as the reference's loops
    const double tp = stem::order_key_value(top[c]), th0 = stem::order_key_value(thick[c]);
    const double th = th0 > tp ? th0 - tp : 0.0;
    if (th == 0) continue;
    zb = zb + th;
    z2 = z2 + th * th;
    nn = nn + 1;
  }
  zb = zb / nn;
  z2 = z2 / nn;
  z2 = std::sqrt(std::max(0.0, z2 - zb * zb));
  *zbar = zb;
  *zsig = z2;
  return ST_OK;
}

// setSupercellTilt1 (:795-939) for integer ng
int tilt1(st_d2bi* t, st_ctx* ctx, int ng, const char* xifile, double theta_max_deg, double rho_max,
          const double* d_x, int64_t ldx, int64_t n, st_tilt_info* info) {
  int hkl[3];
  for (int i = 0; i < 3; ++i) hkl[i] = (int)std::lround(ng * t->g[i]);
  double zbar = 0.0, zsig = 0.0, foil_ms = 0.0;
  if (d_x) {
    const double hd[3] = {(double)hkl[0], (double)hkl[1], (double)hkl[2]};
    t->U = rotate_to_standard_frame(t->k, t->a_cell, hd);
    double dd[3];
    const int rc = foil_thickness(t, ctx, d_x, ldx, n, t->U, dd, &zbar, &zsig, &foil_ms);
    if (rc != ST_OK) return rc;
    if (zbar + 2 * t->a0 > dd[2]) zbar = dd[2];
  } else {
    zbar = t->vsd[2];
  }
  t->foilThickness = zbar;
  const double vv = stem_geom::velocity(t->E * 1000);
  double z = std::fabs(t->foilThickness);
  int rc = best_rotation(ctx, vv, t->k, t->a_cell, t->latt, hkl, xifile, z, theta_max_deg, rho_max, t->U, t->R,
                         info);
  if (rc != ST_OK) return rc;
  z = std::fabs(t->foilThickness / t->R(3, 3));
  const int gi[3] = {(int)std::lround(t->g[0]), (int)std::lround(t->g[1]), (int)std::lround(t->g[2])};
  const double th = tilt_to_dark_field(stem_geom::velocity(t->E * 1000), t->a_cell, gi, t->xig, z, theta_max_deg,
                                       t->U, t->R);
  if (info) {
    info->foil = t->foilThickness;
    info->foil_sigma = zsig;
    info->dark_theta = th;
    info->foil_ms = foil_ms;
  }
  t->vsd[2] = std::fabs(t->vsd[2] / t->R(3, 3));
  t->transformed_supercell();
  t->sg = t->deviation(t->aperture(nullptr));
  return ST_OK;
}

}  // namespace

extern "C" {

int st_d2bi_set_lattice(st_d2bi* h, int32_t lattice) {
  if (!h || lattice < ST_LATTICE_SC || lattice > ST_LATTICE_HCP) return ST_ERR_ARG;
  h->latt = lattice;
  return ST_OK;
}

int st_d2bi_set_supercell_tilt1a(st_d2bi* t, st_ctx* ctx, double ng, const char* xifile, double theta_max,
                                 double rho_max, const double* d_x, int64_t ldx, int64_t n, st_tilt_info* info) {
  if (!t || !ctx) return ST_ERR_ARG;
  if (!(ng >= 0) || !(theta_max > 0) || !(rho_max > 0) || (d_x && (ldx < 3 || n < 1)))
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid tilt search arguments");
  if (info) *info = st_tilt_info{};
  const double dd[3] = {t->vsd[0], t->vsd[1], t->vsd[2]};
  int rc = tilt1(t, ctx, (int)std::floor(ng), xifile, theta_max, rho_max, d_x, ldx, n, info);
  if (rc != ST_OK) return rc;
  const Quat q1 = rotmat_to_quaternion(t->R);
  Quat q2 = q1;
  if (ng - std::floor(ng) > 1.0e-4) {
    std::memcpy(t->vsd, dd, sizeof dd);
    rc = tilt1(t, ctx, (int)std::ceil(ng), xifile, theta_max, rho_max, d_x, ldx, n, nullptr);
    if (rc != ST_OK) return rc;
    q2 = rotmat_to_quaternion(t->R);
  }
  t->R = quaternion_to_rotmat(slerp(q1, q2, ng - std::floor(ng)));
  t->vsd[2] = std::fabs(dd[2] / t->R(3, 3));
  t->transformed_supercell();
  t->sg = t->deviation(t->aperture(nullptr));
  return ST_OK;
}

int st_find_best_rotation(st_ctx* ctx, double v, const double* z0, const double* a_cell, int32_t lattice,
                          const int32_t* hkl, const char* xifile, double foil, double theta_max, double rho_max,
                          double* U, double* R, st_tilt_info* info) {
  if (!ctx) return ST_ERR_ARG;
  if (!z0 || !a_cell || !hkl || !U || !R || !(v > 0) || !(theta_max > 0) || !(rho_max > 0))
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid tilt search arguments");
  if (info) *info = st_tilt_info{};
  const int h[3] = {hkl[0], hkl[1], hkl[2]};
  Mat3 Um, Rm;
  const int rc = best_rotation(ctx, v, z0, Mat3::from(a_cell), lattice, h, xifile, foil, theta_max, rho_max, Um, Rm,
                               info);
  if (rc != ST_OK) return rc;
  std::memcpy(U, Um.m, sizeof Um.m);
  std::memcpy(R, Rm.m, sizeof Rm.m);
  return ST_OK;
}

int st_tilt_scores(st_ctx* ctx, double v, const double* khat, int32_t nk, const double* ghkl, const double* xi_g,
                   int32_t nn, double foil, double* scores) {
  if (!ctx) return ST_ERR_ARG;
  if (!khat || !ghkl || !xi_g || !scores || nk < 1 || nn < 2)
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid tilt score arguments");
  return gpu_scores(ctx, v, khat, nk, ghkl, xi_g, nn, foil, scores, nullptr);
}

int st_tilt_screen(st_ctx* ctx, double v, const double* khat, int32_t nk, const double* ghkl, const double* xi_g,
                   int32_t nn, double foil, double* scores, double* bounds) {
  if (!ctx) return ST_ERR_ARG;
  if (!khat || !ghkl || !xi_g || !scores || !bounds || nk < 1 || nn < 2)
    return stem::ctx_fail(ctx, ST_ERR_ARG, "invalid tilt screen arguments");
  std::vector<double> s32, b32;
  const int rc = gpu_screen(ctx, v, khat, nk, ghkl, xi_g, nn, foil, s32, b32, nullptr);
  if (rc != ST_OK) return rc;
  std::copy(s32.begin(), s32.end(), scores);
  std::copy(b32.begin(), b32.end(), bounds);
  return ST_OK;
}

int st_tilt_to_dark_field(double v, const double* a_cell, const int32_t* hkl, double xi0, double xig, double foil,
                          double theta_max, const double* U, double* R, double* theta) {
  (void)xi0;  // b0 = 1 / xi0 is computed by the reference but does not enter the search
  if (!a_cell || !hkl || !U || !R || !(theta_max > 0)) return ST_ERR_ARG;
  const int h[3] = {hkl[0], hkl[1], hkl[2]};
  Mat3 Rm = Mat3::from(R);
  const double th = tilt_to_dark_field(v, Mat3::from(a_cell), h, xig, foil, theta_max, Mat3::from(U), Rm);
  std::memcpy(R, Rm.m, sizeof Rm.m);
  if (theta) *theta = th;
  return ST_OK;
}

int st_read_extinction_distances(const char* path, int32_t n, const int32_t* hkl, int32_t symmetry, double* xi_g,
                                 int32_t* status) {
  if (!path || n < 0 || (n > 0 && (!hkl || !xi_g)) || !status ||
      (symmetry != ST_SYMMETRY_CUBIC && symmetry != ST_SYMMETRY_HEXAGONAL))
    return ST_ERR_ARG;
  std::vector<int> h(hkl, hkl + 3 * (size_t)n);
  *status = read_extinction_distances(path, n, h.data(), symmetry, xi_g);
  return ST_OK;
}

int st_permitted_reflections(int32_t lattice, double rho, int32_t* hkl, int32_t cap, int32_t* n) {
  if (!n || !(rho >= 0) || rho > 1000 || lattice < 0 || lattice > ST_LATTICE_HCP || cap < 0) return ST_ERR_ARG;
  std::vector<int> tmp(3 * (size_t)std::max(cap, 0));
  *n = permitted_reflections(lattice, rho, hkl ? tmp.data() : nullptr, hkl ? cap : 0);
  if (hkl)
    for (int i = 0; i < 3 * std::min(cap, *n); ++i) hkl[i] = tmp[i];
  return ST_OK;
}

int st_rotmat_to_quaternion(const double* R, double* q) {
  if (!R || !q) return ST_ERR_ARG;
  const Quat r = rotmat_to_quaternion(Mat3::from(R));
  q[0] = r.w, q[1] = r.x, q[2] = r.y, q[3] = r.z;
  return ST_OK;
}

int st_quaternion_to_rotmat(const double* q, double* R) {
  if (!q || !R) return ST_ERR_ARG;
  const Mat3 m = quaternion_to_rotmat(Quat{q[0], q[1], q[2], q[3]});
  std::memcpy(R, m.m, sizeof m.m);
  return ST_OK;
}

int st_slerp(const double* q1, const double* q2, double x, double* q) {
  if (!q1 || !q2 || !q) return ST_ERR_ARG;
  const Quat r = slerp(Quat{q1[0], q1[1], q1[2], q1[3]}, Quat{q2[0], q2[1], q2[2], q2[3]}, x);
  q[0] = r.w, q[1] = r.x, q[2] = r.y, q[3] = r.z;
  return ST_OK;
}

}  // extern "C"
