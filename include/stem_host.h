/*
 * libstem host mirror -- the reference's Fortran host-side set-up of one
 * image, restated in C++ behind a C ABI.
 *
 * In the reference these routines stay in Fortran and a Fortran caller of
 * libstem keeps them; they are here because neither machine of this build has
 * a Fortran compiler, and they give C, C++ and Python callers the reference's
 * DynamicalTwoBeamImaging type API (src/Lib_DynamicalTwoBeamImaging.f90:31-48)
 * on top of st_image.  Each function names the routine it mirrors.
 * Matrices are 3x3 column-major.
 */
#ifndef STEM_HOST_H
#define STEM_HOST_H

#include <stdint.h>

#include "stem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct st_d2bi st_d2bi; /* type(DynamicalTwoBeamImaging) */

/* DynamicalTwoBeamImaging_ctor0 (Lib_DynamicalTwoBeamImaging.f90:145-166):
 * super = SimpleSupercell(a_vox, Nx, Ny, Nz) of the input cell, a0, beam k
 * [uvw], reflection g [hkl], voltage E (keV), voxel subdivisions mxy, mzz. */
int st_d2bi_create(st_d2bi** h, const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double a0, const double* k,
                   const double* g, double E, int32_t mxy, int32_t mzz);
void st_d2bi_destroy(st_d2bi* h);
/* setConventionalUnitCell (:433-441) */
int st_d2bi_set_conventional_unit_cell(st_d2bi* h, const double* a_cell);
/* setVoxelSupercellSize2 (:349-430); all three sides must be nonzero */
int st_d2bi_set_voxel_supercell_size(st_d2bi* h, const double* cuboid_sides);
/* setDeviationParameter (:267-274) */
int st_d2bi_set_deviation_parameter(st_d2bi* h, double sg);
/* setSupercellTilt0 (:567-792) */
int st_d2bi_set_supercell_tilt0(st_d2bi* h);
/* setSupercellTilt2 (:1048-1122) */
int st_d2bi_set_supercell_tilt2(st_d2bi* h, const double* U, const double* R);
/* setExtinctionDistances (:337-345) */
int st_d2bi_set_extinction_distances(st_d2bi* h, double xi0, double xig);
/* setUseDensityField2 (:1127-1134) */
int st_d2bi_set_use_density_field(st_d2bi* h, int32_t use);
/* findImageParameters (:450-482) */
int st_d2bi_find_image_parameters(const st_d2bi* h, double* aperpx, double* xmax, double* modg, int32_t* Mx,
                                  int32_t* My, int32_t* Mz);
/* getRotation (:254-263) */
int st_d2bi_get_rotation(const st_d2bi* h, double* U, double* R);
/* getDeviationParameter without g (:292-307) */
double st_d2bi_get_deviation_parameter(const st_d2bi* h);
/* The prologue of computeD2BI_img (:1635-1852) for process `rank` of
 * `nprocs` and patch jj: the st_image geometry and aa(1:nPrec). */
int st_d2bi_image_geometry(const st_d2bi* h, int64_t nAtoms, int32_t nprocs, int32_t jj, double precAngle,
                           int32_t nPrec, st_geom* geom, double* aa);

/* The same for an arbitrary pixel window [ix0, ix0 + Dx) x [iy0, iy0 + Dy) (clipped to the
 * image): the link-cell box of a patch of that size at that origin.  No counterpart in the
 * reference, whose patches come from the process split; used to recompute chosen tiles of
 * an image (the corrector's fallback). */
int st_d2bi_window_geometry(const st_d2bi* t, int64_t nAtoms, int32_t ix0, int32_t iy0, int32_t Dx, int32_t Dy,
                            double precAngle, int32_t nPrec, st_geom* G, double* aa);
/* computeD2BI_img (:1563-1998) on one process through st_image: the
 * precession-averaged dark-field image (Mx x My, column-major). */
int st_d2bi_compute_img(const st_d2bi* h, st_ctx* ctx, const double* x, int64_t ldx, int64_t nAtoms,
                        double precAngle, int32_t nPrec, int32_t flags, double* img);

/* d2bi program helpers (src/d2bi.f90) */
/* wrapPBC of the atoms read from file (:856-866); x is (ldx, n), in place */
int st_wrap_pbc(const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double* x, int64_t ldx, int64_t n);
/* atom extents after rotateToStandardFrame(k, a_cell, g) (:1201-1223) */
int st_atom_extents(const double* k, const double* g, const double* a_cell, const double* x, int64_t ldx, int64_t n,
                    double* d);
/* tomography tilt R = Rx(theta) R0 for step nn of nTomo (:1365-1372) */
int st_tomography_tilt(double tomoAngle, int32_t nn, int32_t nTomo, const double* R0, double* R);

/* The two passes over the atoms on the GPU, with the host versions' bits.  st_wrap_pbc
 * on device positions d_x (ldx, n), in place, enqueued on stream (0: the context's).
 * st_atom_extents for n_cond conditions (k, g: 3 n_cond values each; 1 <= n_cond <= 32)
 * in one pass over the device positions; d: 3 n_cond host values; waits for the result.
 * For a tomography sweep the atoms are wrapped once and the extents depend only on
 * (k, g), not on the tilt. */
int st_wrap_pbc_device(st_ctx* ctx, const double* a_vox, int32_t Nx, int32_t Ny, int32_t Nz, double* d_x,
                       int64_t ldx, int64_t n, void* stream);
int st_atom_extents_device(st_ctx* ctx, int32_t n_cond, const double* k, const double* g, const double* a_cell,
                           const double* d_x, int64_t ldx, int64_t n, double* d);

/* ---- the -ng tilt search: setSupercellTilt1a / setSupercellTilt1
 * (Lib_DynamicalTwoBeamImaging.f90:795-1045), findBestRotationMatrix and tiltToDarkField
 * (Lib_DiffractionConditions.f90:129-357, 751-927).  The scores of every candidate beam
 * direction against every permitted reflection are computed on the GPU: an FP32 screen of
 * every direction with a bound on its error, then the reference's FP64 arithmetic for the
 * directions that can be within that bound of the best; the host takes the best,
 * re-scoring in the reference's own arithmetic every candidate within the FP64 scores'
 * error bound of it, so that the chosen direction is the one the reference's arithmetic
 * chooses. */

/* Lattice types (Lib_Lattices.f90:65-69) and table symmetries (Lib_ReadExtinctionDistances.f90:20-22) */
#define ST_LATTICE_SC 1
#define ST_LATTICE_BCC 2
#define ST_LATTICE_FCC 3
#define ST_LATTICE_HCP 4
#define ST_SYMMETRY_CUBIC 1
#define ST_SYMMETRY_HEXAGONAL 2

/* What a tilt search did. */
typedef struct {
  int32_t nk;          /* candidate incident vectors (findAllEulerAngles) */
  int32_t nn;          /* permitted reflections within RHO_MAX */
  int32_t ii_best;     /* 1-based index of the chosen incident vector */
  int32_t attempt;     /* 1: THETA_MAX, 2: doubled, 3: no phi limit */
  int32_t xi_status;   /* readExtinctionDistance: 1 all found, 0 some missing, -1 no file */
  int32_t n_recheck;   /* candidates re-scored on the host */
  double ss_best;      /* the chosen score */
  double theta, phi;   /* the tilt angles of the chosen direction (rad) */
  double foil;         /* foil thickness used (A) */
  double foil_sigma;   /* spread of the column thickness with atoms given (A) */
  double dark_theta;   /* tiltToDarkField's tilt about y (rad) */
  double scan_ms;      /* GPU time of the scoring launches, screen and FP64 (CUDA events) */
  double foil_ms;      /* GPU time of the foil-thickness pass (with atoms given) */
  int32_t n_fp64;      /* directions scored in FP64 after the FP32 screen */
  int32_t pad0;
  double screen_ms;    /* GPU time of the FP32 screen alone */
} st_tilt_info;

/* type(Lattice) of the imaging object (the d2bi -lattice option; default bcc) */
int st_d2bi_set_lattice(st_d2bi* h, int32_t lattice);
/* setSupercellTilt1a(this, ng, extinction_distances_filename [, x]) with the module
 * globals THETA_MAX (deg) and RHO_MAX.  d_x: NULL, or the atoms (ldx, n) in device memory
 * for the foil thickness from the atoms (d2bi -surf).  info may be NULL. */
int st_d2bi_set_supercell_tilt1a(st_d2bi* h, st_ctx* ctx, double ng, const char* xifile, double theta_max,
                                 double rho_max, const double* d_x, int64_t ldx, int64_t n, st_tilt_info* info);
/* findBestRotationMatrix(v, z0, A_cell, latt, hkl, U, R, xifile, foil_thickness):
 * U and R column-major. */
int st_find_best_rotation(st_ctx* ctx, double v, const double* z0, const double* a_cell, int32_t lattice,
                          const int32_t* hkl, const char* xifile, double foil, double theta_max, double rho_max,
                          double* U, double* R, st_tilt_info* info);
/* The scores alone: khat (3, nk) incident vectors against reflections ghkl (3, nn) with
 * extinction distances xi_g (nn), for velocity v and foil thickness foil; scores[nk]
 * (host arrays).  The first two reflections are not scored (the reference's [000] and
 * [hkl] slots) and xi_g[0] is the xi_0 of every term. */
int st_tilt_scores(st_ctx* ctx, double v, const double* khat, int32_t nk, const double* ghkl, const double* xi_g,
                   int32_t nn, double foil, double* scores);
/* The FP32 screen of the same scores: scores[nk] and bounds[nk] with |scores - the FP64
 * scores| <= bounds (the search scores in FP64 only the directions this leaves open). */
int st_tilt_screen(st_ctx* ctx, double v, const double* khat, int32_t nk, const double* ghkl, const double* xi_g,
                   int32_t nn, double foil, double* scores, double* bounds);
/* tiltToDarkField(v, A_cell, hkl, xi0, xig, foil_thickness, U, R): R updated in place;
 * theta (may be NULL) receives the tilt about y. */
int st_tilt_to_dark_field(double v, const double* a_cell, const int32_t* hkl, double xi0, double xig, double foil,
                          double theta_max, const double* U, double* R, double* theta);
/* readExtinctionDistance (Lib_ReadExtinctionDistances.f90:29-109): xi_g of n reflections
 * hkl (3, n) under the table symmetry; *status 1 all found, 0 some missing (those
 * keep huge(1.0)), -1 no file or no header. */
int st_read_extinction_distances(const char* path, int32_t n, const int32_t* hkl, int32_t symmetry, double* xi_g,
                                 int32_t* status);
/* permittedReflections (Lib_Lattices.f90:678-735): *n reflections with |hkl| <= rho;
 * the first cap are written to hkl (3, cap) when hkl is not NULL. */
int st_permitted_reflections(int32_t lattice, double rho, int32_t* hkl, int32_t cap, int32_t* n);
/* Lib_Quaternions.f90 RotMatToQuaternion (:246-288; LAPACK DSYEV's dominant eigenvector
 * restated as a Jacobi eigen-solve), quaternionToRotMat (:290-321), slerp (:526-564);
 * q = (w, x, y, z). */
int st_rotmat_to_quaternion(const double* R, double* q);
int st_quaternion_to_rotmat(const double* q, double* R);
int st_slerp(const double* q1, const double* q2, double x, double* q);

#ifdef __cplusplus
}
#endif

#endif
