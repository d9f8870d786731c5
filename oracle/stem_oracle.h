/*
 * ORACLE -- test infrastructure only.
 *
 * CPU restatement, in plain C, of simulated_tem's imaging hot path
 * (src/Lib_DynamicalTwoBeamImaging.f90 computeD2BI_img and its callees, the
 * link-cell list of src/Lib_LinkCell3D.f90, the geometry helpers of
 * src/Lib_SimpleSupercells.f90 and src/Lib_DiffractionConditions.f90, and the
 * PNG blur of src/d2bi.f90).  Only the tests, the smoke check and the CPU
 * baseline leg of the benchmark may load it, and only as the checker: the
 * product path never calls into this library.
 *
 * Parity pins: the reference's shipped 94x94 dark-field image, its 16-bit PNG,
 * the stored neighbour list of test/testLib_LinkCell3D.f90, the electron
 * wavelength of test/testLib_RelativisticElectrons.f90 and the analytic
 * perfect-crystal intensity (intensityAtDepthZ).  The reference itself is
 * Fortran and no Fortran compiler exists on either machine, so there is no
 * compiled reference to run beside this restatement.
 *
 * Arithmetic follows the reference's left-to-right evaluation order; the
 * library is compiled with -ffp-contract=off so that no multiply-add is fused.
 * Matrices are 3x3 column-major: a(i,j) is a[(i-1) + 3*(j-1)].
 */
#ifndef STEM_ORACLE_H
#define STEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OC_OK 0
#define OC_ERR_ARG 1
#define OC_ERR_CAPACITY 2
#define OC_ERR_ALLOC 3

/* Lattice types (Lib_Lattices.f90:65-69) and the symmetry of their
 * extinction-distance tables (Lib_ReadExtinctionDistances.f90:20-22). */
#define OC_LATTICE_CUSTOM 0
#define OC_LATTICE_SC 1
#define OC_LATTICE_BCC 2
#define OC_LATTICE_FCC 3
#define OC_LATTICE_HCP 4
#define OC_SYM_CUBIC 1
#define OC_SYM_HEX 2

/* SimpleSupercell (Lib_SimpleSupercells.f90:51-55). */
typedef struct {
  int Nx, Ny, Nz;
  double a[9];
  double ia[9];
} oc_super;

/* DynamicalTwoBeamImaging state (Lib_DynamicalTwoBeamImaging.f90:59-84). */
typedef struct {
  double k[3], g[3];
  double a0;
  oc_super super;
  double sg;
  int mxy, mzz;
  double xi0, xig;
  double E;
  int useDensityField;
  oc_super gksuper;
  double delta[3];
  double foilThickness;
  double voxelSupercellDimensions[3];
  int nuvw;
  int uvw[3 * 125];
  double a_cell[9];
  double U[9];
  double R[9];
  int test;
} oc_d2bi;

/* Everything the patch loop of computeD2BI_img consumes, as computed by its
 * prologue (Lib_DynamicalTwoBeamImaging.f90:1635-1852). */
typedef struct {
  int Mx, My, Mz;
  int ix0, ix1, iy0, iy1; /* pixel window of the patch, half open */
  int Ex, Ey, Ez;
  int deltaM, nMax0;
  int nuvw;
  double RU[9];
  double delta[3];
  double Ruvw[3 * 27];
  double lc_delta[3];
  double a_col[9], ia_col[9];
  double a_vox[9];
  double g[3];
  double sigma, cut2, i2s2;
  double deltaz, b0, bg;
  int useDensity;
} oc_geom;

/* Counters of the work done, for the roofline and the tests. */
typedef struct {
  int64_t n_kept;      /* atoms binned into the link cells */
  int64_t n_tests;     /* candidate pairs examined by the 27-cell search */
  int64_t n_accepted;  /* pairs with r^2 <= (3 sigma)^2 */
  int64_t n_voxels;
  int max_cell_count;
} oc_stats;

/* Command-line level inputs of d2bi for one diffraction condition
 * (src/d2bi.f90:190-451). */
typedef struct {
  double a_super[9];  /* supercell from the input file */
  double a0in;        /* -a0 (cubic lattice: one value) */
  double k[3], g[3];  /* -k, -g */
  double V;           /* -V (keV) */
  int M[2];           /* -M */
  int tilt_mode;      /* 0: sg = 0 default, 1: -sg, 2: -R [-U] */
  double sg;          /* -sg */
  int haveU;
  double U[9], R[9];  /* -U, -R (column major) */
  int haveD;
  double d0[3];       /* -d */
  double xi0, xig;    /* -xi0, -xig */
  int useDensity;     /* -density */
  int nPrec;          /* -nPrecAngle */
  double precAngle;   /* -precAngle */
  int nTomo;          /* -nTomoAngle */
  double tomoAngle;   /* -tomoAngle (deg) */
  int dark;           /* -dark */
  double ng;          /* -ng (tilt_mode 3) */
  int lattice;        /* -lattice: OC_LATTICE_* */
  int surf;           /* -surf: foil thickness from the atoms */
  double thetaMax;    /* -theta: THETA_MAX (deg) */
  double rhoMax;      /* RHO_MAX */
  char xifile[512];   /* -xifile ("" when absent) */
} oc_args;

/* What the tilt search found (findBestRotationMatrix and setSupercellTilt1). */
typedef struct {
  int nk;           /* incident vectors scored */
  int nn;           /* permitted reflections */
  int ii_best;      /* 1-based index of the best incident vector */
  int attempt;      /* 1: THETA_MAX, 2: doubled, 3: no phi limit */
  int xi_ok;        /* readExtinctionDistance: 1 all found, 0 some missing, -1 no file */
  double ss_best;   /* its score */
  double theta, phi;
  double foil;        /* foil thickness used */
  double foil_sigma;  /* spread of the column thickness (with -surf) */
  double dark_theta;  /* tiltToDarkField's tilt about y */
} oc_tilt_info;

/* --- Lib_SimpleSupercells / Lib_DiffractionConditions / Lib_RelativisticElectrons --- */
double oc_norm2(const double* v);
double oc_det3(const double* M);
void oc_inv3(const double* M, double* N);
void oc_super_ctor(oc_super* s, const double* a, int Nx, int Ny, int Nz);
void oc_wrap_pbc(const oc_super* s, const double* y, double* yp);
double oc_wavelength(double V);
double oc_velocity(double V);
double oc_intensity_at_depth(double xi0, double xig, double sg, double z);
void oc_rotate_to_standard_frame(const double* z0, const double* A_cell, const double* hkl, double* U);

/* --- Lib_DynamicalTwoBeamImaging type API --- */
void oc_d2bi_ctor(oc_d2bi* t, const oc_super* super, double a0, const double* k, const double* g, double E,
                  int mxy, int mzz);
void oc_set_conventional_unit_cell(oc_d2bi* t, const double* a_cell);
int oc_set_voxel_supercell_size(oc_d2bi* t, const double* cuboidSides);
void oc_set_deviation_parameter(oc_d2bi* t, double sg);
void oc_set_supercell_tilt0(oc_d2bi* t);
void oc_set_supercell_tilt2(oc_d2bi* t, const double* U, const double* R);
void oc_set_extinction_distances(oc_d2bi* t, double xi0, double xig);
void oc_set_use_density_field(oc_d2bi* t, int is);
void oc_get_aperture(const oc_d2bi* t, const double* beamTilt, double* g);
double oc_get_deviation_parameter(const oc_d2bi* t, const double* g);
void oc_find_image_parameters(const oc_d2bi* t, double* aperpx, double* xmax, double* modg, int* Mx, int* My,
                              int* Mz);

/* Prologue of computeD2BI_img: geometry of patch (jx, jy) and the precession
 * scattering parameters aa[nPrec] (Lib_DynamicalTwoBeamImaging.f90:1635-1852). */
int oc_image_geometry(const oc_d2bi* t, int64_t nAtoms, int nProcs, int jj, double precAngle, int nPrec,
                      oc_geom* geom, double* aa);

/* Patch loop of computeD2BI_img for one patch: findGdotR, the voxel phase sums
 * and the column integrations.  Adds sum_prec |phi_g|^2 into img (column-major
 * Mx x My) over the patch window.  nthreads > 1 runs the pixel rows on OpenMP
 * threads; the result does not depend on the thread count. */
int oc_patch_image(const oc_geom* geom, const double* aa, int nPrec, const double* x, int64_t ldx, int64_t nAtoms,
                   double* img, oc_stats* stats, int nthreads);

/* Same, restricted to pixel rows [iy_lo, iy_hi) of the patch (used for a
 * bounded CPU timing sample). */
int oc_patch_image_rows(const oc_geom* geom, const double* aa, int nPrec, const double* x, int64_t ldx,
                        int64_t nAtoms, int iy_lo, int iy_hi, double* img, oc_stats* stats, int nthreads);

/* The whole of computeD2BI_img with one process: all patches, then the
 * average over precession angles (Lib_DynamicalTwoBeamImaging.f90:1563-1998). */
int oc_compute_d2bi_img(const oc_d2bi* t, const double* x, int64_t ldx, int64_t nAtoms, double precAngle,
                        int nPrec, double* img, oc_stats* stats, int nthreads);

/* The column integrator (Lib_DynamicalTwoBeamImaging.f90:2316-2480); x is
 * complex interleaved (re, im) of length nz+1, rho of length nz+1. */
double oc_integrate_column(double a, double b0, double bg, double dz, const double* x, const double* rho, int nz);

/* findGdotR into a link-cell list, then the neighbour list of one point:
 * returns the count and fills ids (1-based) and r2 in the reference's order. */
int oc_neighbour_list(const oc_super* lc, const double* pts, int npts, int nMax0, const double* query,
                      double cutoff, int* ids, double* dx, double* r2, int maxn, int* max_count);

/* --- d2bi (src/d2bi.f90) --- */
/* wrapPBC of the atoms and the d2bi setup of one diffraction condition,
 * tomography step nn (0-based).  x is (ldx, nAtoms), wrapped in place. */
int oc_d2bi_setup(const oc_args* args, double* x, int64_t ldx, int64_t nAtoms, int nn, oc_d2bi* t,
                  double* aperpx_out);
/* gaussianBlurImage (src/d2bi.f90:1543-1624). */
void oc_gaussian_blur(const double* f_in, int Nx, int Ny, double t, double* f_out);
/* write_greyscale_png normalise=.true. quantisation (Lib_Png.f90:117-181,
 * Lib_Greyscale.c:234-241): png[y*Nx + x] = 16-bit level of img(x, y). */
void oc_png_levels(const double* img, int Nx, int Ny, uint16_t* levels);
/* outputImgAsPng's contrast mode (src/d2bi.f90:1531-1535), then write_greyscale_png
 * with normalise=.false.: the levels of clamp((v - lo) / (hi - lo), 0, 1). */
void oc_png_levels_window(const double* img, int Nx, int Ny, double lo, double hi, uint16_t* levels);
/* The '(1000f12.7)' records of d2bi's .dat file (src/d2bi.f90:1455): every value in
 * Fortran F12.7 editing, a newline after each 1000 values and after the last; returns
 * the number of bytes written to out. */
long long oc_format_f12_7(const double* v, long long n, char* out);
/* input_lammps (src/Lib_XYZFiles.f90:1108-1117): from byte offset `offset` of the file,
 * n_atoms lines read as id, type, x, y, z (strtod-rounded); x(3, n), types(n).  Returns
 * 0, or 1 + the 0-based index of the first line that does not hold five values. */
long long oc_read_lammps_atoms(const char* path, long long offset, long long n_atoms, double* x, int* types);

/* --- the -ng tilt search --- */
/* readExtinctionDistance (Lib_ReadExtinctionDistances.f90:29-109): xi_g of the
 * n reflections hkl(3, n); 1 all found, 0 some missing (xi_g = huge(1.0)),
 * -1 no file or no header. */
int oc_read_extinction_distances(const char* path, const int* hkl, int n, int symm, double* xi_g);
/* permittedReflections (Lib_Lattices.f90:678-735): the number of reflections;
 * the first cap of them go to hkl(3, cap) when hkl is not NULL. */
int oc_permitted_reflections(int latt, double rho, int* hkl, int cap);
/* scoreForIncidentVector1 (Lib_DiffractionConditions.f90:1835-1867). */
double oc_score_incident_vector(double v, const double* khat, const double* ghkl, const double* xi_g, int nn,
                                double foil);
/* findBestRotationMatrix (Lib_DiffractionConditions.f90:129-357). */
int oc_find_best_rotation(double v, const double* z0, const double* A_cell, int latt, const int* hkl,
                          const char* xifile, double foil, double theta_max_deg, double rho_max, double* U,
                          double* R, oc_tilt_info* info, double* scores, double* khat);
/* The permitted g-vectors (after find_gvectors_permittedReflections' swaps) and their
 * extinction distances, as findBestRotationMatrix scores them; returns nn. */
int oc_tilt_reflections(int latt, const double* A_cell, const int* hkl, double rho, const char* xifile,
                        double* ghkl, double* xi_g, int cap);
/* tiltToDarkField (Lib_DiffractionConditions.f90:751-927). */
int oc_tilt_to_dark_field(double v, const double* A_cell, const int* hkl, double xi0, double xig, double foil,
                          double theta_max_deg, const double* U, double* R, double* theta_out);
/* The golden-section search (Lib_GoldenSection.f90) of f over the bracket [x1, x3]:
 * steps when converged, minus the steps when it ran out of them. */
int oc_golden_minimise(double x1, double x3, double (*f)(double, void*), void* arg, double* xt, double* yt);
/* Lib_Quaternions.f90:246-288, 290-321, 526-564; q = (w, x, y, z). */
void oc_rotmat_to_quaternion(const double* R, double* q);
void oc_quaternion_to_rotmat(const double* q, double* R);
void oc_slerp(const double* q1, const double* q2, double x, double* qx);
/* setSupercellTilt1a (Lib_DynamicalTwoBeamImaging.f90:943-1045); x (ldx, nAtoms)
 * or NULL (foil thickness from the box, no -surf). */
int oc_set_supercell_tilt1a(oc_d2bi* t, double ng, const char* xifile, int latt, double theta_max_deg,
                            double rho_max, const double* x, int64_t ldx, int64_t nAtoms, oc_tilt_info* info);

/* --- the .xyz reader --- */
typedef struct {
  long long n_atoms, n_read;
  int n_columns, n_header_lines, lammps, supercell_kind, supercell_ok;
  int repeats[3];
  double a_super[9];
  long long data_offset, file_bytes;
  char column_description[257];
} oc_xyz_info;
/* ParseReal (NBAX_StringTokenizers.f90:303-420): 1 and *r when a number was found. */
int oc_fortran_parse_real(const char* text, int len, double* r);
/* readHeader (Lib_XYZFiles.f90:507-626) and getSupercell0 (:905-1058). */
int oc_xyz_header(const char* path, oc_xyz_info* info);
/* input0 (Lib_XYZFiles.f90:756-892): the species count, or -(1 + the bad line). */
long long oc_read_xyz_atoms(const char* path, long long offset, long long n, int ncols, double* x, int ldx,
                            int* types, char* names, int cap);

#ifdef __cplusplus
}
#endif

#endif
