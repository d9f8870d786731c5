/*
 * libstem -- GB300 (sm_103a) imaging hot path of simulated_tem's d2bi.
 *
 * C ABI: plain pointers and sizes, no C++ or torch types, callable from the
 * reference's Fortran host through iso_c_binding.  Every entry point returns
 * ST_OK (0) or an ST_ERR_* code; st_last_error() gives the message.
 *
 * Reference interfaces these calls replace (paths are within the reference
 * project):
 *   st_image   -- the patch loop of computeD2BI_img,
 *                 src/Lib_DynamicalTwoBeamImaging.f90:1842-1946 (findGdotR,
 *                 the link-cell neighbour sums of :1877-1895 and the column
 *                 integrator dynamicalTwoBeamIntegrationColumn_phaserho
 *                 :2316-2480).  The geometry and precession set-up before it
 *                 (:1635-1836) and the MPI_Reduce and average after it
 *                 (:1950-1951) stay with the caller, exactly as in the
 *                 reference; ST_FLAG_AVERAGE / ST_FLAG_BRIGHT fold the
 *                 single-process average and the bright-field flip of
 *                 src/d2bi.f90:1396 into the call for callers without MPI.
 *   st_blur    -- gaussianBlurImage, src/d2bi.f90:1543-1624 (private to the
 *                 d2bi program, applied to the PNG output only).
 *   st_create / st_destroy -- no counterpart: the library keeps its device
 *                 buffers across calls (tomography steps, conditions).
 *
 * Matrices are 3x3 column-major, as Fortran stores them: m(i,j) is
 * m[(i-1) + 3*(j-1)].  Images are column-major (0:Mx-1, 0:My-1).
 */
#ifndef STEM_H
#define STEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ST_OK 0
#define ST_ERR_ARG 1      /* invalid argument or unsupported geometry */
#define ST_ERR_CAPACITY 2 /* a link cell holds more than 16 x nMax0 atoms (the reference stops there) */
#define ST_ERR_CUDA 3     /* CUDA runtime error */
#define ST_ERR_TIMEOUT 4  /* a bounded device wait ran out */
#define ST_ERR_ALLOC 5    /* device or host allocation failed */

/* flags */
#define ST_FLAG_FP32 0x1    /* FP32 deposition and integration; FP64 binning and g.r reduction */
#define ST_FLAG_AVERAGE 0x2 /* divide by nPrec (the reference's average after MPI_Reduce) */
#define ST_FLAG_BRIGHT 0x4  /* with ST_FLAG_AVERAGE: return 1 - I (bright field) */
#define ST_FLAG_STATS 0x8   /* count candidate tests and accepted pairs (st_get_stats) */

typedef struct st_ctx st_ctx;

/* Per-image geometry: what computeD2BI_img has computed when it enters its
 * patch loop (Lib_DynamicalTwoBeamImaging.f90:1635-1852). */
typedef struct st_geom {
  /* findGdotR transform y = RU (x + Ruvw[n]) + delta, kept if y - lc_delta
   * lies in the link-cell box; phase g . y (:1160-1265) */
  double RU[9];       /* matmul(R, U), no beam tilt: precession changes only aa */
  double delta[3];
  int32_t nuvw;       /* periodic replicas, <= 27 */
  int32_t pad0;
  double Ruvw[81];    /* replica translations uvw(1)*A1 + uvw(2)*A2 + uvw(3)*A3 */
  double g[3];        /* aperture g-vector (includes 2 pi), getAperture(this) */
  /* link cells (:1753-1773) */
  double a_col[9];    /* link-cell vectors a_column */
  double ia_col[9];   /* inverse3Mat(a_column) */
  int32_t Ex, Ey, Ez;
  int32_t nMax0;      /* link-cell capacity estimate (:1681) */
  double lc_delta[3]; /* offset of the link-cell box for this patch (:1852) */
  /* voxels */
  double a_vox[9];    /* getA(gksuper) */
  int32_t Mx, My, Mz;
  int32_t ix0, ix1, iy0, iy1; /* pixel window of the patch, half open */
  int32_t useDensity;
  /* physics */
  double sigma;       /* a0 / 2 */
  double deltaz;      /* xmax(3) / Mz */
  double b0, bg;      /* pi / xi0, pi / xig */
} st_geom;

typedef struct st_stats {
  int64_t n_atoms;     /* input atoms */
  int64_t n_kept;      /* atoms binned into link cells (all replicas) */
  int64_t n_tests;     /* candidate pairs tested (ST_FLAG_STATS) */
  int64_t n_accepted;  /* pairs with r^2 <= (3 sigma)^2 (ST_FLAG_STATS) */
  int64_t n_voxels;    /* voxels of the patch */
  int32_t max_cell_count;
  int32_t n_prec;
  double ms_bin;       /* device time of the binning kernels (ms) */
  double ms_column;    /* device time of the column kernel (ms) */
  int32_t column_kernel; /* 1 general FP32, 2 slab-ring FP32, 3 general FP64, 4 slab-ring FP64 (the
                            slab ring for at least one image) */
  int32_t ring_variant;  /* occupancy variant of the last slab-ring launch, -1 if none ran */
  int32_t ring_slab_atoms; /* staging capacity per slab of the last slab-ring launch (0 if none ran) */
  int32_t n_launches;    /* kernels the call launched (all attempts; autotuning trials included) */
} st_stats;

/* Context on CUDA device `device` (made current for the calls). */
int st_create(st_ctx** ctx, int device);
void st_destroy(st_ctx* ctx);
const char* st_last_error(const st_ctx* ctx);

/* One image from host buffers (synchronous).
 *   x    : atom positions, Fortran x(ldx, nAtoms); only x(1:3, :) is read (ldx >= 3)
 *   aa   : 2 pi s_g for each precession angle, aa(1:nPrec) (:1808-1831)
 *   img  : Mx x My doubles, column-major, fully overwritten: the patch window
 *          holds sum_prec |phi_g|^2 (or the average / bright field by flags),
 *          every other pixel is 0 -- the reference's d2big2 before MPI_Reduce. */
int st_image(st_ctx* ctx, const st_geom* geom, const double* x, int64_t ldx, int64_t nAtoms, const double* aa,
             int32_t nPrec, int32_t flags, double* img);

/* Same with x and img in device memory, on `stream` (a cudaStream_t, or 0 for
 * the context's stream).  Returns after the image is complete. */
int st_image_device(st_ctx* ctx, const st_geom* geom, const double* d_x, int64_t ldx, int64_t nAtoms,
                    const double* aa, int32_t nPrec, int32_t flags, double* d_img, void* stream);

/* Launch tuning of the slab-ring FP32 kernel.  Its variants differ in the warp
 * tile's shape (8 x 4, 4 x 8 or 16 x 2 pixel columns), the slab capacity of
 * the first staging tier (128 or 96 atoms) and with it the CTAs per SM; the
 * images of variants of one tile shape are identical, those of different
 * shapes agree to FP32 rounding (their atoms are summed in different orders).
 * ST_TUNE_AUTO (the default): the first pass of each kind (angles per pass,
 * density) on images of each shape (image and link-cell dimensions) in a
 * context, with at least 4,096 warp tiles, times every variant on the real
 * work, keeps the fastest for the context's later calls on that kind and
 * shape, and leaves that variant's own images.  ST_TUNE_OFF: variant 0 always.
 * mode >= 0: that variant always.  No counterpart in the reference. */
#define ST_TUNE_AUTO (-1)
#define ST_TUNE_OFF (-2)
int st_tune(st_ctx* ctx, int32_t mode);
/* Number of slab-ring variants (valid forced modes are 0 .. count - 1). */
int st_tune_variants(void);
/* A variant's name ("8x4 slab96" ...); "invalid" out of range. */
const char* st_tune_variant_name(int32_t variant);

/* st_image_device restricted to chosen tiles: d_tile_mask (device, one byte per mask_T x
 * mask_T pixel tile, ceil(Mx / mask_T) tiles per row, row-major) selects the tiles whose
 * columns are computed; the other pixels are left 0.  mask_T a multiple of 8, the
 * geometry's window origin a multiple of 8 (x) and 4 (y).  The binning is that of the
 * whole window.  Used to recompute only the tiles a faster estimate cannot be trusted on
 * (the learned corrector's fallback).  No counterpart in the reference. */
int st_image_device_masked(st_ctx* ctx, const st_geom* geom, const double* d_x, int64_t ldx, int64_t nAtoms,
                           const double* aa, int32_t nPrec, int32_t flags, double* d_img,
                           const unsigned char* d_tile_mask, int32_t mask_T, void* stream);

/* One image of a batch: its geometry, its atoms, its precession parameters
 * aa(1:nPrec) in host memory, and its output.  x and img are device pointers
 * for st_batch_device and host pointers for st_batch. */
typedef struct st_job {
  const st_geom* geom;
  const double* x; /* (ldx, nAtoms) */
  int64_t ldx;
  int64_t nAtoms;
  const double* aa;
  int32_t nPrec;
  int32_t pad0;
  double* img; /* Mx x My column-major, overwritten as by st_image */
} st_job;

/* Many images in one call: tomography tilts, precession sets, g-vectors or
 * independent cells of uneven size.  No counterpart in the reference, which
 * images one condition per computeD2BI_img call; each image is the one
 * st_image_device makes for its job.  The binning runs once over the
 * candidates of all jobs and, on the FP32 path, the columns of all jobs run
 * as one persistent launch that hands out warp tiles from a global counter.
 * A batch of 2^31 or more candidates (nuvw x nAtoms summed over its jobs) runs
 * as consecutive groups below that size.  flags apply to every job.  Returns
 * after every image is complete; st_get_stats then sums over the batch. */
int st_batch_device(st_ctx* ctx, int32_t n_jobs, const st_job* jobs, int32_t flags, void* stream);

/* st_batch_device from host buffers, the call a Fortran driver of a tilt
 * series or a set of cells makes.  Jobs that name the same atoms (same x,
 * ldx and nAtoms) share one device copy, so a tilt series uploads its atoms
 * once.  The images are copied back before it returns. */
int st_batch(st_ctx* ctx, int32_t n_jobs, const st_job* jobs, int32_t flags);

/* A batch recorded as a CUDA graph, for the same images computed again and
 * again (a trajectory whose atoms move, a sweep repeated on new data): the
 * binning, the persistent column launch(es), the epilogues and the read-back
 * of the overflow counters are replayed without host work.  The plan keeps
 * copies of the geometries and aa; the device buffers x and img of the jobs
 * must stay allocated while the plan exists (their contents may change, nAtoms
 * may not).  The plan owns its own device memory (the context's stays free
 * for other calls) and inherits the context's tuning.
 *
 * st_plan_create runs the batch once (the images are then complete) and
 * records it.  st_plan_launch enqueues one replay on `stream` and returns.
 * st_plan_wait waits for it; when the replay's binning outgrew the recorded
 * capacity or a slab overflowed, it recomputes the batch on the eager path
 * (then the images are right) and records the plan again.  No counterpart in
 * the reference. */
typedef struct st_plan st_plan;
int st_plan_create(st_ctx* ctx, int32_t n_jobs, const st_job* jobs, int32_t flags, void* stream, st_plan** plan);
int st_plan_launch(st_plan* plan, void* stream);
int st_plan_wait(st_plan* plan, void* stream);
/* Statistics of the plan's last eager run (counts) or replay (n_kept). */
int st_plan_stats(const st_plan* plan, st_stats* out);
const char* st_plan_last_error(const st_plan* plan);
void st_plan_destroy(st_plan* plan);

/* Gaussian blur of width t pixels (src/d2bi.f90:1543-1624) from host buffers;
 * in and out are nx x ny doubles, column-major; out is overwritten. */
int st_blur(st_ctx* ctx, const double* in, int32_t nx, int32_t ny, double t, double* out);

/* Same in device memory, on `stream` (0: the context's stream). */
int st_blur_device(st_ctx* ctx, const double* d_in, int32_t nx, int32_t ny, double t, double* d_out, void* stream);

/* Counters and kernel times of the last st_image / st_image_device call. */
int st_get_stats(const st_ctx* ctx, st_stats* out);

/* Limits of st_blur_noalloc's fixed scratch (16.8 MB of device memory). */
#define ST_BLUR_NOALLOC_MAX_PIXELS (1 << 21) /* nx * ny <= 2,097,152 */
#define ST_BLUR_NOALLOC_MAX_NX 4096          /* nx <= 4096 */
#define ST_BLUR_NOALLOC_MAX_NK 1023          /* ceiling(5 t) <= 1023, i.e. t <= 204.6 pixels */

/* The blur of st_blur_device for callers that cannot let a library allocate
 * GPU memory: a Fortran host under an MPI or batch runtime that owns the
 * device memory pool, code imaging inside a fixed memory budget, or a caller
 * that must not allocate between steps it later replays.  No counterpart in
 * the reference (its blur runs on the CPU).
 *
 * d_in and d_out are caller-owned device buffers of nx * ny doubles
 * (column-major); the output equals st_blur's bit for bit.  Nothing is
 * allocated: no cudaMalloc, no cudaFree, no allocating library call.  The one
 * intermediate (the x-pass image and its column weights) lives in a fixed
 * file-scope device array that every GPU loading the library holds until the
 * process exits; larger images than the limits above return ST_ERR_ARG with
 * the reason in err.  The first call in each CUDA context (per device, and again
 * after a device reset or under another context) looks that array's device
 * address up (cudaGetSymbolAddress, which may load the library's GPU module):
 * make that first call outside any stream capture.  Calls share the array and
 * it keeps the last call's contents; every entry is rewritten before it is
 * read, but calls whose work overlaps on the GPU (concurrent streams, or
 * threads on one device without ordering) race on it.  The kernels are
 * enqueued on `stream` (a cudaStream_t, 0 for the legacy default stream) and
 * the call returns without waiting.  err (optional, err_len bytes) receives a
 * message on failure. */
int st_blur_noalloc(const double* d_in, int32_t nx, int32_t ny, double t, double* d_out, void* stream, char* err,
                    int32_t err_len);

/* ---- Output files of d2bi: the .dat image and the 16-bit PNG ----------------------
 * The .dat file (src/d2bi.f90:1429-1457): header lines, then '(2i8)' nx ny, then the
 * image column-major in records of '(1000f12.7)'.  The header fields, as d2bi writes
 * them: */
typedef struct st_dat_header {
  char version[32];   /* "# d2bi v.<version>" */
  int32_t miller4;    /* 1: k and g are 4-index (hexagonal) vectors */
  double k[4], g[4];  /* '(a,3f10.3)' or '(a,4f10.3)' */
  double modg;        /* |g| (1/A), '(f12.5)' after g */
  int32_t nM, M[3];   /* '(a,3i8)': the first nM values */
  double V;           /* keV, '(a,3f10.0)' */
  double xi0, xig;    /* A, '(a,3f12.5)' */
  int32_t has_ng;     /* 1: the '# n_g' line ('(a,f8.3)') is written */
  double ng;
  double sg;          /* 1/A, '(a,3f12.5)' */
  double xmax[3];     /* img space (A), '(a,3f12.3)' */
  double aperpx;      /* scale (A/px), '(a,3f12.5)' */
  double rotation[9]; /* matmul(R, U) column-major, '(a,9f12.6)' */
} st_dat_header;

/* The header text (up to and including the '(2i8)' size line) into buf (cap bytes,
 * NUL-terminated); *len = its length.  Host only.  Fortran F editing: rounded to
 * nearest, at least one integer digit when the field has room, a trailing '.' for
 * zero decimals, asterisks when the number does not fit. */
int st_format_dat_header(const st_dat_header* h, int32_t nx, int32_t ny, char* buf, int64_t cap, int64_t* len);

/* Bytes of the '(1000f12.7)' records of n values: 12 n plus a newline per record. */
int64_t st_dat_text_bytes(int64_t n);

/* The '(1000f12.7)' records of n device values d_v into device memory d_text (cap bytes,
 * at least st_dat_text_bytes(n)); enqueued on stream (0: the context's stream),
 * returns without waiting. */
int st_format_dat_device(st_ctx* ctx, const double* d_v, int64_t n, char* d_text, int64_t cap, void* stream);

/* Write a .dat file: header, size line, records (formatted on the GPU).  img is the host
 * image (nx x ny, column-major).  Written to <path>.tmp, then renamed to path. */
int st_write_dat(st_ctx* ctx, const char* path, const st_dat_header* h, const double* img, int32_t nx, int32_t ny);

/* The 16-bit levels of d2bi's PNG output (outputImgAsPng, src/d2bi.f90:1509-1538, and
 * write_greyscale_png, src/Lib_Png.f90:117-181 with src/Lib_Greyscale.c:230-245): with
 * iso_min == iso_max the image is normalised to [0, 1 - 1/65536] by its minimum and
 * maximum, otherwise scaled to (v - iso_min) / (iso_max - iso_min) and clamped to [0, 1];
 * the level is (int)(65536 f) of the FP32 value f clamped to [0, 0.999984741].
 * d_levels: nx * ny native-endian uint16, image order (x fastest).  No blur here (see
 * st_write_png); enqueued on stream, returns without waiting. */
int st_png_levels_device(st_ctx* ctx, const double* d_img, int32_t nx, int32_t ny, double iso_min, double iso_max,
                         uint16_t* d_levels, void* stream);

/* A 16-bit greyscale PNG (no interlace, filter none, zlib stored blocks) of the levels
 * (nx x ny, row y = levels[nx y .. nx y + nx - 1]) into out (cap bytes); *len = the file
 * size.  Host only.  Decoders see the same pixels as in d2bi's PNG files. */
int64_t st_png16_bytes(int32_t nx, int32_t ny);
int st_encode_png16(const uint16_t* levels, int32_t nx, int32_t ny, uint8_t* out, int64_t cap, int64_t* len);

/* d2bi's PNG file of a host image: the blur of width blur_t pixels first when blur_t > 0
 * (gaussianBlurImage), then the levels above, then the PNG; written to <path>.tmp, then
 * renamed to path. */
int st_write_png(st_ctx* ctx, const char* path, const double* img, int32_t nx, int32_t ny, double iso_min,
                 double iso_max, double blur_t);

/* ---- Input: the LAMMPS data files d2bi reads (src/Lib_XYZFiles.f90) ----------------- */
typedef struct st_lammps_info {
  int64_t n_atoms;      /* the "atoms" line */
  int32_t n_types;      /* the "atom types" line */
  int32_t pad0;
  double lo[3], hi[3];  /* the xlo xhi, ylo yhi, zlo zhi lines */
  int64_t data_offset;  /* byte offset of the first atom line */
  int64_t file_bytes;
} st_lammps_info;

/* The header of a LAMMPS data file, read as readHeader_lammps and input_lammps read it
 * (src/Lib_XYZFiles.f90:628-716, 1092-1101).  Host only. */
int st_lammps_header(const char* path, st_lammps_info* info);

/* The atom lines of a LAMMPS Atoms block in device memory (d_text, n_bytes, starting at
 * the first atom line): for atom i, the line's id, type, x, y, z as a list-directed read
 * gives them (src/Lib_XYZFiles.f90:1108-1117): d_x[i ldx + 0..2] = x, y, z (correctly
 * rounded), d_types[i] = type (d_types may be null).  Blanks and commas separate values;
 * the rest of a line is ignored.  A missing or malformed value returns ST_ERR_ARG with the
 * first such line (0-based within the block) in *bad_line (-1 when none).  Waits for the
 * parse to finish. */
int st_parse_atoms_device(st_ctx* ctx, const char* d_text, int64_t n_bytes, int64_t n_atoms, double* d_x,
                          int64_t ldx, int32_t* d_types, int64_t* bad_line, void* stream);

/* The number parser of st_parse_atoms_device, on the host: the correctly rounded FP64 value
 * of the decimal number starting at text (len bytes; Fortran D exponents accepted), *used =
 * the characters it spans.  ST_ERR_ARG for malformed text or a value outside the parser's
 * exact range (normal numbers from about 1e-20 to 1e38). */
int st_parse_real(const char* text, int64_t len, double* out, int32_t* used);

/* A LAMMPS data file into host arrays: x(ldx, n_atoms) rows 0..2 = positions (ldx >= 3;
 * other rows untouched), types (n_atoms values, may be null).  info: the header
 * (st_lammps_header); the atom lines are parsed on the GPU. */
int st_read_lammps(st_ctx* ctx, const char* path, const st_lammps_info* info, double* x, int64_t ldx,
                   int32_t* types);

/* ---- Input: the (extended) .xyz files d2bi reads (src/Lib_XYZFiles.f90:507-626, 756-892,
 * 905-1058) -------------------------------------------------------------------------- */
#define ST_XYZ_SUPERCELL_NONE 0
#define ST_XYZ_SUPERCELL_LATTICE 1  /* extended xyz: Lattice="..." on the description line */
#define ST_XYZ_SUPERCELL_BOXSIZE 2  /* PARCAS: boxsize on the description line */
#define ST_XYZ_SUPERCELL_HEADER 3   /* a "supercell" comment line and three vector lines */
#define ST_XYZ_SPECIES_MAX 1000     /* input0's limit on distinct species names */
#define ST_XYZ_NAME_LEN 6           /* XYZFILE_ATOMNAMELENGTH: names keep 6 characters */

typedef struct st_xyz_info {
  int64_t n_atoms;             /* the count line's first token (parseInt) */
  int64_t n_read;              /* the count line read list-directed (input0); -1 if it is not an integer */
  int32_t n_columns;           /* numbers after the species on the first atom line */
  int32_t n_header_lines;      /* comment lines (# % !) before the count line */
  int32_t lammps;              /* 1: the first line starts "LAMMPS" (read with st_lammps_header) */
  int32_t supercell_kind;      /* ST_XYZ_SUPERCELL_* */
  int32_t supercell_ok;        /* getSupercell's ok */
  int32_t repeats[3];          /* the cell repeats of the "supercell" header form (else 1) */
  double a_super[9];           /* the supercell, column-major (identity when not found) */
  int64_t data_offset;         /* byte offset of the first atom line */
  int64_t file_bytes;
  char column_description[257];  /* the line after the count line (256 characters kept) */
} st_xyz_info;

/* The header of an .xyz file as readHeader and getSupercell0 read it; the supercell numbers
 * through the reference's own ParseReal (NBAX_StringTokenizers.f90:303-420), not a correctly
 * rounded conversion, so that they carry the reference's bits.  Host only.  ST_ERR_ARG for a
 * missing file, no count line, or fewer than three numbers on the first atom line. */
int st_xyz_header(const char* path, st_xyz_info* info);

/* The atom lines of an .xyz file in device memory (d_text, n_bytes, from the first atom
 * line): line i is read list-directed as `species, x(1:n_columns)` (input0): the species
 * keeps its first 6 characters; the numbers are correctly rounded.  d_x[i ldx + c] for
 * c < min(ldx, n_columns) (other rows untouched); d_types[i] (may be null) = 1 + the
 * species' index in order of first appearance; species (may be null) receives the names
 * (6 characters each, blank padded) of the first species_cap of the *n_species species.
 * A line with a missing or malformed value returns ST_ERR_ARG with the first such line
 * (0-based) in *bad_line.  More than ST_XYZ_SPECIES_MAX species is an error, as in input0.
 * Waits for the parse to finish. */
int st_parse_xyz_device(st_ctx* ctx, const char* d_text, int64_t n_bytes, int64_t n_atoms, int32_t n_columns,
                        double* d_x, int64_t ldx, int32_t* d_types, int32_t* n_species, char* species,
                        int32_t species_cap, int64_t* bad_line, void* stream);

/* An .xyz file into host arrays: x(ldx, n) with n = info->n_read atoms (columns as for
 * st_parse_xyz_device), types and the species names as there.  info: st_xyz_header. */
int st_read_xyz(st_ctx* ctx, const char* path, const st_xyz_info* info, double* x, int64_t ldx, int32_t* types,
                int32_t* n_species, char* species, int32_t species_cap);

/* The reference's ParseReal on the host (the header-value parser of st_xyz_header): the
 * value of the first number-like run of text (len bytes) and whether one was found. */
int st_fortran_parse_real(const char* text, int64_t len, double* out, int32_t* ok);

#ifdef __cplusplus
}
#endif

#endif
