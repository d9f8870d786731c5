// Internal declarations shared by the libstem translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/stem.h"

namespace stem {

// Fixed-size kernel parameters of the link-cell binning (K1).
// One image (job) of a batch; the binning kernels read these from device memory.
struct BinParams {
  int64_t n_atoms;
  int64_t cap;  // capacity of the kept-atom arrays; more kept atoms set the overflow condition
  int64_t ldx;
  const double* x;    // positions (ldx, n_atoms) in device memory
  int64_t cand_base;  // first candidate of this job in the batch (candidates of job j: nuvw * n_atoms)
  int64_t cell_base;  // first link cell of this job in the batch's concatenated cell arrays
  int nuvw;
  int Ex, Ey, Ez;
  int64_t n_cells;
  double RU[9];
  double delta[3];
  double Ruvw[81];
  double lc_delta[3];
  double ia[9];  // inverse link-cell vectors
  double g[3];
  double a_col[3];  // diagonal of the link-cell vectors (cuboid cells)
  // FP32 copies for the FP64 path's reject prefilter
  float RUf[9];
  float Ruvwf[81];
  float shiftf[3];  // delta - lc_delta
  float iaf[3];     // diagonal of ia
  // FP32 imaging path (k_bin_atoms_fp32): link-cell coordinates c = A x + B(nn) and g.y in
  // cycles = gA x + gB(nn), the x part per atom in FP64, the replica part B(nn) per job, both
  // summed in 64-bit fixed point of 2^-36 (cells or cycles)
  int64_t atom_base;  // first atom of this job in the batch
  double Afx[9];      // (ia RU)(a, k) * 2^36, row-major
  double gAfx[3];     // (g^T RU)(k) / (2 pi) * 2^36
  long long Bfx[81];  // round(2^36 * ia (RU Ruvw(nn) + delta - lc_delta)), 3 per replica
  long long gBfx[27]; // round(2^36 * frac(g . (RU Ruvw(nn) + delta) / (2 pi)))
  float Bf[81];       // B(nn) in cells, for the FP32 reject prefilter
  float a_colf[3];
  int fix_ok;         // 0: |B| too large for the fixed point; every candidate takes the exact arithmetic
};

// Output of the binning: atoms sorted by link cell, each cell in the
// reference's insertion order (replica-major, then atom order).
struct BinnedAtoms {
  int* cell_start;     // n_cells + 1
  int* cell_count;     // n_cells
  // FP64 records
  double4_32a* f64;        // fx, fy, fz (fractional offset in the cell), unused
  double2* cs64;       // cos(g.y), sin(g.y)
  // FP32 records
  float4* p32;         // a_col11*fx, a_col22*fy, a_col33*fz, bits(packed cell)
  float2* cs32;        // cos, sin of the FP64-reduced phase
  uint4* fr32;         // 2^-32 units of the cell fractions (x, y, z, -): the cutoff's exact recheck
  float* ph32;         // the FP64-reduced phase in cycles, [-1/2, 1/2)
};

// A kept atom's record of the FP32 path as the binning makes it (same size as double4_32a).
struct alignas(16) Rec32 {
  float4 p;          // a_col11*fx, a_col22*fy, a_col33*fz, bits(packed cell)
  float tc;          // phase g.y / 2 pi, reduced to [-1/2, 1/2) cycles
  unsigned frac[3];  // 2^-32 units of the cell fractions fx, fy, fz (the fixed point's top 32 bits)
};

struct Scratch {
  // binning temporaries, sized for nuvw * n_atoms candidates
  int* tmp_key = nullptr;   // candidate index nn * N + jj
  int* tmp_cell = nullptr;  // linear cell index
  int* tmp_slot = nullptr;  // arrival slot within the cell (atomic order)
  double4_32a* tmp_f = nullptr; // fx, fy, fz, g.y (FP64 path); Rec32 (FP32 path)
  int* perm = nullptr;      // position-in-cell -> tmp index
  int* block_sums = nullptr;
  unsigned long long* counters = nullptr;  // [0] kept, [1] max cell count, [2] tests, [3] accepted, [4] slab overflow
  size_t cap_candidates = 0;
  size_t cap_cells = 0;
  size_t cap_blocks = 0;
  // per-image tables of the voxel columns
  int2* xtab = nullptr;  // (home cell, unused) per ix
  double* xfv = nullptr; // fractional voxel offset per ix
  int2* ytab = nullptr;
  double* yfv = nullptr;
  int2* ztab = nullptr;  // (home cell, FP32 bits of the slab-ring kernel's scaled slice depth) per iz
  double* zfv = nullptr;
  size_t cap_x = 0, cap_y = 0, cap_z = 0;
  double* aa = nullptr;
  float* aaf = nullptr;
  size_t cap_prec = 0;
};

struct ColumnParams {
  int Mx, My, Mz;
  int ix0, ix1, iy0, iy1;
  int Ex, Ey, Ez;
  int n_prec;
  int prec_offset;  // first precession angle of this pass
  int accumulate;   // add into img instead of overwriting
  int use_density;
  int check_cells;  // restrict to the 27 cells around the home cell (needed when a cell is < 3 sigma)
  int trunc_z;      // the z cells are shorter than 3 sigma (the slab ring applies the 27-cell rule in z)
  int want_stats;
  int finalize;          // the slab ring's last pass: write (sum) / fin_scale, or 1 - that when fin_bright
  int fin_bright;
  double fin_scale;
  double a11, a22, a33;  // link-cell sides (cuboid)
  double cut2;           // (3 sigma)^2
  double i2s2;           // 1 / (2 sigma^2)
  double sigma;
  double b0, bg, dz;
  const int* cell_start;
  const double4_32a* f64;
  const double2* cs64;
  const float4* p32;
  const float2* cs32;
  const uint4* fr32;
  const float* ph32;
  const int2* xtab;
  const double* xfv;
  const int2* ytab;
  const double* yfv;
  const int2* ztab;
  const double* zfv;
  const double* aa;
  const float* aaf;
  double* img;
  unsigned long long* counters;  // [0] kept atoms: above `cap` the binning overflowed and the kernel exits
  int64_t cap;
  // null, or one byte per mask_T x mask_T pixel tile (mask_ntx tiles per row): the columns of
  // tiles whose byte is 0 are not computed (mask_T a multiple of 8, window origin aligned)
  const unsigned char* tile_mask;
  int mask_T, mask_ntx;
};

// Whether warp tile (tx, ty) of a column launch is to be computed.
__device__ __forceinline__ bool tile_wanted(const ColumnParams& p, int tx, int ty, int tile_x, int tile_y) {
  if (!p.tile_mask) return true;
  return p.tile_mask[((p.iy0 + ty * tile_y) / p.mask_T) * p.mask_ntx + (p.ix0 + tx * tile_x) / p.mask_T] != 0;
}

// launchers (return cudaError_t of the launches)
// Binning of a batch: jobs (device memory, n_jobs entries) with atoms [0, total_atoms),
// candidates [0, total_cand) and cells [0, total_cells) concatenated in job order.
// fp32: the FP32 path's records (Rec32); else the FP64 path's, in the reference's rounded
// arithmetic.
// Kernels the imaging path has launched on this host thread; run_images resets it per
// call and reports the count in st_stats.n_launches.
inline int& launch_count() {
  static thread_local int n = 0;
  return n;
}

cudaError_t launch_bin(const BinParams* d_jobs, int n_jobs, int64_t total_atoms, int64_t total_cand,
                       int64_t total_cells, int64_t cap, Scratch& s, BinnedAtoms& b, bool fp32, cudaStream_t st);
cudaError_t launch_bin_finalize(const BinParams* d_jobs, int n_jobs, int64_t total_cells, int64_t cap, Scratch& s,
                                BinnedAtoms& b, bool fp32, cudaStream_t st);
cudaError_t launch_column_fp32(const ColumnParams& p, cudaStream_t st);

// A job of the persistent slab-ring FP32 column kernels: an image and the first warp
// tile it owns in the batch's tile sequence, for each tile shape (8 x 4, 4 x 8, 16 x 2).
constexpr int kRingShapes = 3;
struct ColumnJob {
  ColumnParams p;
  int tile_base[kRingShapes];
  int pad;
};
int column_tiles(const ColumnParams& p, int shape = 0);  // warp tiles of one image in `shape`
// The slab-ring launch.  `tiles`: the pass's warp tiles in each shape (host array).
// `variant` 0 .. ring_variant_count() - 1 selects the kernel, its tile shape, slab
// capacity and CTAs per SM (ring_variant_name); the images of different variants agree to
// FP32 rounding, those of one variant to the last bit.  `slab_tier` 1, 2: 192, 256 atoms
// per slab (dense footprints), with variant 0's 8 x 4 tiles, so at those tiers every
// variant gives variant 0's bits.  `masked`: some jobs carry a tile mask (then max_np must
// be 1 and stats false).
cudaError_t launch_column_fp32_ring(const ColumnJob* d_jobs, int n_jobs, const int* tiles, int max_np, bool density,
                                    bool stats, int variant, int slab_tier, bool masked, unsigned* work,
                                    const unsigned long long* counters, int64_t cap, cudaStream_t st);
int ring_variant_count();
const char* ring_variant_name(int variant);
int ring_variant_slab(int variant);  // atoms per slab of the variant's first tier
int ring_np_bucket(int max_np);  // the kernel template (angles per pass) serving max_np angles
namespace ring3 {
// third generation (k_column_v3.cuh), one instance set per angle bucket NP
struct Ring3Args {
  const ColumnJob* jobs;
  int n_jobs;
  const int* tiles;  // per shape
  bool density, stats, masked;
  int variant, tier;
  unsigned* work;
  const unsigned long long* counters;
  int64_t cap;
  cudaStream_t st;
};
template <int NP>
cudaError_t ring3_launch_np(const Ring3Args& a);
extern template cudaError_t ring3_launch_np<1>(const Ring3Args&);
extern template cudaError_t ring3_launch_np<2>(const Ring3Args&);
extern template cudaError_t ring3_launch_np<4>(const Ring3Args&);
extern template cudaError_t ring3_launch_np<8>(const Ring3Args&);
extern template cudaError_t ring3_launch_np<16>(const Ring3Args&);
}  // namespace ring3
cudaError_t launch_column_fp64(const ColumnParams& p, cudaStream_t st);
// The FP64 slab-ring launch (k_column_f64ring.cu) over the jobs of one pass of at most 4
// precession angles; slab tiers 0, 1, 2 stage 128, 192, 256 atoms; `four`: every job's
// steps of four slices fit the ring (four_slices_fit).
cudaError_t launch_column_fp64_ring(const ColumnJob* d_jobs, int n_jobs, int tiles, int max_np, int slab_tier,
                                    bool masked, bool four, unsigned* work, const unsigned long long* counters,
                                    int64_t cap, cudaStream_t st);
// Whether every step of four slices (z = 0, 4, 8 ...) of an image has home z cells that
// rise by at most one cell without wrapping, so that the cells the step needs (one more on
// either side) fit the slab ring's four slots.
bool four_slices_fit(const st_geom* g);
cudaError_t launch_epilogue(double* img, int Mx, int My, int ix0, int ix1, int iy0, int iy1, double scale,
                            int bright, cudaStream_t st);
cudaError_t launch_blur(const double* d_in, double* d_tmp, double* d_out, int nx, int ny, const double* d_kernel,
                        int nk, cudaStream_t st);

__host__ __device__ inline int pack_cell(int cx, int cy, int cz) { return cx | (cy << 10) | (cz << 20); }

// Output files (k_output.cu).  PNG levels: d_part holds 2 kLevelParts doubles (partial
// minima and maxima), d_ab 2 (the level map); d_levels nx * ny values.
constexpr int kLevelParts = 256;
cudaError_t launch_png_levels(const double* d_img, int nx, int ny, double iso_min, double iso_max, double* d_part,
                              double* d_ab, uint16_t* d_levels, cudaStream_t st);
// '(1000f12.7)' records of n values (st_dat_text_bytes(n) bytes)
cudaError_t launch_format_dat(const double* d_v, int64_t n, char* d_text, cudaStream_t st);
// Geometry over the atoms (k_geom.cu)
struct GeomWrap {
  double a[9], ia[9];  // voxel supercell and its inverse, column-major
  int N[3];
};
constexpr int kMaxRot = 32;       // conditions per extents pass
constexpr int kExtentBlocks = 1024;
struct GeomRot {
  double U[9 * kMaxRot];  // rotations to the standard frame, column-major
  int n;
};
cudaError_t launch_wrap_pbc(const GeomWrap& w, double* d_x, int64_t ldx, int64_t n, cudaStream_t st);
// The -ng tilt search (k_tilt.cu).  TiltScores: the constants of the reference's
// score arithmetic, computed on the host; the launch writes scores[nk] from khat(3, nk),
// ghkl(3, nn) and bg[nn] = PI / xi_g.
struct TiltScores {
  double cst;        // 2 ME v / HBAR
  double hbar2on2m;  // HBAR^2 / (2 ME)
  double den;        // 2 PI HBAR v
  double twopi;      // 2 PI
  double b0;         // PI / xi_g(1)
  double foil;       // foil thickness L
  int nk, nn;
};
constexpr int kTiltSlice = 128;  // reflections per task of the score launch
int tilt_slices(int nn);         // slices per incident vector: the partial sums per score
// d_part: nk * tilt_slices(nn) partial sums, vector-major
cudaError_t launch_tilt_scores(const TiltScores& p, const double* d_khat, const double* d_ghkl, const double* d_bg,
                               double* d_part, cudaStream_t st);
// the FP32 screen on FP32 copies of the inputs: d_part2 holds nk * tilt_slices(nn) pairs
// (partial score, bound on its error)
cudaError_t launch_tilt_screen(const TiltScores& p, const float* d_khat, const float* d_ghkl, const float* d_bg,
                               float* d_part2, cudaStream_t st);
// findFoilThickness's column grid: the atoms' highest and lowest z per column over the
// replicas, as order keys (order_key_value turns one back into its double).
struct FoilGrid {
  double RU[9];      // column-major
  double delta[3];
  double Ruvw[81];   // replica offsets
  double ddx, ddy;   // Nx / d1, Ny / d2
  double id3;        // 1 / d3
  int Nx, Ny, nuvw;
};
constexpr size_t kFoilSmemMax = 96 * 1024;  // grids up to 6,144 columns merge in shared memory
cudaError_t launch_foil_thickness(const FoilGrid& f, const double* d_x, int64_t ldx, int64_t n,
                                  unsigned long long* d_top, unsigned long long* d_thick, double top0, double thick0,
                                  cudaStream_t st);
double order_key_value(unsigned long long k);
// context accessors for the host translation units (stem_ctx.cu)
cudaStream_t ctx_stream(st_ctx* c, void* stream);  // stream, or the context's when null; makes its device current
int ctx_fail(st_ctx* c, int code, const char* msg);
int ctx_cuda_fail(st_ctx* c, cudaError_t e, const char* where);
// scratch of the extents pass: *part (kExtentBlocks * kMaxRot * 6 doubles), *out (6 * kMaxRot)
cudaError_t ctx_geom_scratch(st_ctx* c, double** part, double** out);
cudaError_t ctx_tilt_scratch(st_ctx* c, size_t n_doubles, double** p);  // device doubles, grown on demand
// d_part: kExtentBlocks * kMaxRot * 6 doubles; d_out: 6 per rotation (min x, y, z, max x, y, z)
cudaError_t launch_extents(const GeomRot& rot, const double* d_x, int64_t ldx, int64_t n, double* d_part,
                           double* d_out, cudaStream_t st);
// LAMMPS Atoms block (k_parse.cu): d_seg holds parse_segments(n_bytes) values, d_starts
// n_atoms; *d_bad = the first malformed atom line, or all ones
int64_t parse_segments(int64_t n_bytes);
cudaError_t launch_parse_atoms(const char* d_text, int64_t n_bytes, int64_t n_atoms, long long* d_seg,
                               long long* d_starts, double* d_x, int64_t ldx, int* d_types,
                               unsigned long long* d_bad, cudaStream_t st);
// .xyz atom lines (k_parse.cu): species keys (6 bytes) and ncols numbers per line, the first
// min(ldx, ncols) into d_x; then species numbers in order of first appearance.
// d_scratch: species_scratch(n) values; the table of first appearances sits at
// species_table_offset() (1000 keys, then the count; a count of 1001 means too many).
cudaError_t launch_parse_xyz(const char* d_text, int64_t n_bytes, int64_t n_atoms, int ncols, long long* d_seg,
                             long long* d_starts, double* d_x, int64_t ldx, unsigned long long* d_keys,
                             unsigned long long* d_bad, cudaStream_t st);
int64_t species_scratch(int64_t n_atoms);
int species_table_offset();
cudaError_t launch_species(const unsigned long long* d_keys, int64_t n, unsigned long long* d_scratch,
                           int32_t* d_types, cudaStream_t st);

}  // namespace stem
