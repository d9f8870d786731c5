// libstem C ABI: context, device memory and the image / batch / blur entry points.
//
// An image replaces the patch loop of computeD2BI_img
// (src/Lib_DynamicalTwoBeamImaging.f90:1842-1946): K1 bins the atoms
// (findGdotR), K2+K3 compute the voxel field and integrate every column, and
// an epilogue applies the optional average over precession angles and the
// bright-field flip.  A batch runs K1 once over the candidates of all its
// images and K2+K3 as one persistent launch over all their warp tiles.
// st_blur is gaussianBlurImage (src/d2bi.f90:1543-1624).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "internal.h"

using namespace stem;

struct st_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  Scratch s;
  BinnedAtoms b{};
  size_t cap_kept = 0;
  size_t cap_cells = 0;
  double* d_x = nullptr;
  size_t cap_x = 0;
  double* d_img = nullptr;
  size_t cap_img = 0;
  double* d_blur = nullptr;  // in, tmp (+w_stripe), out
  size_t cap_blur = 0;
  double* d_kern = nullptr;
  size_t cap_kern = 0;
  BinParams* d_binjobs = nullptr;
  size_t cap_binjobs = 0;
  ColumnJob* d_coljobs = nullptr;
  size_t cap_coljobs = 0;
  unsigned* d_work = nullptr;
  double* d_bx = nullptr;  // st_batch: packed atoms of the distinct atom arrays
  size_t cap_bx = 0;
  double* d_bimg = nullptr;  // st_batch: images
  size_t cap_bimg = 0;
  unsigned long long* h_counters = nullptr;  // pinned
  void* h_stage = nullptr;                   // pinned staging for tables and job descriptors
  cudaEvent_t ev_stage = nullptr;            // recorded after the last copy out of h_stage
  size_t cap_stage = 0;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  st_stats stats{};
  int64_t last_kept = 0;       // kept atoms of the previous call: sizes the next one
  bool fp32_general = false;   // STEM_FP32_KERNEL=general: always use k_column_fp32
  bool fp64_general = false;   // STEM_FP64_KERNEL=general: always use k_column_fp64
  int min_slab_tier = 0;       // STEM_RING_SLABS=192 or 256: start the slab ring at that capacity
  int last_column_kernel = 0;  // 1 general FP32, 2 slab-ring FP32, 3 general FP64, 4 slab-ring FP64
  int tune_mode = ST_TUNE_AUTO;
  std::map<uint64_t, int> ring_tuned;  // (pass kind, image and link-cell shape) -> fastest slab-ring variant
  std::map<uint64_t, int> ring_big;  // (pass kind, image and link-cell shape) -> slab tier it needs (1, 2)
  cudaEvent_t tev[3] = {nullptr, nullptr, nullptr};
  int last_ring_variant = -1;
  double* d_lvaux = nullptr;  // PNG levels: partial minima/maxima and the level map
  size_t cap_lvaux = 0;
  uint16_t* d_levels = nullptr;
  size_t cap_levels = 0;
  char* d_text = nullptr;  // .dat records; LAMMPS text
  size_t cap_text = 0;
  long long* d_pseg = nullptr;  // LAMMPS parse: segment counts, line starts
  size_t cap_pseg = 0;
  long long* d_pstart = nullptr;
  size_t cap_pstart = 0;
  unsigned long long* d_pbad = nullptr;
  size_t cap_pbad = 0;
  void* h_text = nullptr;  // pinned staging of a data file
  size_t cap_htext = 0;
  double* d_geom = nullptr;  // extents pass: partial and final minima / maxima
  size_t cap_geom = 0;
  double* d_tilt = nullptr;  // tilt search: incident vectors, reflections, scores; foil-thickness grid
  size_t cap_tilt = 0;
  unsigned long long* d_keys = nullptr;  // .xyz reader: species key per atom line
  size_t cap_keys = 0;
  unsigned long long* d_species = nullptr;  // .xyz reader: species tables
  size_t cap_species = 0;
};

namespace {

int fail(st_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(st_ctx* c, cudaError_t e, const char* where) {
  return fail(c, ST_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
cudaError_t ensure(T*& p, size_t& cap, size_t need) {
  if (need <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  size_t n = need + need / 4 + 64;
  cudaError_t e = cudaMalloc((void**)&p, n * sizeof(T));
  if (e == cudaSuccess) cap = n;
  return e;
}

cudaError_t ensure_host(void*& p, size_t& cap, size_t bytes) {
  if (bytes <= cap && p) return cudaSuccess;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  size_t n = bytes + bytes / 4 + 256;
  cudaError_t e = cudaMallocHost(&p, n);
  if (e == cudaSuccess) cap = n;
  return e;
}

// Arrays indexed by kept atom (binning temporaries and records).
bool alloc_kept(st_ctx* c, size_t need) {
  if (need <= c->cap_kept && c->b.p32) return true;
  size_t k = 0;
  cudaError_t e = cudaSuccess;
  auto grow = [&](auto*& p) {
    size_t cap = c->cap_kept;
    if (e == cudaSuccess) e = ensure(p, cap, need);
    k = cap;
  };
  grow(c->s.tmp_key);
  grow(c->s.tmp_cell);
  grow(c->s.tmp_slot);
  grow(c->s.tmp_f);
  grow(c->s.perm);
  grow(c->b.f64);
  grow(c->b.cs64);
  grow(c->b.p32);
  grow(c->b.cs32);
  grow(c->b.fr32);
  grow(c->b.ph32);
  if (e != cudaSuccess) return false;
  c->cap_kept = k;
  c->s.cap_candidates = k;
  return true;
}

int __float_as_int_host(float v) {
  int b;
  std::memcpy(&b, &v, sizeof b);
  return b;
}

bool is_cuboid(const double* m) {
  return m[1] == 0.0 && m[2] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[6] == 0.0 && m[7] == 0.0;
}

// Home link cell and fractional offset of voxel index i along one axis:
// zi = ia * (a_vox * i - lc_delta); h = mod(floor(zi) + 16 N, N); fv = zi - h
// (Lib_DynamicalTwoBeamImaging.f90:1878-1879, Lib_LinkCell3D.f90:1547-1560).
void axis_table(int n, double a_vox, double lcd, double ia, int N, int2* tab, double* fv) {
  for (int i = 0; i < n; ++i) {
    const double xx = a_vox * (double)i - lcd;
    const double zi = ia * xx;
    int h = (int)std::floor(zi) + 16 * N;
    h = h % N;
    if (h < 0) h += N;  // the reference's mod of a non-negative value
    tab[i] = make_int2(h, 0);
    fv[i] = zi - (double)h;
  }
}

// Slice depths for the slab-ring kernel, in the .y half of the z table: the depth of
// slice z (FP32 bits) in units scaled by s = sqrt(log2 e / (2 sigma^2)), measured from the
// origin of the home cell of the even slice of its pair (z & ~1), which is the frame the
// kernel marches in.  Computed in FP64 exactly as a33 (fv + dh) s, rounded once to FP32.
void depth_table(const st_geom* g, int2* tab, const double* fv) {
  const double i2s2 = 1 / (2 * g->sigma * g->sigma);
  const double sd = std::sqrt(i2s2 * 1.4426950408889634);
  const double a33 = g->a_col[8];
  for (int z = 0; z < g->Mz; ++z) {
    const int h_even = tab[z & ~1].x;
    const float v = (z & 1) ? (float)(a33 * (fv[z] + (double)(tab[z].x - h_even)) * sd) : (float)(a33 * fv[z] * sd);
    tab[z].y = __float_as_int_host(v);
  }
}

bool four_slices_fit(const st_geom* g) {
  std::vector<int2> tab((size_t)g->Mz);
  std::vector<double> fv((size_t)g->Mz);
  axis_table(g->Mz, g->a_vox[8], g->lc_delta[2], g->ia_col[8], g->Ez, tab.data(), fv.data());
  for (int z0 = 0; z0 < g->Mz; z0 += 4) {
    const int last = std::min(z0 + 3, g->Mz - 1);
    for (int z = z0 + 1; z <= last; ++z)
      if (tab[z].x < tab[z - 1].x) return false;  // wrapped
    if (tab[last].x - tab[z0].x > 1) return false;
  }
  return true;
}

int validate(st_ctx* c, const st_geom* g, int64_t ldx, int64_t nAtoms, int32_t nPrec) {
  if (!g) return fail(c, ST_ERR_ARG, "geometry is null");
  if (ldx < 3) return fail(c, ST_ERR_ARG, "ldx must be >= 3");
  if (nAtoms < 0) return fail(c, ST_ERR_ARG, "nAtoms must be >= 0");
  if (nPrec < 1) return fail(c, ST_ERR_ARG, "nPrec must be >= 1");
  if (g->Mx < 1 || g->My < 1 || g->Mz < 1) return fail(c, ST_ERR_ARG, "Mx, My, Mz must be >= 1");
  if (g->ix0 < 0 || g->ix1 > g->Mx || g->ix0 > g->ix1 || g->iy0 < 0 || g->iy1 > g->My || g->iy0 > g->iy1)
    return fail(c, ST_ERR_ARG, "patch window outside the image");
  if (g->Ex < 1 || g->Ey < 1 || g->Ez < 1 || g->Ex > 1023 || g->Ey > 1023 || g->Ez > 1023)
    return fail(c, ST_ERR_ARG, "link-cell counts must be in 1..1023 per axis");
  if (g->nuvw < 1 || g->nuvw > 27) return fail(c, ST_ERR_ARG, "nuvw must be in 1..27");
  if ((double)g->nuvw * (double)nAtoms >= 2147483647.0)
    return fail(c, ST_ERR_ARG, "nuvw * nAtoms exceeds 2^31 - 1 candidates");
  if (!is_cuboid(g->a_vox) || !is_cuboid(g->a_col) || !is_cuboid(g->ia_col))
    return fail(c, ST_ERR_ARG, "voxel and link cells must be cuboids (diagonal a_vox, a_col, ia_col)");
  if (!(g->sigma > 0.0) || !(g->deltaz > 0.0)) return fail(c, ST_ERR_ARG, "sigma and deltaz must be > 0");
  return ST_OK;
}

// One image of a call, as the host sees it.
struct Job {
  const st_geom* g;
  const double* d_x;
  int64_t ldx, n_atoms;
  const double* aa;  // host
  int n_prec;
  double* d_img;
  const unsigned char* tile_mask = nullptr;  // device; see ColumnParams
  int mask_T = 0;
};

BinParams bin_params(const Job& j, int64_t cand_base, int64_t cell_base, int64_t atom_base) {
  const st_geom* g = j.g;
  BinParams bp;
  memset(&bp, 0, sizeof bp);
  bp.n_atoms = j.n_atoms;
  bp.ldx = j.ldx;
  bp.x = j.d_x;
  bp.cand_base = cand_base;
  bp.cell_base = cell_base;
  bp.nuvw = g->nuvw;
  bp.Ex = g->Ex;
  bp.Ey = g->Ey;
  bp.Ez = g->Ez;
  bp.n_cells = (int64_t)g->Ex * g->Ey * g->Ez;
  memcpy(bp.RU, g->RU, sizeof bp.RU);
  memcpy(bp.delta, g->delta, sizeof bp.delta);
  memcpy(bp.Ruvw, g->Ruvw, sizeof bp.Ruvw);
  memcpy(bp.lc_delta, g->lc_delta, sizeof bp.lc_delta);
  memcpy(bp.ia, g->ia_col, sizeof bp.ia);
  memcpy(bp.g, g->g, sizeof bp.g);
  bp.a_col[0] = g->a_col[0];
  bp.a_col[1] = g->a_col[4];
  bp.a_col[2] = g->a_col[8];
  for (int i = 0; i < 9; ++i) bp.RUf[i] = (float)g->RU[i];
  for (int i = 0; i < 81; ++i) bp.Ruvwf[i] = (float)g->Ruvw[i];
  for (int i = 0; i < 3; ++i) bp.shiftf[i] = (float)(g->delta[i] - g->lc_delta[i]);
  bp.iaf[0] = (float)g->ia_col[0];
  bp.iaf[1] = (float)g->ia_col[4];
  bp.iaf[2] = (float)g->ia_col[8];
  // the FP32 path's fixed-point form (2^-36): c = A x + B(nn), g.y / 2 pi = gA x + gB(nn),
  // matrices column-major as in st_geom (M(a, b) = M[a + 3 b])
  const double S = 68719476736.0, inv2pi = 0.15915494309189533577;
  bp.atom_base = atom_base;
  bp.fix_ok = 1;
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k) {
      double s_ak = 0.0;
      for (int b = 0; b < 3; ++b) s_ak += g->ia_col[a + 3 * b] * g->RU[b + 3 * k];
      bp.Afx[3 * a + k] = s_ak * S;
    }
  for (int k = 0; k < 3; ++k) {
    double s_k = 0.0;
    for (int a = 0; a < 3; ++a) s_k += g->g[a] * g->RU[a + 3 * k];
    bp.gAfx[k] = s_k * inv2pi * S;
  }
  for (int nn = 0; nn < g->nuvw; ++nn) {
    double w[3];  // RU Ruvw(nn) + delta
    for (int b = 0; b < 3; ++b) {
      w[b] = g->delta[b];
      for (int k = 0; k < 3; ++k) w[b] += g->RU[b + 3 * k] * g->Ruvw[3 * nn + k];
    }
    double gw = 0.0;
    for (int a = 0; a < 3; ++a) {
      double ba = 0.0;
      for (int b = 0; b < 3; ++b) ba += g->ia_col[a + 3 * b] * (w[b] - g->lc_delta[b]);
      if (!(std::fabs(ba) < 16384.0)) bp.fix_ok = 0;  // beyond 2^14 cells: the exact arithmetic throughout
      bp.Bfx[3 * nn + a] = bp.fix_ok ? std::llrint(ba * S) : 0;
      bp.Bf[3 * nn + a] = (float)ba;
      gw += g->g[a] * w[a];
    }
    const double cyc = gw * inv2pi;
    bp.gBfx[nn] = std::isfinite(cyc) ? std::llrint((cyc - std::rint(cyc)) * S) : 0;
    if (!std::isfinite(cyc)) bp.fix_ok = 0;
  }
  for (int a = 0; a < 3; ++a) bp.a_colf[a] = (float)bp.a_col[a];
  for (int i = 0; i < 9; ++i)
    if (!std::isfinite(bp.Afx[i])) bp.fix_ok = 0;
  return bp;
}

// The records of the kept atoms (reallocated when a call keeps more atoms than they hold).
void point_at_kept(const st_ctx* c, ColumnParams& cp) {
  cp.f64 = c->b.f64;
  cp.cs64 = c->b.cs64;
  cp.p32 = c->b.p32;
  cp.cs32 = c->b.cs32;
  cp.fr32 = c->b.fr32;
  cp.ph32 = c->b.ph32;
}

ColumnParams column_params(st_ctx* c, const Job& j, int64_t cell_base, size_t xoff, size_t yoff, size_t zoff,
                           size_t aoff, int flags) {
  const st_geom* g = j.g;
  ColumnParams cp;
  memset(&cp, 0, sizeof cp);
  cp.Mx = g->Mx;
  cp.My = g->My;
  cp.Mz = g->Mz;
  cp.ix0 = g->ix0;
  cp.ix1 = g->ix1;
  cp.iy0 = g->iy0;
  cp.iy1 = g->iy1;
  cp.Ex = g->Ex;
  cp.Ey = g->Ey;
  cp.Ez = g->Ez;
  cp.n_prec = j.n_prec;
  cp.use_density = g->useDensity;
  cp.want_stats = (flags & ST_FLAG_STATS) ? 1 : 0;
  cp.a11 = g->a_col[0];
  cp.a22 = g->a_col[4];
  cp.a33 = g->a_col[8];
  cp.cut2 = (3 * g->sigma) * (3 * g->sigma);
  cp.i2s2 = 1 / (2 * g->sigma * g->sigma);
  cp.sigma = g->sigma;
  cp.b0 = g->b0;
  cp.bg = g->bg;
  cp.dz = g->deltaz;
  // link cells narrower than 3 sigma truncate the search to 27 cells: test the cell offsets too
  const double r3 = 3 * g->sigma * (1.0 + 1e-6) + 1e-6;
  cp.check_cells = (cp.a11 < r3 || cp.a22 < r3 || cp.a33 < r3) ? 1 : 0;
  cp.trunc_z = cp.a33 < r3 ? 1 : 0;
  cp.cell_start = c->b.cell_start + cell_base;
  point_at_kept(c, cp);
  cp.xtab = c->s.xtab + xoff;
  cp.xfv = c->s.xfv + xoff;
  cp.ytab = c->s.ytab + yoff;
  cp.yfv = c->s.yfv + yoff;
  cp.ztab = c->s.ztab + zoff;
  cp.zfv = c->s.zfv + zoff;
  cp.aa = c->s.aa + aoff;
  cp.aaf = c->s.aaf + aoff;
  cp.img = j.d_img;
  cp.counters = c->s.counters;
  cp.tile_mask = j.tile_mask;
  cp.mask_T = j.mask_T;
  cp.mask_ntx = j.mask_T > 0 ? (g->Mx + j.mask_T - 1) / j.mask_T : 0;
  return cp;
}

// Times every slab-ring variant once on the same pass (each overwrites the pass's
// images) and returns the fastest in `best`, or -1 when the binning overflowed (the
// timings mean nothing then).  A variant whose slabs overflowed its staging is left out
// (its counter is cleared for the next trial).  The variants' images agree to FP32
// rounding, not to the bit, so the pass ends with the chosen variant's own output.
template <typename F>
cudaError_t tune_ring(st_ctx* c, F&& launch_variant, int64_t cap, cudaStream_t st, int& best) {
  best = -1;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; ++i)
    if (!c->tev[i]) e = cudaEventCreate(&c->tev[i]);
  const int nv = ring_variant_count();
  std::vector<float> ms(nv, 0.f);
  std::vector<char> valid(nv, 0);
  unsigned long long h[5];
  int last = -1;  // the last trial that ran (its output, whole or partial, is in the images)
  for (int v = 0; v < nv && e == cudaSuccess; ++v) {
    cudaEventRecord(c->tev[0], st);
    e = launch_variant(v);
    last = v;
    cudaEventRecord(c->tev[1], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(c->tev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[v], c->tev[0], c->tev[1]);
    if (e == cudaSuccess) e = cudaMemcpy(h, c->s.counters, sizeof h, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) break;
    if ((int64_t)h[0] > cap) return cudaSuccess;
    if (h[4] != 0) {
      e = cudaMemsetAsync(c->s.counters + 4, 0, sizeof(unsigned long long), st);
      continue;
    }
    valid[v] = 1;
  }
  if (e != cudaSuccess) return e;
  for (int v = 0; v < nv; ++v)
    if (valid[v] && (best < 0 || ms[v] < ms[best])) best = v;
  if (best >= 0 && best != last) e = launch_variant(best);  // the pass's images from the chosen variant
  if (best >= 0) c->last_ring_variant = best;
  return e;
}

// The slab-ring FP32 kernel needs cells of at least 3 sigma (no truncated
// search) and at least one voxel thick in z.
// The slab ring needs link cells of at least 3 sigma in x and y: then every atom within
// 3 sigma of a column lies in its 9 cells around it in x-y.  The reference's grid makes them
// so (Dx + 2 deltaM voxels over floor(Dx / deltaM + 2) cells, deltaM = ceil(3 sigma / the
// smaller in-plane voxel side)); the margin allows rounding only.  In z the kernel applies
// the 27-cell rule itself, so cells shorter than 3 sigma qualify.
bool ring_eligible(const ColumnParams& cp, bool stats) {
  if (cp.tile_mask && (cp.n_prec != 1 || stats)) return false;  // masked ring: one angle, no statistics
  const double r3 = 3 * cp.sigma * (1.0 - 1e-9);
  return cp.a11 >= r3 && cp.a22 >= r3 && cp.Ez <= cp.Mz;
}

// A recorded call (st_plan): the instantiated graph and what its kernels were recorded with.
struct GraphOut {
  cudaGraphExec_t exec = nullptr;
  int64_t cap = 0;    // kept-atom capacity the binning was recorded with
  bool ring = false;  // the slab-ring kernel ran (its slab overflow needs the eager path)
};

// Image the jobs: binning of all, then the column kernels, then the epilogues.
int run_images(st_ctx* c, const std::vector<Job>& jobs, int32_t flags, cudaStream_t st, GraphOut* gout = nullptr) {
  const int n = (int)jobs.size();
  const bool fp32 = (flags & ST_FLAG_FP32) != 0;
  launch_count() = 0;
  // concatenation offsets
  std::vector<int64_t> cand_base(n + 1, 0), cell_base(n + 1, 0), atom_base(n + 1, 0);
  std::vector<size_t> xoff(n + 1, 0), yoff(n + 1, 0), zoff(n + 1, 0), aoff(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    const st_geom* g = jobs[i].g;
    cand_base[i + 1] = cand_base[i] + (int64_t)g->nuvw * jobs[i].n_atoms;
    atom_base[i + 1] = atom_base[i] + jobs[i].n_atoms;
    cell_base[i + 1] = cell_base[i] + (int64_t)g->Ex * g->Ey * g->Ez;
    xoff[i + 1] = xoff[i] + g->Mx;
    yoff[i + 1] = yoff[i] + g->My;
    zoff[i + 1] = zoff[i] + g->Mz;
    aoff[i + 1] = aoff[i] + ((jobs[i].n_prec + 1) & ~1);  // even: the FP32 ring reads angle pairs
  }
  const int64_t total_cand = cand_base[n], total_cells = cell_base[n];
  // kept atoms are indexed by int (cell starts, permutation): at most total_cand of them
  if (total_cand >= 2147483647LL) return fail(c, ST_ERR_ARG, "a binning pass holds more than 2^31 - 1 candidates");
  if (total_cells >= 2147483647LL) return fail(c, ST_ERR_ARG, "a call holds more than 2^31 - 1 link cells");

  // ---- device buffers that do not depend on the kept-atom count
  cudaError_t e = cudaSuccess;
  {
    size_t cc = c->cap_cells;
    e = ensure(c->b.cell_start, cc, (size_t)total_cells + 1);
    cc = c->cap_cells;
    if (e == cudaSuccess) e = ensure(c->b.cell_count, cc, (size_t)total_cells + 1);
    size_t nb = c->s.cap_blocks;
    if (e == cudaSuccess) e = ensure(c->s.block_sums, nb, (size_t)(total_cells / 1024 + 2));
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating cell buffers");
    c->cap_cells = cc;
    c->s.cap_blocks = nb;
    if (!c->s.counters) {
      e = cudaMalloc((void**)&c->s.counters, 8 * sizeof(unsigned long long));
      if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_work, sizeof(unsigned));
      if (e != cudaSuccess) return cuda_fail(c, e, "allocating counters");
    }
    size_t cx = c->s.cap_x;
    e = ensure(c->s.xtab, cx, xoff[n]);
    cx = c->s.cap_x;
    if (e == cudaSuccess) e = ensure(c->s.xfv, cx, xoff[n]);
    size_t cy = c->s.cap_y;
    if (e == cudaSuccess) e = ensure(c->s.ytab, cy, yoff[n]);
    cy = c->s.cap_y;
    if (e == cudaSuccess) e = ensure(c->s.yfv, cy, yoff[n]);
    size_t cz = c->s.cap_z;
    if (e == cudaSuccess) e = ensure(c->s.ztab, cz, zoff[n]);
    cz = c->s.cap_z;
    if (e == cudaSuccess) e = ensure(c->s.zfv, cz, zoff[n]);
    size_t cp = c->s.cap_prec;
    if (e == cudaSuccess) e = ensure(c->s.aa, cp, aoff[n]);
    cp = c->s.cap_prec;
    if (e == cudaSuccess) e = ensure(c->s.aaf, cp, aoff[n]);
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating tables");
    c->s.cap_x = cx;
    c->s.cap_y = cy;
    c->s.cap_z = cz;
    c->s.cap_prec = cp;
  }

  // ---- kept-atom arrays: sized by what the previous call kept, else 4 atoms per input atom.
  // They are allocated before the column parameters, which point into them.
  int64_t n_atoms_all = 0;
  for (const Job& j : jobs) n_atoms_all += j.n_atoms;
  int64_t cap = c->last_kept > 0 ? c->last_kept + c->last_kept / 4 + 65536 : 4 * n_atoms_all + 65536;
  if (cap > total_cand + 1) cap = total_cand + 1;
  if (!alloc_kept(c, (size_t)cap)) return cuda_fail(c, cudaErrorMemoryAllocation, "allocating binning buffers");

  // ---- column parameters. On the FP32 path every image whose link cells allow it goes
  // to the persistent slab-ring kernel (passes of 16 precession angles); the others,
  // and every image of the FP64 path, get per-image launches.
  std::vector<ColumnParams> cps(n);
  std::vector<int> ring_jobs;  // images of the persistent launch
  std::vector<char> on_ring(n, 0);
  bool dens = false;
  int max_np = 1, ring_np = 1;
  for (int i = 0; i < n; ++i) {
    cps[i] = column_params(c, jobs[i], cell_base[i], xoff[i], yoff[i], zoff[i], aoff[i], flags);
    max_np = std::max(max_np, jobs[i].n_prec);
    if (!(fp32 ? c->fp32_general : c->fp64_general) && ring_eligible(cps[i], (flags & ST_FLAG_STATS) != 0)) {
      on_ring[i] = 1;
      ring_jobs.push_back(i);
      dens = dens || cps[i].use_density;
      ring_np = std::max(ring_np, jobs[i].n_prec);
    }
  }
  if (ring_np > 1) {  // masked ring instances march one angle: masked images then go per image
    std::vector<int> kept;
    for (int r : ring_jobs) {
      if (cps[r].tile_mask) on_ring[r] = 0;
      else kept.push_back(r);
    }
    if (kept.size() != ring_jobs.size()) {
      ring_jobs.swap(kept);
      dens = false;
      for (int r : ring_jobs) dens = dens || cps[r].use_density;
    }
  }
  const bool ring = !ring_jobs.empty();
  const int n_ring = (int)ring_jobs.size();
  const int width = fp32 ? 16 : 4;
  const int passes = (ring_np + width - 1) / width;
  std::vector<ColumnJob> cj;
  std::vector<int> pass_tiles((size_t)passes * kRingShapes, 0);  // per pass, per tile shape
  if (ring) {
    // the density variant of the kernel serves every image of the launch when any image uses it;
    // an image without the density field then gets rho = 1 from use_density = 0 in the sample
    cj.resize((size_t)n_ring * passes);
    for (int pass = 0; pass < passes; ++pass) {
      int tiles[kRingShapes] = {0, 0, 0};
      for (int r = 0; r < n_ring; ++r) {
        ColumnJob& J = cj[(size_t)pass * n_ring + r];
        J.p = cps[ring_jobs[r]];
        J.p.prec_offset = pass * width;
        J.p.accumulate = pass > 0 ? 1 : 0;
        // the average (and bright-field flip) in the store of the image's last pass, unless
        // the image is tile-masked (its epilogue also covers the columns the mask leaves)
        J.p.finalize = (flags & ST_FLAG_AVERAGE) && !J.p.tile_mask && J.p.prec_offset < J.p.n_prec &&
                       J.p.prec_offset + width >= J.p.n_prec;
        J.p.fin_scale = (double)J.p.n_prec;
        J.p.fin_bright = (flags & ST_FLAG_BRIGHT) ? 1 : 0;
        J.pad = 0;
        for (int sh = 0; sh < kRingShapes; ++sh) {
          J.tile_base[sh] = tiles[sh];
          if (J.p.prec_offset < J.p.n_prec) tiles[sh] += column_tiles(J.p, sh);  // fewer angles: none this pass
        }
      }
      for (int sh = 0; sh < kRingShapes; ++sh) pass_tiles[(size_t)pass * kRingShapes + sh] = tiles[sh];
    }
  }

  // ---- per-image tables and job descriptors, staged through pinned memory
  const size_t tab_bytes = (xoff[n] + yoff[n] + zoff[n]) * (sizeof(int2) + sizeof(double)) + aoff[n] * 12;
  const size_t job_bytes = (size_t)n * sizeof(BinParams) + cj.size() * sizeof(ColumnJob);
  // the staging buffer may still feed a previous call's copies (a call that failed before
  // its final synchronisation), and growing it frees it: wait for those copies alone, not
  // for the stream, so that the host builds the tables while work already queued (st_image's
  // atom upload) runs
  if (c->ev_stage) cudaEventSynchronize(c->ev_stage);
  e = ensure_host(c->h_stage, c->cap_stage, tab_bytes + job_bytes + 256);
  if (e == cudaSuccess) e = ensure(c->d_binjobs, c->cap_binjobs, (size_t)n);
  if (e == cudaSuccess && !cj.empty()) e = ensure(c->d_coljobs, c->cap_coljobs, cj.size());
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating job descriptors");
  unsigned char* hp = (unsigned char*)c->h_stage;
  int2* hxt = (int2*)hp;
  int2* hyt = hxt + xoff[n];
  int2* hzt = hyt + yoff[n];
  double* hxf = (double*)(hzt + zoff[n]);
  double* hyf = hxf + xoff[n];
  double* hzf = hyf + yoff[n];
  double* haa = hzf + zoff[n];
  float* haaf = (float*)(haa + aoff[n]);
  unsigned char* hjobs = (unsigned char*)(((uintptr_t)(haaf + aoff[n]) + 63) & ~(uintptr_t)63);
  BinParams* hbp = (BinParams*)hjobs;
  ColumnJob* hcj = (ColumnJob*)(hjobs + (size_t)n * sizeof(BinParams));
  for (int i = 0; i < n; ++i) {
    const st_geom* g = jobs[i].g;
    axis_table(g->Mx, g->a_vox[0], g->lc_delta[0], g->ia_col[0], g->Ex, hxt + xoff[i], hxf + xoff[i]);
    axis_table(g->My, g->a_vox[4], g->lc_delta[1], g->ia_col[4], g->Ey, hyt + yoff[i], hyf + yoff[i]);
    axis_table(g->Mz, g->a_vox[8], g->lc_delta[2], g->ia_col[8], g->Ez, hzt + zoff[i], hzf + zoff[i]);
    depth_table(g, hzt + zoff[i], hzf + zoff[i]);
    for (int k = 0; k < jobs[i].n_prec; ++k) {
      haa[aoff[i] + k] = jobs[i].aa[k];
      haaf[aoff[i] + k] = (float)jobs[i].aa[k];
    }
    for (size_t k = aoff[i] + jobs[i].n_prec; k < aoff[i + 1]; ++k) {  // pad to a pair
      haa[k] = 0.0;
      haaf[k] = 0.f;
    }
    hbp[i] = bin_params(jobs[i], cand_base[i], cell_base[i], atom_base[i]);
  }
  for (size_t k = 0; k < cj.size(); ++k) hcj[k] = cj[k];
  cudaMemcpyAsync(c->s.xtab, hxt, xoff[n] * sizeof(int2), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.ytab, hyt, yoff[n] * sizeof(int2), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.ztab, hzt, zoff[n] * sizeof(int2), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.xfv, hxf, xoff[n] * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.yfv, hyf, yoff[n] * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.zfv, hzf, zoff[n] * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.aa, haa, aoff[n] * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->s.aaf, haaf, aoff[n] * sizeof(float), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->d_binjobs, hbp, (size_t)n * sizeof(BinParams), cudaMemcpyHostToDevice, st);
  if (!cj.empty()) cudaMemcpyAsync(c->d_coljobs, hcj, cj.size() * sizeof(ColumnJob), cudaMemcpyHostToDevice, st);
  if (!c->ev_stage) cudaEventCreateWithFlags(&c->ev_stage, cudaEventDisableTiming);
  if (c->ev_stage) cudaEventRecord(c->ev_stage, st);

  // ---- per-image column launches (general FP32 or FP64 kernel), epilogues, image clearing
  auto columns_per_image = [&](int64_t kept_cap, bool all) -> cudaError_t {
    cudaError_t ce = cudaSuccess;
    for (int i = 0; i < n && ce == cudaSuccess; ++i) {
      if (on_ring[i] && !all) continue;
      ColumnParams cp = cps[i];
      cp.cap = kept_cap;
      if (cp.ix1 <= cp.ix0 || cp.iy1 <= cp.iy0) continue;
      for (int off = 0; off < cp.n_prec && ce == cudaSuccess; off += width) {
        cp.prec_offset = off;
        cp.accumulate = off > 0 ? 1 : 0;
        ce = fp32 ? launch_column_fp32(cp, st) : launch_column_fp64(cp, st);
      }
    }
    return ce;
  };
  bool ring_ok = ring;  // false once a slab overflowed even 256-atom staging: the general kernel
  auto epilogues = [&]() -> cudaError_t {
    cudaError_t ce = cudaSuccess;
    if (!(flags & ST_FLAG_AVERAGE)) return ce;
    for (int i = 0; i < n && ce == cudaSuccess; ++i) {
      const st_geom* g = jobs[i].g;
      if (g->ix1 <= g->ix0 || g->iy1 <= g->iy0) continue;
      if (ring_ok && on_ring[i] && !cps[i].tile_mask) continue;  // finished by the ring's last pass
      ce = launch_epilogue(jobs[i].d_img, g->Mx, g->My, g->ix0, g->ix1, g->iy0, g->iy1, (double)jobs[i].n_prec,
                           (flags & ST_FLAG_BRIGHT) ? 1 : 0, st);
    }
    return ce;
  };
  auto clear_images = [&]() -> cudaError_t {
    // every image is cleared before any column kernel runs, so jobs may share one image
    // buffer with disjoint windows; a shared buffer is cleared once
    cudaError_t ce = cudaSuccess;
    for (int i = 0; i < n && ce == cudaSuccess; ++i) {
      bool seen = false;
      for (int k = 0; k < i && !seen; ++k) seen = jobs[k].d_img == jobs[i].d_img;
      if (!seen) ce = cudaMemsetAsync(jobs[i].d_img, 0, sizeof(double) * (size_t)jobs[i].g->Mx * jobs[i].g->My, st);
    }
    return ce;
  };

  // Everything a call enqueues after the tables: binning, clearing, column kernels,
  // epilogues and the read-back of the counters.  `capturing`: no events, no tuning
  // (the variants and the kernel choice of the eager run are replayed).
  const bool stats = (flags & ST_FLAG_STATS) != 0;
  std::vector<int> pass_variant(passes, 0);
  // a pass's kind (angles per pass, density, precision) and the shape of its images (the first
  // ring image's image and link-cell dimensions): the key of the slab tier an earlier call of
  // this context needed, and of the variant it tuned
  auto big_key = [&](int pass) -> uint64_t {
    uint64_t h = (uint64_t)(ring_np_bucket(std::min(width, ring_np - pass * width)) * 2 + (dens ? 1 : 0)) +
                 (fp32 ? 0u : 1000u);
    if (!ring_jobs.empty()) {
      const st_geom* g = jobs[ring_jobs[0]].g;
      const int dims[6] = {g->Mx, g->My, g->Mz, g->Ex, g->Ey, g->Ez};
      for (int d : dims) h = h * 1000003ull + (uint64_t)d;
    }
    return h;
  };
  int big = c->min_slab_tier;  // slab tier: 128, 192, 256 atoms
  for (int pass = 0; pass < passes; ++pass) {
    auto it = c->ring_big.find(big_key(pass));
    if (it != c->ring_big.end()) big = std::max(big, it->second);
  }
  bool masked = false;  // tile-masked ring jobs take the masked kernel instances
  for (int r : ring_jobs) masked = masked || cps[r].tile_mask != nullptr;
  bool four64 = !fp32 && !ring_jobs.empty();  // the FP64 ring marches four slices per step where all fit
  for (int r : ring_jobs) four64 = four64 && four_slices_fit(jobs[r].g);
  // with_bin false: the column phase only, on the binning already in place
  auto enqueue = [&](bool capturing, bool with_bin) -> cudaError_t {
    cudaError_t ce = cudaSuccess;
    if (!capturing) cudaEventRecord(c->ev[0], st);
    if (with_bin) {
      ce = launch_bin(c->d_binjobs, n, atom_base[n], total_cand, total_cells, cap, c->s, c->b, fp32, st);
      if (ce == cudaSuccess) ce = launch_bin_finalize(c->d_binjobs, n, total_cells, cap, c->s, c->b, fp32, st);
    }
    if (ce == cudaSuccess) ce = clear_images();
    if (!capturing) cudaEventRecord(c->ev[1], st);
    for (int pass = 0; ring_ok && pass < passes && ce == cudaSuccess; ++pass) {
      const int np_pass = std::min(width, ring_np - pass * width);
      auto ring_launch = [&](int v) {
        if (!fp32)
          return launch_column_fp64_ring(c->d_coljobs + (size_t)pass * n_ring, n_ring,
                                         pass_tiles[(size_t)pass * kRingShapes], np_pass, big, masked, four64,
                                         c->d_work, c->s.counters, cap, st);
        return launch_column_fp32_ring(c->d_coljobs + (size_t)pass * n_ring, n_ring,
                                       pass_tiles.data() + (size_t)pass * kRingShapes, np_pass,
                                       dens, stats, v, big, masked, c->d_work, c->s.counters, cap, st);
      };
      if (capturing) {
        ce = ring_launch(pass_variant[pass]);
        continue;
      }
      // the variant tuned for this kind of pass (angles, density) on images of this shape
      const uint64_t key = big_key(pass);
      int v = 0;
      if (c->tune_mode >= 0 && fp32) {
        v = c->tune_mode;
      } else if (c->tune_mode == ST_TUNE_AUTO && !stats && fp32) {  // the FP64 ring has one variant
        auto it = c->ring_tuned.find(key);
        if (it != c->ring_tuned.end()) {
          v = it->second;
        } else if (pass == 0 && pass_tiles[0] >= 4096 && !big && !masked) {
          // autotune on the real work: the first pass overwrites its images, and the tuner
          // ends with the chosen variant's output; keep it for the later calls of this context
          ce = tune_ring(c, ring_launch, cap, st, v);
          if (ce == cudaSuccess && v >= 0) {
            c->ring_tuned[key] = v;
            pass_variant[pass] = v;
            continue;
          }
          v = 0;
        }
      }
      if (ce == cudaSuccess) ce = ring_launch(v);
      pass_variant[pass] = v;
      c->last_ring_variant = stats ? 0 : v;
    }
    if (ce == cudaSuccess && (!ring_ok || n_ring < n)) ce = columns_per_image(cap, !ring_ok);
    if (ce == cudaSuccess) ce = epilogues();
    if (!capturing) cudaEventRecord(c->ev[2], st);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(c->h_counters, c->s.counters, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    return ce;
  };

  for (int attempt = 0;; ++attempt) {
    if (attempt > 0) {
      // grown kept-atom arrays move: point the column parameters and the ring's job table at them
      // (the previous attempt ended with a stream synchronisation, so the staging buffer is free)
      if (!alloc_kept(c, (size_t)cap)) return cuda_fail(c, cudaErrorMemoryAllocation, "allocating binning buffers");
      for (ColumnParams& cp : cps) point_at_kept(c, cp);
      for (size_t k = 0; k < cj.size(); ++k) point_at_kept(c, hcj[k].p);
      if (!cj.empty()) {
        e = cudaMemcpyAsync(c->d_coljobs, hcj, cj.size() * sizeof(ColumnJob), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "copying column jobs");
        if (c->ev_stage) cudaEventRecord(c->ev_stage, st);
      }
    }
    e = enqueue(false, true);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(c, e, "image kernels");
    if ((int64_t)c->h_counters[0] > cap) {
      if (attempt > 0) return fail(c, ST_ERR_ALLOC, "binning capacity did not converge");
      cap = (int64_t)c->h_counters[0] + (int64_t)c->h_counters[0] / 8 + 1024;  // grow and redo
      continue;
    }
    while (ring_ok && c->h_counters[4] != 0 && big < 2) {
      // a slab held more atoms than this tier stages: the column phase again with the next
      // (192, then 256 atoms), and this context keeps it for these kinds of pass on images
      // of this shape
      ++big;
      for (int pass = 0; pass < passes; ++pass) c->ring_big[big_key(pass)] = big;
      cudaMemsetAsync(c->s.counters + 2, 0, 3 * sizeof(unsigned long long), st);
      e = enqueue(false, false);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return cuda_fail(c, e, "image kernels (larger slabs)");
    }
    if (ring_ok && c->h_counters[4] != 0) {
      // a slab held more atoms than the ring kernel stages: recompute every image with the general kernel
      ring_ok = false;
      cudaMemsetAsync(c->s.counters + 2, 0, 3 * sizeof(unsigned long long), st);
      e = clear_images();
      if (e == cudaSuccess) e = columns_per_image(cap, true);
      if (e == cudaSuccess) e = epilogues();
      cudaEventRecord(c->ev[2], st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->h_counters, c->s.counters, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return cuda_fail(c, e, "image kernels (general FP32 kernel)");
    }
    break;
  }
  const bool used_ring = ring_ok;
  const int n_launches = launch_count();  // before the graph recording, which launches nothing now
  if (gout) {
    // record the same work as a CUDA graph for replay (st_plan)
    if (gout->exec) cudaGraphExecDestroy(gout->exec);
    gout->exec = nullptr;
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      const cudaError_t ce = enqueue(true, true);
      e = cudaStreamEndCapture(st, &graph);
      if (ce != cudaSuccess) e = ce;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&gout->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "recording the CUDA graph");
    gout->cap = cap;
    gout->ring = used_ring;
  }
  c->last_kept = (int64_t)c->h_counters[0];
  c->last_column_kernel = !fp32 ? (used_ring && !ring_jobs.empty() ? 4 : 3) : (used_ring ? 2 : 1);

  st_stats& S = c->stats;
  memset(&S, 0, sizeof S);
  S.n_atoms = n_atoms_all;
  S.n_kept = (int64_t)c->h_counters[0];
  S.max_cell_count = (int32_t)c->h_counters[1];
  S.n_tests = (int64_t)c->h_counters[2];
  S.n_accepted = (int64_t)c->h_counters[3];
  for (const Job& j : jobs) S.n_voxels += (int64_t)(j.g->ix1 - j.g->ix0) * (j.g->iy1 - j.g->iy0) * j.g->Mz;
  S.n_prec = max_np;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  S.ms_bin = ms;
  cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]);
  S.ms_column = ms;
  S.column_kernel = c->last_column_kernel;
  S.ring_variant = used_ring ? c->last_ring_variant : -1;
  S.ring_slab_atoms =
      used_ring && !ring_jobs.empty() ? (big == 0 ? ring_variant_slab(S.ring_variant) : big == 1 ? 192 : 256) : 0;
  S.n_launches = n_launches;
  // the reference stops when a link cell needs more than 16 x nMax0 slots; a batch's
  // largest cell is checked against the smallest nMax0 of its images
  int min_nmax0 = 0;
  for (const Job& j : jobs)
    if (j.g->nMax0 > 0 && (min_nmax0 == 0 || j.g->nMax0 < min_nmax0)) min_nmax0 = j.g->nMax0;
  if (min_nmax0 > 0 && S.max_cell_count > 16 * min_nmax0) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "a link cell holds %d atoms, more than 16 x nMax0 = %d (the reference stops in "
             "Lib_LinkCell3d::add0 here)",
             S.max_cell_count, 16 * min_nmax0);
    return fail(c, ST_ERR_CAPACITY, buf);
  }
  return ST_OK;
}

}  // namespace

extern "C" int st_create(st_ctx** out, int device) {
  if (!out) return ST_ERR_ARG;
  *out = nullptr;
  st_ctx* c = new st_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete c;
    return ST_ERR_CUDA;
  }
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_counters, 8 * sizeof(unsigned long long));
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  if (e != cudaSuccess) {
    delete c;
    return ST_ERR_CUDA;
  }
  const char* kv = std::getenv("STEM_FP32_KERNEL");
  c->fp32_general = kv && std::strcmp(kv, "general") == 0;
  const char* kv64 = std::getenv("STEM_FP64_KERNEL");
  c->fp64_general = kv64 && std::strcmp(kv64, "general") == 0;
  const char* ks = std::getenv("STEM_RING_SLABS");
  c->min_slab_tier = !ks ? 0 : std::strcmp(ks, "256") == 0 ? 2 : std::strcmp(ks, "192") == 0 ? 1 : 0;
  *out = c;
  return ST_OK;
}

extern "C" void st_destroy(st_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* dev_ptrs[] = {c->s.tmp_key, c->s.tmp_cell, c->s.tmp_slot, c->s.tmp_f, c->s.perm, c->s.block_sums,
                      c->s.counters, c->s.xtab, c->s.xfv, c->s.ytab, c->s.yfv, c->s.ztab, c->s.zfv, c->s.aa,
                      c->s.aaf, c->b.cell_start, c->b.cell_count, c->b.f64, c->b.cs64, c->b.p32, c->b.cs32,
                      c->b.fr32, c->b.ph32, c->d_x, c->d_img, c->d_blur, c->d_kern, c->d_binjobs, c->d_coljobs, c->d_work, c->d_bx, c->d_bimg,
                      c->d_lvaux, c->d_levels, c->d_text, c->d_pseg, c->d_pstart, c->d_pbad, c->d_geom, c->d_tilt, c->d_keys, c->d_species};
  for (void* p : dev_ptrs)
    if (p) cudaFree(p);
  if (c->h_counters) cudaFreeHost(c->h_counters);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->h_text) cudaFreeHost(c->h_text);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->tev)
    if (e) cudaEventDestroy(e);
  if (c->ev_stage) cudaEventDestroy(c->ev_stage);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int st_tune(st_ctx* c, int32_t mode) {
  if (!c) return ST_ERR_ARG;
  if (mode != ST_TUNE_AUTO && mode != ST_TUNE_OFF && (mode < 0 || mode >= ring_variant_count()))
    return fail(c, ST_ERR_ARG, "tuning mode must be ST_TUNE_AUTO, ST_TUNE_OFF or a variant index");
  c->tune_mode = mode;
  return ST_OK;
}

extern "C" int st_tune_variants(void) { return ring_variant_count(); }

extern "C" const char* st_tune_variant_name(int32_t variant) { return ring_variant_name(variant); }

extern "C" const char* st_last_error(const st_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int st_get_stats(const st_ctx* c, st_stats* out) {
  if (!c || !out) return ST_ERR_ARG;
  *out = c->stats;
  return ST_OK;
}

extern "C" int st_image_device(st_ctx* c, const st_geom* g, const double* d_x, int64_t ldx, int64_t nAtoms,
                               const double* aa, int32_t nPrec, int32_t flags, double* d_img, void* stream) {
  if (!c) return ST_ERR_ARG;
  int rc = validate(c, g, ldx, nAtoms, nPrec);
  if (rc != ST_OK) return rc;
  if (!aa || !d_img || (nAtoms > 0 && !d_x)) return fail(c, ST_ERR_ARG, "null buffer");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  std::vector<Job> jobs{Job{g, d_x, ldx, nAtoms, aa, nPrec, d_img}};
  return run_images(c, jobs, flags, st);
}

namespace {

// Checks the jobs of a batch call and converts them to the internal form.
int collect_jobs(st_ctx* c, int32_t n_jobs, const st_job* jobs, std::vector<Job>& js) {
  if (n_jobs < 1 || !jobs) return fail(c, ST_ERR_ARG, "a batch needs at least one job");
  js.clear();
  js.reserve(n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    const st_job& j = jobs[i];
    int rc = validate(c, j.geom, j.ldx, j.nAtoms, j.nPrec);
    if (rc != ST_OK) {
      c->err = "job " + std::to_string(i) + ": " + c->err;
      return rc;
    }
    if (!j.aa || !j.img || (j.nAtoms > 0 && !j.x))
      return fail(c, ST_ERR_ARG, "job " + std::to_string(i) + ": null buffer");
    js.push_back(Job{j.geom, j.x, j.ldx, j.nAtoms, j.aa, j.nPrec, j.img});
  }
  return ST_OK;
}

// One binning pass and one persistent launch per group of jobs with fewer than 2^31
// candidates (replicas x atoms) in total; most batches are a single group.
int run_batch(st_ctx* c, const std::vector<Job>& js, int32_t flags, cudaStream_t st) {
  const int n_jobs = (int)js.size();
  st_stats total{};
  total.ring_variant = -1;  // none ran
  int first = 0;
  while (first < n_jobs) {
    int last = first;
    int64_t cand = 0;
    while (last < n_jobs) {
      const int64_t jc = (int64_t)js[last].g->nuvw * js[last].n_atoms;
      if (last > first && cand + jc >= 2147483647LL) break;
      cand += jc;
      ++last;
    }
    std::vector<Job> group(js.begin() + first, js.begin() + last);
    const int rc = run_images(c, group, flags, st);
    if (rc != ST_OK) return rc;
    const st_stats& S = c->stats;
    total.n_atoms += S.n_atoms;
    total.n_kept += S.n_kept;
    total.n_tests += S.n_tests;
    total.n_accepted += S.n_accepted;
    total.n_voxels += S.n_voxels;
    total.max_cell_count = std::max(total.max_cell_count, S.max_cell_count);
    total.n_prec = std::max(total.n_prec, S.n_prec);
    total.ms_bin += S.ms_bin;
    total.ms_column += S.ms_column;
    total.column_kernel = std::max(total.column_kernel, S.column_kernel);
    total.ring_variant = std::max(total.ring_variant, S.ring_variant);
    total.ring_slab_atoms = std::max(total.ring_slab_atoms, S.ring_slab_atoms);
    total.n_launches += S.n_launches;
    first = last;
  }
  c->stats = total;
  return ST_OK;
}

}  // namespace

extern "C" int st_image_device_masked(st_ctx* c, const st_geom* g, const double* d_x, int64_t ldx, int64_t nAtoms,
                                      const double* aa, int32_t nPrec, int32_t flags, double* d_img,
                                      const unsigned char* d_tile_mask, int32_t mask_T, void* stream) {
  if (!c) return ST_ERR_ARG;
  int rc = validate(c, g, ldx, nAtoms, nPrec);
  if (rc != ST_OK) return rc;
  if (!aa || !d_img || !d_tile_mask || (nAtoms > 0 && !d_x)) return fail(c, ST_ERR_ARG, "null buffer");
  if (mask_T < 8 || mask_T % 8 != 0 || g->ix0 % 8 != 0 || g->iy0 % 4 != 0)
    return fail(c, ST_ERR_ARG, "mask tiles must be a multiple of 8 pixels and the window origin aligned to them");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  Job j{g, d_x, ldx, nAtoms, aa, nPrec, d_img};
  j.tile_mask = d_tile_mask;
  j.mask_T = mask_T;
  std::vector<Job> jobs{j};
  return run_images(c, jobs, flags, st);
}

extern "C" int st_batch_device(st_ctx* c, int32_t n_jobs, const st_job* jobs, int32_t flags, void* stream) {
  if (!c) return ST_ERR_ARG;
  std::vector<Job> js;
  int rc = collect_jobs(c, n_jobs, jobs, js);
  if (rc != ST_OK) return rc;
  cudaSetDevice(c->device);
  return run_batch(c, js, flags, stream ? (cudaStream_t)stream : c->stream);
}

extern "C" int st_batch(st_ctx* c, int32_t n_jobs, const st_job* jobs, int32_t flags) {
  if (!c) return ST_ERR_ARG;
  std::vector<Job> js;
  int rc = collect_jobs(c, n_jobs, jobs, js);
  if (rc != ST_OK) return rc;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  // device layout: the distinct atom arrays packed to (3, n), then the images
  std::vector<size_t> x_off(n_jobs), img_off(n_jobs);
  std::vector<int> src_of(n_jobs);
  std::vector<int> srcs;  // first job of each distinct atom array
  size_t n_x = 0, n_img = 0;
  for (int i = 0; i < n_jobs; ++i) {
    int s = -1;
    for (int k = (int)srcs.size() - 1; k >= 0 && s < 0; --k) {
      const Job& o = js[srcs[k]];
      if (o.d_x == js[i].d_x && o.ldx == js[i].ldx && o.n_atoms == js[i].n_atoms) s = k;
    }
    if (s < 0) {
      s = (int)srcs.size();
      srcs.push_back(i);
      x_off[i] = n_x;
      n_x += (size_t)3 * js[i].n_atoms;
    } else {
      x_off[i] = x_off[srcs[s]];
    }
    src_of[i] = s;
    img_off[i] = n_img;
    n_img += (size_t)js[i].g->Mx * js[i].g->My;
  }
  cudaError_t e = ensure(c->d_bx, c->cap_bx, n_x > 0 ? n_x : 1);
  if (e == cudaSuccess) e = ensure(c->d_bimg, c->cap_bimg, n_img);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating batch buffers");
  for (int i : srcs) {
    const Job& j = js[i];
    if (j.n_atoms == 0) continue;
    if (j.ldx == 3)
      e = cudaMemcpyAsync(c->d_bx + x_off[i], j.d_x, sizeof(double) * 3 * (size_t)j.n_atoms, cudaMemcpyHostToDevice,
                          st);
    else
      e = cudaMemcpy2DAsync(c->d_bx + x_off[i], 3 * sizeof(double), j.d_x, (size_t)j.ldx * sizeof(double),
                            3 * sizeof(double), (size_t)j.n_atoms, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "copying atoms");
  }
  std::vector<Job> dj(js);
  for (int i = 0; i < n_jobs; ++i) {
    dj[i].d_x = c->d_bx + x_off[i];
    dj[i].ldx = 3;
    dj[i].d_img = c->d_bimg + img_off[i];
  }
  rc = run_batch(c, dj, flags, st);
  if (rc != ST_OK) return rc;
  for (int i = 0; i < n_jobs && e == cudaSuccess; ++i)
    e = cudaMemcpyAsync(js[i].d_img, c->d_bimg + img_off[i], sizeof(double) * (size_t)js[i].g->Mx * js[i].g->My,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying images");
  return ST_OK;
}

// ---------------------------------------------------------------------------
// Plans: batches recorded as CUDA graphs
// ---------------------------------------------------------------------------

struct st_plan {
  struct Group {
    st_ctx* c = nullptr;  // private context: the recorded pointers are its buffers
    std::vector<Job> jobs;
    GraphOut g;
  };
  int device = 0;
  int32_t flags = 0;
  std::vector<st_geom> geoms;
  std::vector<std::vector<double>> aas;
  std::vector<Group> groups;
  std::string err;
  st_stats stats{};
};

namespace {

int plan_fail(st_plan* p, int code, const std::string& msg) {
  p->err = msg;
  return code;
}

// Eager run of one group, recorded into its graph.
int plan_record(st_plan* p, st_plan::Group& G, cudaStream_t st) {
  const int rc = run_images(G.c, G.jobs, p->flags, st, &G.g);
  if (rc != ST_OK) return plan_fail(p, rc, G.c->err);
  return ST_OK;
}

void plan_sum_stats(st_plan* p) {
  st_stats t{};
  for (auto& G : p->groups) {
    const st_stats& S = G.c->stats;
    t.n_atoms += S.n_atoms;
    t.n_kept += S.n_kept;
    t.n_tests += S.n_tests;
    t.n_accepted += S.n_accepted;
    t.n_voxels += S.n_voxels;
    t.max_cell_count = std::max(t.max_cell_count, S.max_cell_count);
    t.n_prec = std::max(t.n_prec, S.n_prec);
    t.ms_bin += S.ms_bin;
    t.ms_column += S.ms_column;
    t.column_kernel = std::max(t.column_kernel, S.column_kernel);
    t.ring_variant = std::max(t.ring_variant, S.ring_variant);
    t.ring_slab_atoms = std::max(t.ring_slab_atoms, S.ring_slab_atoms);
    t.n_launches += S.n_launches;
  }
  p->stats = t;
}

}  // namespace

extern "C" int st_plan_create(st_ctx* c, int32_t n_jobs, const st_job* jobs, int32_t flags, void* stream,
                              st_plan** out) {
  if (!c || !out) return ST_ERR_ARG;
  *out = nullptr;
  std::vector<Job> js;
  int rc = collect_jobs(c, n_jobs, jobs, js);
  if (rc != ST_OK) return rc;
  cudaSetDevice(c->device);
  st_plan* p = new st_plan();
  p->device = c->device;
  p->flags = flags;
  p->geoms.resize(n_jobs);
  p->aas.resize(n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    p->geoms[i] = *js[i].g;
    p->aas[i].assign(js[i].aa, js[i].aa + js[i].n_prec);
    js[i].g = &p->geoms[i];
    js[i].aa = p->aas[i].data();
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  // groups below 2^31 candidates, each with its own context
  int first = 0;
  while (first < n_jobs) {
    int last = first;
    int64_t cand = 0;
    while (last < n_jobs) {
      const int64_t jc = (int64_t)js[last].g->nuvw * js[last].n_atoms;
      if (last > first && cand + jc >= 2147483647LL) break;
      cand += jc;
      ++last;
    }
    st_plan::Group G;
    rc = st_create(&G.c, c->device);
    if (rc != ST_OK) {
      st_plan_destroy(p);
      return fail(c, rc, "creating the plan's context");
    }
    G.c->tune_mode = c->tune_mode;
    G.c->ring_tuned = c->ring_tuned;
    G.c->fp32_general = c->fp32_general;
    G.c->fp64_general = c->fp64_general;
    G.jobs.assign(js.begin() + first, js.begin() + last);
    p->groups.push_back(G);
    first = last;
  }
  for (auto& G : p->groups) {
    // the private stream of the group's context records; the eager run is ordered after
    // the caller's stream (its atoms may just have been written there)
    cudaEvent_t ready;
    cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    cudaEventRecord(ready, st);
    cudaStreamWaitEvent(G.c->stream, ready, 0);
    cudaEventDestroy(ready);
    rc = plan_record(p, G, G.c->stream);
    if (rc != ST_OK) {
      const std::string msg = p->err;
      st_plan_destroy(p);
      return fail(c, rc, "recording the plan: " + msg);
    }
  }
  plan_sum_stats(p);
  *out = p;
  return ST_OK;
}

extern "C" int st_plan_launch(st_plan* p, void* stream) {
  if (!p) return ST_ERR_ARG;
  cudaSetDevice(p->device);
  cudaStream_t st = (cudaStream_t)stream;
  for (auto& G : p->groups) {
    const cudaError_t e = cudaGraphLaunch(G.g.exec, st);
    if (e != cudaSuccess) return plan_fail(p, ST_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
  }
  return ST_OK;
}

extern "C" int st_plan_wait(st_plan* p, void* stream) {
  if (!p) return ST_ERR_ARG;
  cudaSetDevice(p->device);
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return plan_fail(p, ST_ERR_CUDA, std::string("plan replay: ") + cudaGetErrorString(e));
  // the groups ran one after another on the stream and share nothing, so each group's
  // counters (read back by its last graph node) tell whether its images are complete
  int64_t kept = 0;
  for (auto& G : p->groups) {
    const unsigned long long* h = G.c->h_counters;
    kept += (int64_t)h[0];
    if ((int64_t)h[0] > G.g.cap || (G.g.ring && h[4] != 0)) {
      const int rc = plan_record(p, G, G.c->stream);  // eager recompute, then record again
      if (rc != ST_OK) return rc;
      e = cudaStreamSynchronize(G.c->stream);
      if (e != cudaSuccess) return plan_fail(p, ST_ERR_CUDA, std::string("plan rerun: ") + cudaGetErrorString(e));
    }
  }
  plan_sum_stats(p);
  p->stats.n_kept = std::max(p->stats.n_kept, kept);
  return ST_OK;
}

extern "C" int st_plan_stats(const st_plan* p, st_stats* out) {
  if (!p || !out) return ST_ERR_ARG;
  *out = p->stats;
  return ST_OK;
}

extern "C" const char* st_plan_last_error(const st_plan* p) { return p ? p->err.c_str() : "null plan"; }

extern "C" void st_plan_destroy(st_plan* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  for (auto& G : p->groups) {
    if (G.g.exec) cudaGraphExecDestroy(G.g.exec);
    st_destroy(G.c);
  }
  delete p;
}

extern "C" int st_image(st_ctx* c, const st_geom* g, const double* x, int64_t ldx, int64_t nAtoms, const double* aa,
                        int32_t nPrec, int32_t flags, double* img) {
  if (!c) return ST_ERR_ARG;
  int rc = validate(c, g, ldx, nAtoms, nPrec);
  if (rc != ST_OK) return rc;
  if (!img || !aa || (nAtoms > 0 && !x)) return fail(c, ST_ERR_ARG, "null buffer");
  cudaSetDevice(c->device);
  cudaError_t e = ensure(c->d_x, c->cap_x, (size_t)3 * (nAtoms > 0 ? nAtoms : 1));
  if (e == cudaSuccess) e = ensure(c->d_img, c->cap_img, (size_t)g->Mx * g->My);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating image buffers");
  if (nAtoms > 0) {
    // x(1:3, :) of a Fortran (ldx, nAtoms) array, packed to (3, nAtoms)
    if (ldx == 3)
      e = cudaMemcpyAsync(c->d_x, x, sizeof(double) * 3 * (size_t)nAtoms, cudaMemcpyHostToDevice, c->stream);
    else
      e = cudaMemcpy2DAsync(c->d_x, 3 * sizeof(double), x, (size_t)ldx * sizeof(double), 3 * sizeof(double),
                            (size_t)nAtoms, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "copying atoms");
  }
  rc = st_image_device(c, g, c->d_x, 3, nAtoms, aa, nPrec, flags, c->d_img, c->stream);
  if (rc != ST_OK) return rc;
  e = cudaMemcpyAsync(img, c->d_img, sizeof(double) * (size_t)g->Mx * g->My, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying image");
  return ST_OK;
}

namespace {

// kernel(0:Nk) of gaussianBlurImage: Nk = max(5, ceiling(5 t)), exp(-k^2 / (2 t^2)).
int blur_kernel(double t, std::vector<double>& k) {
  int nk = (int)std::ceil(t * 5);
  if (nk < 5) nk = 5;
  k.assign(nk + 1, 0.0);
  const double i2s2 = 1 / (2 * t * t);
  k[0] = 1.0;
  for (int i = 1; i <= nk; ++i) k[i] = std::exp(-(i * i * i2s2));
  return nk;
}

}  // namespace

extern "C" int st_blur_device(st_ctx* c, const double* d_in, int32_t nx, int32_t ny, double t, double* d_out,
                              void* stream) {
  if (!c) return ST_ERR_ARG;
  if (!d_in || !d_out || nx < 1 || ny < 1) return fail(c, ST_ERR_ARG, "invalid blur arguments");
  if (!(t > 0.0) || !(t < 1e6)) return fail(c, ST_ERR_ARG, "blur width t must be in (0, 1e6) pixels");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  std::vector<double> k;
  const int nk = blur_kernel(t, k);
  const size_t n = (size_t)nx * ny;
  cudaError_t e = ensure(c->d_blur, c->cap_blur, 3 * n + nx);
  if (e == cudaSuccess) e = ensure(c->d_kern, c->cap_kern, (size_t)nk + 1);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating blur buffers");
  e = cudaMemcpyAsync(c->d_kern, k.data(), (nk + 1) * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_blur(d_in, c->d_blur + n, d_out, nx, ny, c->d_kern, nk, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "blur");
  return ST_OK;
}

extern "C" int st_blur(st_ctx* c, const double* in, int32_t nx, int32_t ny, double t, double* out) {
  if (!c) return ST_ERR_ARG;
  if (!in || !out || nx < 1 || ny < 1) return fail(c, ST_ERR_ARG, "invalid blur arguments");
  cudaSetDevice(c->device);
  const size_t n = (size_t)nx * ny;
  cudaError_t e = ensure(c->d_blur, c->cap_blur, 3 * n + nx);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating blur buffers");
  e = cudaMemcpyAsync(c->d_blur, in, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying blur input");
  // input at d_blur[0, n), scratch at [n, 2n + nx), output at [2n + nx, 3n + nx)
  double* d_out = c->d_blur + 2 * n + nx;
  int rc = st_blur_device(c, c->d_blur, nx, ny, t, d_out, c->stream);
  if (rc != ST_OK) return rc;
  e = cudaMemcpyAsync(out, d_out, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying blur output");
  return ST_OK;
}

// ---------------------------------------------------------------------------------------
// Output files (src/d2bi.f90:1429-1457 and 1509-1538): the levels and the f12.7 records on
// the GPU (k_output.cu), the header and the PNG container on the host (host_output.cpp).
namespace {

// write bytes to <path>.tmp, then rename it to path (as d2bi does with mv)
int write_file(st_ctx* c, const char* path, const std::vector<std::pair<const char*, size_t>>& parts) {
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(c, ST_ERR_ARG, "cannot open " + tmp + " for writing");
  bool ok = true;
  for (const auto& p : parts) ok = ok && std::fwrite(p.first, 1, p.second, f) == p.second;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(c, ST_ERR_ARG, std::string("writing ") + path + " failed");
  }
  return ST_OK;
}

}  // namespace

extern "C" int st_png_levels_device(st_ctx* c, const double* d_img, int32_t nx, int32_t ny, double iso_min,
                                    double iso_max, uint16_t* d_levels, void* stream) {
  if (!c) return ST_ERR_ARG;
  if (!d_img || !d_levels || nx < 1 || ny < 1) return fail(c, ST_ERR_ARG, "invalid PNG level arguments");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  cudaError_t e = ensure(c->d_lvaux, c->cap_lvaux, (size_t)2 * kLevelParts + 2);
  if (e == cudaSuccess)
    e = launch_png_levels(d_img, nx, ny, iso_min, iso_max, c->d_lvaux, c->d_lvaux + 2 * kLevelParts, d_levels, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "PNG levels");
  return ST_OK;
}

extern "C" int st_write_png(st_ctx* c, const char* path, const double* img, int32_t nx, int32_t ny, double iso_min,
                            double iso_max, double blur_t) {
  if (!c) return ST_ERR_ARG;
  if (!path || !img || nx < 1 || ny < 1) return fail(c, ST_ERR_ARG, "invalid PNG arguments");
  cudaSetDevice(c->device);
  const size_t n = (size_t)nx * ny;
  cudaError_t e = ensure(c->d_blur, c->cap_blur, 3 * n + nx);
  if (e == cudaSuccess) e = ensure(c->d_levels, c->cap_levels, n);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating PNG buffers");
  e = cudaMemcpyAsync(c->d_blur, img, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the PNG image");
  const double* src = c->d_blur;
  if (blur_t > 0) {  // outputImgAsPng blurs first when png_blur > 0
    double* d_out = c->d_blur + 2 * n + nx;
    const int rc = st_blur_device(c, c->d_blur, nx, ny, blur_t, d_out, c->stream);
    if (rc != ST_OK) return rc;
    src = d_out;
  }
  int rc = st_png_levels_device(c, src, nx, ny, iso_min, iso_max, c->d_levels, c->stream);
  if (rc != ST_OK) return rc;
  std::vector<uint16_t> lv(n);
  e = cudaMemcpyAsync(lv.data(), c->d_levels, n * sizeof(uint16_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "PNG levels");
  const int64_t cap = st_png16_bytes(nx, ny);
  std::vector<uint8_t> png((size_t)cap);
  int64_t len = 0;
  rc = st_encode_png16(lv.data(), nx, ny, png.data(), cap, &len);
  if (rc != ST_OK) return fail(c, rc, "PNG encoding (image too large for one IDAT chunk)");
  return write_file(c, path, {{(const char*)png.data(), (size_t)len}});
}

extern "C" int st_format_dat_device(st_ctx* c, const double* d_v, int64_t n, char* d_text, int64_t cap,
                                    void* stream) {
  if (!c) return ST_ERR_ARG;
  if (!d_v || !d_text || n < 0 || cap < st_dat_text_bytes(n)) return fail(c, ST_ERR_ARG, "invalid .dat arguments");
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const cudaError_t e = launch_format_dat(d_v, n, d_text, st);
  if (e != cudaSuccess) return cuda_fail(c, e, ".dat records");
  return ST_OK;
}

extern "C" int st_write_dat(st_ctx* c, const char* path, const st_dat_header* h, const double* img, int32_t nx,
                            int32_t ny) {
  if (!c) return ST_ERR_ARG;
  if (!path || !h || !img || nx < 1 || ny < 1) return fail(c, ST_ERR_ARG, "invalid .dat arguments");
  std::vector<char> head(4096);
  int64_t hlen = 0;
  int rc = st_format_dat_header(h, nx, ny, head.data(), (int64_t)head.size(), &hlen);
  if (rc != ST_OK) return fail(c, rc, "invalid .dat header");
  cudaSetDevice(c->device);
  const size_t n = (size_t)nx * ny;
  const int64_t tb = st_dat_text_bytes((int64_t)n);
  cudaError_t e = ensure(c->d_img, c->cap_img, n);
  if (e == cudaSuccess) e = ensure(c->d_text, c->cap_text, (size_t)tb);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating .dat buffers");
  e = cudaMemcpyAsync(c->d_img, img, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the .dat image");
  rc = st_format_dat_device(c, c->d_img, (int64_t)n, c->d_text, tb, c->stream);
  if (rc != ST_OK) return rc;
  std::vector<char> text((size_t)tb);
  e = cudaMemcpyAsync(text.data(), c->d_text, (size_t)tb, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, ".dat records");
  return write_file(c, path, {{head.data(), (size_t)hlen}, {text.data(), (size_t)tb}});
}

// ---------------------------------------------------------------------------------------
// Input: the atom lines of LAMMPS data files parsed on the GPU (k_parse.cu)

extern "C" int st_parse_atoms_device(st_ctx* c, const char* d_text, int64_t n_bytes, int64_t n_atoms, double* d_x,
                                     int64_t ldx, int32_t* d_types, int64_t* bad_line, void* stream) {
  if (!c) return ST_ERR_ARG;
  if (bad_line) *bad_line = -1;
  if (!d_text || n_bytes < 0 || n_atoms < 0 || !d_x || ldx < 3)
    return fail(c, ST_ERR_ARG, "invalid atom-line arguments");
  if (n_atoms == 0) return ST_OK;
  if (n_bytes == 0) {
    if (bad_line) *bad_line = 0;
    return fail(c, ST_ERR_ARG, "no atom lines");
  }
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  cudaError_t e = ensure(c->d_pseg, c->cap_pseg, (size_t)parse_segments(n_bytes) + 1);
  if (e == cudaSuccess) e = ensure(c->d_pstart, c->cap_pstart, (size_t)n_atoms);
  if (e == cudaSuccess) e = ensure(c->d_pbad, c->cap_pbad, 1);
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating parse buffers");
  e = launch_parse_atoms(d_text, n_bytes, n_atoms, c->d_pseg, c->d_pstart, d_x, ldx, d_types, c->d_pbad, st);
  unsigned long long bad = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_counters, c->d_pbad, sizeof bad, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "parsing atom lines");
  bad = c->h_counters[0];
  if (bad != ~0ull) {
    if (bad_line) *bad_line = (int64_t)bad;
    return fail(c, ST_ERR_ARG, "atom line " + std::to_string(bad + 1) +
                                   " of the Atoms block is missing or malformed (id type x y z expected)");
  }
  return ST_OK;
}

extern "C" int st_read_lammps(st_ctx* c, const char* path, const st_lammps_info* info, double* x, int64_t ldx,
                              int32_t* types) {
  if (!c) return ST_ERR_ARG;
  if (!path || !info || !x || ldx < 3 || info->n_atoms < 0 || info->data_offset < 0)
    return fail(c, ST_ERR_ARG, "invalid LAMMPS read arguments");
  const int64_t n = info->n_atoms;
  if (n == 0) return ST_OK;
  cudaSetDevice(c->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, ST_ERR_ARG, std::string("cannot open ") + path);
  std::fseek(f, 0, SEEK_END);
  const long long size = std::ftell(f);
  const long long nb = size - info->data_offset;
  if (nb <= 0) {
    std::fclose(f);
    return fail(c, ST_ERR_ARG, "no atom lines after the header");
  }
  cudaError_t e = ensure_host(c->h_text, c->cap_htext, (size_t)nb);
  if (e == cudaSuccess) e = ensure(c->d_text, c->cap_text, (size_t)nb);
  if (e == cudaSuccess) e = ensure(c->d_x, c->cap_x, (size_t)3 * n);
  if (e != cudaSuccess) {
    std::fclose(f);
    return cuda_fail(c, e, "allocating read buffers");
  }
  std::fseek(f, info->data_offset, SEEK_SET);
  const size_t got = std::fread(c->h_text, 1, (size_t)nb, f);
  std::fclose(f);
  if (got != (size_t)nb) return fail(c, ST_ERR_ARG, std::string("reading ") + path + " failed");
  e = cudaMemcpyAsync(c->d_text, c->h_text, (size_t)nb, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the atom lines");
  int32_t* d_types = nullptr;
  if (types) {
    e = ensure(c->d_bimg, c->cap_bimg, (size_t)(n + 1) / 2);  // n int32 in the batch-image scratch
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating read buffers");
    d_types = reinterpret_cast<int32_t*>(c->d_bimg);
  }
  int64_t bad = -1;
  const int rc = st_parse_atoms_device(c, c->d_text, nb, n, c->d_x, 3, d_types, &bad, c->stream);
  if (rc != ST_OK) return rc;
  std::vector<double> xs;
  double* dst = x;
  if (ldx != 3) {
    xs.resize((size_t)3 * n);
    dst = xs.data();
  }
  e = cudaMemcpyAsync(dst, c->d_x, (size_t)3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && types)
    e = cudaMemcpyAsync(types, d_types, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the positions");
  if (ldx != 3)
    for (int64_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) x[i * ldx + k] = xs[(size_t)3 * i + k];
  return ST_OK;
}

extern "C" int st_parse_xyz_device(st_ctx* c, const char* d_text, int64_t n_bytes, int64_t n_atoms,
                                   int32_t n_columns, double* d_x, int64_t ldx, int32_t* d_types, int32_t* n_species,
                                   char* species, int32_t species_cap, int64_t* bad_line, void* stream) {
  if (!c) return ST_ERR_ARG;
  if (bad_line) *bad_line = -1;
  if (n_species) *n_species = 0;
  if (!d_text || n_bytes < 0 || n_atoms < 0 || !d_x || ldx < 1 || n_columns < 3 || n_columns > 1000 ||
      species_cap < 0 || (species_cap > 0 && !species))
    return fail(c, ST_ERR_ARG, "invalid xyz atom-line arguments");
  if (n_atoms == 0) return ST_OK;
  if (n_bytes == 0) {
    if (bad_line) *bad_line = 0;
    return fail(c, ST_ERR_ARG, "no atom lines");
  }
  cudaSetDevice(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  cudaError_t e = ensure(c->d_pseg, c->cap_pseg, (size_t)parse_segments(n_bytes) + 1);
  if (e == cudaSuccess) e = ensure(c->d_pstart, c->cap_pstart, (size_t)n_atoms);
  if (e == cudaSuccess) e = ensure(c->d_pbad, c->cap_pbad, 1);
  if (e == cudaSuccess) e = ensure(c->d_keys, c->cap_keys, (size_t)n_atoms);
  if (e == cudaSuccess) e = ensure(c->d_species, c->cap_species, (size_t)species_scratch(n_atoms));
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating parse buffers");
  e = launch_parse_xyz(d_text, n_bytes, n_atoms, n_columns, c->d_pseg, c->d_pstart, d_x, ldx, c->d_keys, c->d_pbad,
                       st);
  unsigned long long bad = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_counters, c->d_pbad, sizeof bad, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "parsing atom lines");
  bad = c->h_counters[0];
  if (bad != ~0ull) {
    if (bad_line) *bad_line = (int64_t)bad;
    return fail(c, ST_ERR_ARG, "atom line " + std::to_string(bad + 1) +
                                   " of the .xyz file is missing or malformed (species and " +
                                   std::to_string(n_columns) + " numbers expected)");
  }
  e = launch_species(c->d_keys, n_atoms, c->d_species, d_types, st);
  std::vector<unsigned long long> table(1001);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(table.data(), c->d_species + species_table_offset(), 1001 * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "numbering species");
  const int cnt = (int)table[1000];
  if (cnt > ST_XYZ_SPECIES_MAX) return fail(c, ST_ERR_ARG, "more than 1000 species names in the .xyz file");
  if (n_species) *n_species = cnt;
  for (int k = 0; k < cnt && k < species_cap; ++k)
    for (int j = 0; j < ST_XYZ_NAME_LEN; ++j) species[k * ST_XYZ_NAME_LEN + j] = (char)((table[k] >> (8 * j)) & 0xFF);
  return ST_OK;
}

extern "C" int st_read_xyz(st_ctx* c, const char* path, const st_xyz_info* info, double* x, int64_t ldx,
                           int32_t* types, int32_t* n_species, char* species, int32_t species_cap) {
  if (!c) return ST_ERR_ARG;
  if (!path || !info || !x || ldx < 1 || info->lammps || info->data_offset < 0 || info->n_columns < 3)
    return fail(c, ST_ERR_ARG, "invalid xyz read arguments");
  if (info->n_read < 0) return fail(c, ST_ERR_ARG, "the atom count line does not read as an integer");
  if (info->n_read > info->n_atoms) return fail(c, ST_ERR_ARG, "more atoms on the count line than expected");
  const int64_t n = info->n_read;
  if (n_species) *n_species = 0;
  if (n == 0) return ST_OK;
  cudaSetDevice(c->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, ST_ERR_ARG, std::string("cannot open ") + path);
  std::fseek(f, 0, SEEK_END);
  const long long size = std::ftell(f);
  const long long nb = size - info->data_offset;
  if (nb <= 0) {
    std::fclose(f);
    return fail(c, ST_ERR_ARG, "no atom lines after the header");
  }
  const int nc = info->n_columns;
  const int64_t lx = ldx < nc ? ldx : nc;  // columns kept
  cudaError_t e = ensure_host(c->h_text, c->cap_htext, (size_t)nb);
  if (e == cudaSuccess) e = ensure(c->d_text, c->cap_text, (size_t)nb);
  if (e == cudaSuccess) e = ensure(c->d_x, c->cap_x, (size_t)lx * n);
  if (e != cudaSuccess) {
    std::fclose(f);
    return cuda_fail(c, e, "allocating read buffers");
  }
  std::fseek(f, info->data_offset, SEEK_SET);
  const size_t got = std::fread(c->h_text, 1, (size_t)nb, f);
  std::fclose(f);
  if (got != (size_t)nb) return fail(c, ST_ERR_ARG, std::string("reading ") + path + " failed");
  e = cudaMemcpyAsync(c->d_text, c->h_text, (size_t)nb, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the atom lines");
  int32_t* d_types = nullptr;
  if (types) {
    e = ensure(c->d_bimg, c->cap_bimg, (size_t)(n + 1) / 2);  // n int32 in the batch-image scratch
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating read buffers");
    d_types = reinterpret_cast<int32_t*>(c->d_bimg);
  }
  int64_t bad = -1;
  const int rc = st_parse_xyz_device(c, c->d_text, nb, n, nc, c->d_x, lx, d_types, n_species, species, species_cap,
                                     &bad, c->stream);
  if (rc != ST_OK) return rc;
  std::vector<double> xs;
  double* dst = x;
  if (ldx != lx) {
    xs.resize((size_t)lx * n);
    dst = xs.data();
  }
  e = cudaMemcpyAsync(dst, c->d_x, (size_t)lx * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && types)
    e = cudaMemcpyAsync(types, d_types, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "copying the positions");
  if (ldx != lx)
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = 0; k < lx; ++k) x[i * ldx + k] = xs[(size_t)lx * i + k];
  return ST_OK;
}

// ---------------------------------------------------------------------------------------
// Accessors for the host translation units (host_d2bi.cpp: geometry over the atoms)
namespace stem {
cudaStream_t ctx_stream(st_ctx* c, void* stream) {
  cudaSetDevice(c->device);
  return stream ? (cudaStream_t)stream : c->stream;
}
int ctx_fail(st_ctx* c, int code, const char* msg) { return fail(c, code, msg); }
int ctx_cuda_fail(st_ctx* c, cudaError_t e, const char* where) { return cuda_fail(c, e, where); }
cudaError_t ctx_geom_scratch(st_ctx* c, double** part, double** out) {
  const size_t np = (size_t)kExtentBlocks * kMaxRot * 6;
  const cudaError_t e = ensure(c->d_geom, c->cap_geom, np + 6 * kMaxRot);
  if (e == cudaSuccess) {
    *part = c->d_geom;
    *out = c->d_geom + np;
  }
  return e;
}
cudaError_t ctx_tilt_scratch(st_ctx* c, size_t n_doubles, double** p) {
  const cudaError_t e = ensure(c->d_tilt, c->cap_tilt, n_doubles);
  if (e == cudaSuccess) *p = c->d_tilt;
  return e;
}
}  // namespace stem

