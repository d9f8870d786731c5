// The slab-ring FP32 column launch: the tuning variants of the slab-ring kernel
// (k_column_v3.cuh) behind one entry point.
//
// Variants (st_tune, the autotuner's candidates), all computing the pixel loop of
// computeD2BI_img (Lib_DynamicalTwoBeamImaging.f90:1870-1900) on the slab ring:
//   0  8 x 4 columns per warp, 128-atom slabs, 4 CTAs per SM
//   1  8 x 4, 96-atom slabs, 5 CTAs per SM (3 with 16 angles)
//   2  4 x 8, 128-atom slabs
//   3  4 x 8, 96-atom slabs
//   4  16 x 2, 128-atom slabs
//   5  16 x 2, 96-atom slabs
// Slab tiers 1 and 2 (192 and 256 atoms) use 8 x 4 tiles.  Statistics use variant 0's
// kernel; a tile-masked launch uses its variant's tile shape, so the masked columns equal
// the plain image's bit for bit.
#include "internal.h"

namespace stem {

namespace {
constexpr int kShapeTX[kRingShapes] = {8, 4, 16};
constexpr int kVariants = 6;
const char* const kNames[kVariants] = {"8x4 slab128", "8x4 slab96", "4x8 slab128", "4x8 slab96", "16x2 slab128",
                                       "16x2 slab96"};
}  // namespace

int column_tiles(const ColumnParams& p, int shape) {
  const int tx = kShapeTX[shape], ty = 32 / tx;
  const int Wd = p.ix1 - p.ix0, Hd = p.iy1 - p.iy0;
  if (Wd <= 0 || Hd <= 0) return 0;
  return ((Wd + tx - 1) / tx) * ((Hd + ty - 1) / ty);
}

int ring_variant_count() { return kVariants; }

int ring_np_bucket(int max_np) { return max_np <= 1 ? 1 : max_np <= 2 ? 2 : max_np <= 4 ? 4 : max_np <= 8 ? 8 : 16; }

int ring_variant_slab(int variant) { return variant == 1 || variant == 3 || variant == 5 ? 96 : 128; }

const char* ring_variant_name(int variant) {
  return variant >= 0 && variant < kVariants ? kNames[variant] : "invalid";
}

cudaError_t launch_column_fp32_ring(const ColumnJob* d_jobs, int n_jobs, const int* tiles, int max_np, bool density,
                                    bool stats, int variant, int slab_tier, bool masked, unsigned* work,
                                    const unsigned long long* counters, int64_t cap, cudaStream_t st) {
  if (variant < 0 || variant >= kVariants) variant = 0;
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  if (tiles[0] <= 0) return cudaSuccess;
  if (masked && (max_np != 1 || stats)) return cudaErrorInvalidValue;
  ring3::Ring3Args a{d_jobs, n_jobs, tiles, density, stats, masked, stats ? 0 : variant, slab_tier, work, counters,
                     cap, st};
  switch (ring_np_bucket(max_np)) {
    case 1: return ring3::ring3_launch_np<1>(a);
    case 2: return ring3::ring3_launch_np<2>(a);
    case 4: return ring3::ring3_launch_np<4>(a);
    case 8: return ring3::ring3_launch_np<8>(a);
    default: return ring3::ring3_launch_np<16>(a);
  }
}

}  // namespace stem
