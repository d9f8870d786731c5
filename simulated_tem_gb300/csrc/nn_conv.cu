// Convolution kernels of the learned corrector on the fifth-generation tensor cores.
//
// Forward (and input-gradient) convolution, 3 x 3 ("same" padding) or 1 x 1, over NHWC
// BF16 activations: an implicit GEMM D[p, co] = sum_k A[p, k] B[co, k], p the output
// pixel, k = (tap, ci).  A tile is 128 consecutive pixels of one image row (two adjacent
// rows for BN <= 64) x BN output channels; each row's FP32 accumulator lives in TMEM (BN
// columns).  No thread
// touches the operands: one thread moves them, one issues the MMAs, four warps drain TMEM.
//
// Per chunk of KC input channels the producer loads a halo tile: the input rows y - 1 ..
// y + R (R output rows; from y for 1 x 1), pixels x0 - 1 .. x0 + 128, as (KC / 8) slabs
// of 130 rows x 16 bytes (8 channels) per input row; output row y + q reads the input
// rows from y - 1 + q, and every row's MMAs read each weight slot.  In such a slab the rows are 16 bytes apart, so
// the K-major core matrices (8 rows x 16 bytes) of the pixels shifted by dx start 16 dx
// bytes further: all nine taps read the same tile through shifted descriptors (LBO =
// slab pitch between 8-channel groups, SBO = 128 between 8-pixel groups).  Outside the
// image the TMA box is zero-filled: the padding.  The weights of each (tap, chunk) come
// into a ring of B slots ([BN rows][16 bytes] per 8-channel group) as one contiguous bulk
// copy: before the convolution a small kernel writes the weights in exactly that order
// (per output-channel tile, chunk and tap), so the copy reads whole 32-byte sectors
// (a tensor box of 16-byte rows 2 x taps x Cin bytes apart used half of each sector).
//
// The kernel is persistent: a CTA takes tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...
// and its rings run on from one tile to the next, so the loads of the next tile overlap
// the MMAs of this one; two TMEM accumulators let the epilogue of one tile overlap the
// MMAs of the next.  Warp roles (192 threads): warps 0-3 epilogue (warp w reads TMEM lanes
// 32w .. 32w + 31), warp 4 lane 0 loads, warp 5 lane 0 issues the MMAs.  mbarriers: A
// stages and B slots full (TMA bytes) / empty (MMA commit); accumulators full (MMA
// commit) / empty (one arrival per epilogue warp).
//
// Every wait on an mbarrier is bounded and watches a shared abort flag; a wait that runs
// out records an error in g_nn_error, the producer waits (bounded) for every load it
// issued, the MMAs issued so far are waited for, and TMEM is always freed.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "nn.h"
#include "tc_sm100.cuh"

namespace stem {
namespace nn {

__device__ int g_nn_error = 0;  // first failure code of a corrector kernel (0 = none)

namespace {

constexpr int kThreads = 128;              // weight-gradient kernel
constexpr int kTileThreads = 192;          // persistent forward kernel: 4 epilogue warps, producer, issuer
constexpr uint32_t kWaitLimit = 1u << 20;  // polls of an mbarrier before giving up (about a second)
constexpr int kTileX = 128;                // output pixels per tile (one image row)
constexpr int kHalo = kTileX + 2;          // input pixels per halo row
constexpr int kSlab = 2176;                // bytes per (input row, 8 channels) slab: 130 x 16 rounded to 128
// weight ring depth: as many slots as leave room for two CTAs per SM (TMEM allows two at
// BN = 128); each slot holds KC/16 MMAs of work, and the ring must cover the latency of
// the TMA loads that refill it
__host__ __device__ constexpr int b_slots(int BN) { return BN >= 128 ? 7 : 8; }
// output rows per tile: two rows read each weight slot and share two halo rows, but need
// twice the TMEM columns; at BN = 128 that would leave one CTA per SM (measured slower)
__host__ __device__ constexpr int rows_per_tile(int BN) { return BN >= 128 ? 1 : 2; }

struct ConvArgs {
  const unsigned char* wb;    // blocked weights: [Cout tile][chunk][tap] blocks of one B slot
  const float* bias;          // [Cout] or null
  const __nv_bfloat16* mask;  // [B][H][W][Cout] or null: outputs where mask <= 0 are zeroed
  void* y;                    // [B][H][W][Cout], BF16 or FP32
  int B, H, W, Cin, Cout, taps, relu, y_fp32;
  int n_ntiles;               // output-channel tiles
  int xtiles, n_tiles;        // tiles: (x tile, row group, image, channel tile)
};

template <int BN, int KC, int NR>
struct TSmem {
  static constexpr int kBSlots = b_slots(BN);
  alignas(1024) unsigned char a[2][(NR + rows_per_tile(BN) - 1) * (KC / 8) * kSlab];
  alignas(1024) unsigned char b[kBSlots][(KC / 8) * BN * 16];
  alignas(8) unsigned long long a_full[2], a_empty[2], b_full[kBSlots], b_empty[kBSlots], acc_full[2],
      acc_empty[2], done;
  uint32_t tmem;
  int abort;
};

// bounded wait that gives up early when another role has aborted
__device__ __forceinline__ bool wait_or_abort(uint32_t mbar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    if (tc::mbar_try_wait(mbar, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  return false;
}

struct Tile {
  int xt, y, img, n0;  // y: the first of the tile's rows_per_tile(BN) output rows
};
__device__ __forceinline__ Tile tile_of(const ConvArgs& a, int t, int BN) {
  Tile r;
  r.xt = t % a.xtiles;
  int rest = t / a.xtiles;
  const int rows = rows_per_tile(BN), groups = (a.H + rows - 1) / rows;
  r.y = (rest % groups) * rows;
  rest /= groups;
  r.img = rest % a.B;
  r.n0 = (rest / a.B) * BN;
  return r;
}

// NR = 3 input rows for a 3 x 3 convolution, 1 for 1 x 1 (then taps = 1).
template <int BN, int KC, int NR>
__global__ void __launch_bounds__(kTileThreads) k_conv_fwd(const ConvArgs a, const __grid_constant__ CUtensorMap tmx) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TSmem<BN, KC, NR>& S = *reinterpret_cast<TSmem<BN, KC, NR>*>(
      smem_raw + ((1024 - ((uintptr_t)smem_raw & 1023)) & 1023));
  constexpr int kTaps = NR == 3 ? 9 : 1;
  constexpr int kG = KC / 8;                        // 8-channel groups per chunk
  constexpr int kRowsPerTile = rows_per_tile(BN);
  constexpr int kInRows = NR + kRowsPerTile - 1;   // halo rows per tile
  constexpr uint32_t kBytesA = kInRows * kG * kHalo * 16;
  constexpr uint32_t kBytesB = kG * BN * 16;
  constexpr uint32_t kCols = 2 * kRowsPerTile * BN;  // two buffers of one accumulator per row
  constexpr int kBSlots = TSmem<BN, KC, NR>::kBSlots;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int nchunks = a.Cin / KC;
  volatile int* abort = &S.abort;

  if (warp == 5) tc::tmem_alloc(tc::smem_addr(&S.tmem), kCols);
  if (t == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(tc::smem_addr(&S.a_full[i]), 1);
      tc::mbar_init(tc::smem_addr(&S.a_empty[i]), 1);
      tc::mbar_init(tc::smem_addr(&S.acc_full[i]), 1);
      tc::mbar_init(tc::smem_addr(&S.acc_empty[i]), 4);
    }
    for (int i = 0; i < kBSlots; ++i) {
      tc::mbar_init(tc::smem_addr(&S.b_full[i]), 1);
      tc::mbar_init(tc::smem_addr(&S.b_empty[i]), 1);
    }
    tc::mbar_init(tc::smem_addr(&S.done), 1);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;

  if (warp == 4) {
    if (lane == 0) {
      // ---- producer: halo tiles and weight slots, in the order the MMAs consume them
      int na[2] = {0, 0}, nb[kBSlots] = {};  // loads armed per stage / slot
      int ca = 0;                            // chunks issued
      int sb = 0, rb = 0;                    // weight slot of the next load, and its round
      bool ok = true;
      for (int tt = blockIdx.x; tt < a.n_tiles && ok; tt += gridDim.x) {
        const Tile tl = tile_of(a, tt, BN);
        for (int c = 0; c < nchunks && ok; ++c, ++ca) {
          const int sa = ca & 1;
          if (ca >= 2 && !wait_or_abort(tc::smem_addr(&S.a_empty[sa]), ((ca - 2) >> 1) & 1, abort)) {
            ok = false;
            break;
          }
          const uint32_t fa = tc::smem_addr(&S.a_full[sa]);
          tc::mbar_arrive_expect_tx(fa, kBytesA);
          ++na[sa];
          for (int r = 0; r < kInRows; ++r)
            for (int g = 0; g < kG; ++g)
              tc::tma_load_4d(tc::smem_addr(S.a[sa] + (r * kG + g) * kSlab), &tmx, c * KC + 8 * g,
                              tl.xt * kTileX - 1, tl.y + r - (NR == 3 ? 1 : 0), tl.img, fa);
          for (int tap = 0; tap < kTaps; ++tap) {
            if (rb >= 1 && !wait_or_abort(tc::smem_addr(&S.b_empty[sb]), (rb - 1) & 1, abort)) {
              ok = false;
              break;
            }
            const uint32_t fb = tc::smem_addr(&S.b_full[sb]);
            tc::mbar_arrive_expect_tx(fb, kBytesB);
            ++nb[sb];
            tc::bulk_load(tc::smem_addr(S.b[sb]),
                          a.wb + ((size_t)((tl.n0 / BN) * nchunks + c) * kTaps + tap) * kBytesB, kBytesB, fb);
            if (++sb == kBSlots) {
              sb = 0;
              ++rb;
            }
          }
        }
      }
      // every load issued has landed before the CTA may leave (bounded)
      for (int i = 0; i < 2; ++i)
        if (na[i] > 0 && !tc::mbar_wait(tc::smem_addr(&S.a_full[i]), (na[i] - 1) & 1, kWaitLimit)) *abort = 1;
      for (int i = 0; i < kBSlots; ++i)
        if (nb[i] > 0 && !tc::mbar_wait(tc::smem_addr(&S.b_full[i]), (nb[i] - 1) & 1, kWaitLimit)) *abort = 1;
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // ---- MMA issuer
      constexpr uint32_t idesc = tc::make_idesc_bf16(128, BN);
      int ca = 0, k = 0;   // chunks and tiles consumed
      int sb = 0, rb = 0;  // weight slot of the next tap, and its round
      bool ok = true;
      for (int tt = blockIdx.x; tt < a.n_tiles && ok; tt += gridDim.x, ++k) {
        const int buf = k & 1;
        if (k >= 2 && !wait_or_abort(tc::smem_addr(&S.acc_empty[buf]), ((k >> 1) - 1) & 1, abort)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t acc = tmem + (uint32_t)(buf * kRowsPerTile * BN);  // row q at + q BN
        for (int c = 0; c < nchunks && ok; ++c, ++ca) {
          const int sa = ca & 1;
          if (!wait_or_abort(tc::smem_addr(&S.a_full[sa]), (ca >> 1) & 1, abort)) {
            ok = false;
            break;
          }
          const uint64_t adesc0 = tc::make_desc(tc::smem_addr(S.a[sa]), kSlab, 128);
          for (int tap = 0; tap < kTaps; ++tap) {
            if (!wait_or_abort(tc::smem_addr(&S.b_full[sb]), rb & 1, abort)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const int dy = NR == 3 ? tap / 3 : 0, dx = NR == 3 ? tap % 3 : 1;  // halo row / column offset
            // start addresses in 16-byte units (descriptor bits 0-13); output row q reads
            // halo rows dy + q, one row group (kG slabs) further
            uint64_t ad = adesc0 + (uint64_t)(dy * kG * (kSlab / 16) + dx);
            uint64_t bd = tc::make_desc(tc::smem_addr(S.b[sb]), BN * 16, 128);
            const uint32_t first = (c == 0 && tap == 0) ? 0u : 1u;
#pragma unroll
            for (int s = 0; s < KC / 16; ++s) {
#pragma unroll
              for (int q = 0; q < kRowsPerTile; ++q)
                tc::mma_bf16(acc + (uint32_t)(q * BN), ad + (uint64_t)(q * kG * (kSlab / 16)), bd, idesc,
                             (s == 0) ? first : 1u);
              ad += 2 * kSlab / 16;
              bd += 2 * BN;
            }
            tc::mma_commit(tc::smem_addr(&S.b_empty[sb]));
            if (++sb == kBSlots) {
              sb = 0;
              ++rb;
            }
          }
          if (!ok) break;
          tc::mma_commit(tc::smem_addr(&S.a_empty[sa]));
        }
        if (!ok) break;
        tc::mma_commit(tc::smem_addr(&S.acc_full[buf]));
      }
      tc::mma_commit(tc::smem_addr(&S.done));  // arrives when every MMA issued above has completed
      if (!tc::mbar_wait(tc::smem_addr(&S.done), 0, kWaitLimit)) *abort = 1;
    }
  } else {
    // ---- epilogue warps 0-3: TMEM lanes 32 warp .. 32 warp + 31 = pixels of the tile
    int k = 0;
    for (int tt = blockIdx.x; tt < a.n_tiles; tt += gridDim.x, ++k) {
      const Tile tl = tile_of(a, tt, BN);
      const int buf = k & 1;
      if (!wait_or_abort(tc::smem_addr(&S.acc_full[buf]), (k >> 1) & 1, abort)) break;
      tc::fence_after_sync();
#pragma unroll 1
      for (int q = 0; q < kRowsPerTile; ++q) {
      float v[BN];
      {
        uint32_t reg[BN];
        if constexpr (BN >= 32) {
#pragma unroll
          for (int col = 0; col < BN; col += 32)
            tc::tmem_ld32_nowait(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)((buf * kRowsPerTile + q) * BN + col),
                                 reg + col);
          tc::tmem_wait_ld();
        }
#pragma unroll
        for (int c2 = 0; c2 < BN; ++c2) v[c2] = __uint_as_float(reg[c2]);
      }
      if (q == kRowsPerTile - 1) {  // the buffer's last TMEM read: the MMAs may refill it
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(&S.acc_empty[buf])) : "memory");
      }
      const int xw = tl.xt * kTileX + 32 * warp + lane;
      if (xw < a.W && tl.y + q < a.H) {
        const size_t p = ((size_t)tl.img * a.H + tl.y + q) * a.W + xw;
#pragma unroll
        for (int col = 0; col < BN; col += 8) {
          const int n = tl.n0 + col;
          if (n >= a.Cout) break;
          float* vv = v + col;
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            if (a.bias) vv[i] += a.bias[n + i];
            if (a.relu) vv[i] = fmaxf(vv[i], 0.f);
          }
          if (a.mask) {  // gradient through the ReLU that produced this layer's input
            const uint4 mv = *reinterpret_cast<const uint4*>(a.mask + p * a.Cout + n);
            const __nv_bfloat16* m = reinterpret_cast<const __nv_bfloat16*>(&mv);
#pragma unroll
            for (int i = 0; i < 8; ++i)
              if (!(__bfloat162float(m[i]) > 0.f)) vv[i] = 0.f;
          }
          if (a.y_fp32) {
            float* dst = reinterpret_cast<float*>(a.y) + p * a.Cout + n;
            *reinterpret_cast<float4*>(dst) = make_float4(vv[0], vv[1], vv[2], vv[3]);
            *reinterpret_cast<float4*>(dst + 4) = make_float4(vv[4], vv[5], vv[6], vv[7]);
          } else {
            __align__(16) __nv_bfloat162 h[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(vv[2 * i], vv[2 * i + 1]);
            *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.y) + p * a.Cout + n) =
                *reinterpret_cast<const uint4*>(h);
          }
        }
      }
      }
    }
  }
  __syncthreads();
  if (t == 0 && S.abort) atomicCAS(&g_nn_error, 0, 1);
  tc::fence_after_sync();
  if (warp == 5) tc::tmem_dealloc(tmem, kCols);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// BF16 tensor map of `rank` dims (innermost first) with a box; zero fill outside.
bool make_map(CUtensorMap* m, const void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides_bytes,
              const cuuint32_t* box) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), dims, strides_bytes, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Blocked weights: wb[nt][c][tap][g][n][8] = w[nt BN + n][tap][c KC + 8 g + 0..7] (zero for
// output channels past Cout), one 16-byte vector per thread.
__global__ void k_block_weights(const uint4* __restrict__ w, int Cout, int taps, int Cin, int BN, int KC,
                                uint4* __restrict__ wb, long long n_vec) {
  const int kG = KC / 8, nchunks = Cin / KC;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_vec;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    const int n = (int)(r % BN);
    r /= BN;
    const int g = (int)(r % kG);
    r /= kG;
    const int tap = (int)(r % taps);
    r /= taps;
    const int c = (int)(r % nchunks);
    const int nt = (int)(r / nchunks);
    const int co = nt * BN + n;
    wb[i] = co < Cout ? w[((long long)co * taps + tap) * (Cin / 8) + c * kG + g] : make_uint4(0, 0, 0, 0);
  }
}

// Device buffer of the blocked weights, one per device, grown on demand and kept (growing
// it synchronises the device).  Callers on several host threads or streams take turns:
// the buffer's mutex is held from the blocking kernel to the convolution's launch, and a
// new user's stream waits for the event recorded after the last convolution that read it.
struct BlockedWeights {
  unsigned char* p = nullptr;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
};
constexpr int kMaxDevices = 64;
BlockedWeights g_wb[kMaxDevices];
std::mutex g_wb_mu;

cudaError_t blocked_weights(BlockedWeights& b, const __nv_bfloat16* w, int Cout, int taps, int Cin, int BN, int KC,
                            cudaStream_t st) {
  const int n_nt = (Cout + BN - 1) / BN;
  const size_t bytes = (size_t)n_nt * BN * taps * Cin * 2;
  cudaError_t e = cudaSuccess;
  if (!b.done) {
    e = cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  if (bytes > b.bytes) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) return e;
    b.bytes = bytes;
  }
  e = cudaStreamWaitEvent(st, b.done, 0);  // the previous convolution that read the buffer
  if (e != cudaSuccess) return e;
  const long long n_vec = (long long)(bytes / 16);
  const int blocks = (int)((n_vec + 255) / 256 < 1024 ? (n_vec + 255) / 256 : 1024);
  k_block_weights<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint4*>(w), Cout, taps, Cin, BN, KC,
                                          reinterpret_cast<uint4*>(b.p), n_vec);
  return cudaGetLastError();
}

template <int BN, int KC, int NR>
cudaError_t launch_fwd(const __nv_bfloat16* x, const __nv_bfloat16* w, ConvArgs a, cudaStream_t st) {
  CUtensorMap tmx;
  const cuuint64_t xd[4] = {(cuuint64_t)a.Cin, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.B};
  const cuuint64_t xs[3] = {(cuuint64_t)a.Cin * 2, (cuuint64_t)a.W * a.Cin * 2, (cuuint64_t)a.H * a.W * a.Cin * 2};
  const cuuint32_t xb[4] = {8, kHalo, 1, 1};
  if (!make_map(&tmx, x, 4, xd, xs, xb)) return cudaErrorInvalidValue;
  if (a.taps != (NR == 3 ? 9 : 1) || a.Cin % KC != 0) return cudaErrorInvalidValue;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_wb_mu);
  BlockedWeights& bw = g_wb[dev];
  e = blocked_weights(bw, w, a.Cout, a.taps, a.Cin, BN, KC, st);
  if (e != cudaSuccess) return e;
  a.wb = bw.p;
  // CTAs per SM: shared memory, and TMEM (2 kRowsPerTile BN columns each, 512 per SM)
  constexpr int kRowsPerTile = rows_per_tile(BN);
  const size_t per_sm = 232448, need = sizeof(TSmem<BN, KC, NR>) + 1024;
  int ctas = (int)(per_sm / (need + 1024));
  ctas = ctas < 1 ? 1 : ctas;
  if (ctas * 2 * kRowsPerTile * BN > 512) ctas = 512 / (2 * kRowsPerTile * BN);
  const size_t smem = per_sm / ctas - 1024 > need ? per_sm / ctas - 1024 : need;
  e = cudaFuncSetAttribute(k_conv_fwd<BN, KC, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  a.n_ntiles = (a.Cout + BN - 1) / BN;
  a.xtiles = (a.W + kTileX - 1) / kTileX;
  const long long tiles =
      (long long)a.xtiles * ((a.H + kRowsPerTile - 1) / kRowsPerTile) * a.B * a.n_ntiles;
  if (tiles >= (1LL << 31)) return cudaErrorInvalidValue;
  a.n_tiles = (int)tiles;
  const int grid = a.n_tiles < ctas * sms ? a.n_tiles : ctas * sms;
  k_conv_fwd<BN, KC, NR><<<grid, kTileThreads, smem, st>>>(a, tmx);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaEventRecord(bw.done, st);
}

template <int KC, int NR>
cudaError_t launch_fwd_n(const __nv_bfloat16* x, const __nv_bfloat16* w, const ConvArgs& a, cudaStream_t st) {
  if (a.Cout <= 32) return launch_fwd<32, KC, NR>(x, w, a, st);
  if (a.Cout <= 64) return launch_fwd<64, KC, NR>(x, w, a, st);
  return launch_fwd<128, KC, NR>(x, w, a, st);
}

}  // namespace

int conv_fwd(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
             const float* bias, int relu, const __nv_bfloat16* mask, void* y, int y_fp32, cudaStream_t st) {
  if (!x || !w || !y || B < 1 || H < 1 || W < 1) return 1;
  if (Cin < 16 || Cin % 16 != 0 || Cout < 8 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return 1;
  if ((long long)B * H * W >= (1LL << 31)) return 1;
  // TMA: 16-byte aligned tensors (every stride is a multiple of 16 bytes: Cin % 8 == 0)
  if (((uintptr_t)x & 15) || ((uintptr_t)w & 15)) return 1;
  // wide, shallow layers: the strip-persistent kernel (resident weights, rolling input rows)
  const int rs = conv_fwd_strip(x, B, H, W, Cin, w, Cout, taps, bias, relu, mask, y, y_fp32, st);
  if (rs >= 0) return rs;
  ConvArgs a{nullptr, bias, mask, y, B, H, W, Cin, Cout, taps, relu, y_fp32, 1, 1, 1};
  cudaError_t e;
  if (taps == 9)
    e = Cin % 32 == 0 ? launch_fwd_n<32, 3>(x, w, a, st) : launch_fwd_n<16, 3>(x, w, a, st);
  else
    e = Cin % 32 == 0 ? launch_fwd_n<32, 1>(x, w, a, st) : launch_fwd_n<16, 1>(x, w, a, st);
  return e == cudaSuccess ? 0 : 2;
}

namespace {

// ---------------------------------------------------------------------------
// Weight gradient: gw[co, t, ci] += sum_p gy[p, co] x[p + d_t, ci]
// ---------------------------------------------------------------------------
// GEMM per tap with K = pixels: A[co, p] = gy[p, co], B_t[ci, p] = x[p + d_t, ci], both
// transposed while staged (K-major tiles, p along K).  A CTA owns 128 output channels x
// BN input channels x TG taps (TG x BN TMEM columns) for one range of pixels, in chunks
// of 64 pixels; the A tile of a chunk serves all TG taps.  Partial sums over the CTA's
// pixels go to the CTA's slice of a workspace (one slice per pixel split), which a second
// kernel adds to the FP32 gradient in split order: the result does not depend on the
// order in which CTAs finish (training is reproducible).
struct WgradArgs {
  const __nv_bfloat16* x;   // [B][H][W][Cin]
  const __nv_bfloat16* gy;  // [B][H][W][Cout]
  float* ws;                // [splits][Cout][taps][Cin] partial sums
  int B, H, W, Cin, Cout, taps;
  int chunks_per_cta;       // 64-pixel chunks per CTA (pixel split)
};

template <int BN, int TG>
struct WSmem {
  alignas(1024) unsigned char a[2][128 * 64 * 2];
  alignas(1024) unsigned char b[2][TG][BN * 64 * 2];
  alignas(8) unsigned long long mbar[2];
  uint32_t tmem;
};

__host__ __device__ constexpr int tmem_cols(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512; }

// Stage 8 consecutive channels of pixel p (or zeros) as column kp of rows r0 .. r0 + 7.
__device__ __forceinline__ void put_column8(unsigned char* tile, int r0, int kp, const __nv_bfloat16* src) {
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (src) v = *reinterpret_cast<const uint4*>(src);
  const unsigned short* h = reinterpret_cast<const unsigned short*>(&v);
#pragma unroll
  for (int i = 0; i < 8; ++i) *reinterpret_cast<unsigned short*>(tile + tc::tile_offset(r0 + i, kp, 64)) = h[i];
}

template <int BN, int TG>
__global__ void __launch_bounds__(kThreads) k_conv_wgrad(const WgradArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  WSmem<BN, TG>& S = *reinterpret_cast<WSmem<BN, TG>*>(smem_raw + ((1024 - ((uintptr_t)smem_raw & 1023)) & 1023));
  const int t = threadIdx.x, warp = t >> 5;
  const int m0 = blockIdx.y * 128;                    // output channels
  const int n_ctiles = (a.Cin + BN - 1) / BN;
  const int c0 = (blockIdx.z % n_ctiles) * BN;        // input channels
  const int t0 = (blockIdx.z / n_ctiles) * TG;        // first tap of the group
  const int ntap = min(TG, a.taps - t0);
  const int npix = a.B * a.H * a.W;
  const int chunk0 = blockIdx.x * a.chunks_per_cta;
  const int nchunks = max(0, min(a.chunks_per_cta, (npix + 63) / 64 - chunk0));
  constexpr int kCols = tmem_cols(TG * BN);

  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&S.tmem), kCols);
  if (t == 0) {
    tc::mbar_init(tc::smem_addr(&S.mbar[0]), 1);
    tc::mbar_init(tc::smem_addr(&S.mbar[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  constexpr uint32_t idesc = tc::make_idesc_bf16(128, BN);

  const int kp = t & 63, half = t >> 6;
  bool ok = true;
  int issued = 0;
  for (int c = 0; c < nchunks; ++c) {
    const int st = c & 1;
    if (c >= 2) ok = tc::mbar_wait(tc::smem_addr(&S.mbar[st]), ((c - 2) >> 1) & 1, kWaitLimit);
    ok = __syncthreads_and(ok);
    if (!ok) break;
    const int p = (chunk0 + c) * 64 + kp;
    int b = 0, yh = 0, xw = 0;
    if (p < npix) {
      xw = p % a.W;
      const int rest = p / a.W;
      yh = rest % a.H;
      b = rest / a.H;
    }
    // A: 128 output channels x 64 pixels
    for (int g = half; g < 16; g += 2) {
      const int co = m0 + 8 * g;
      const __nv_bfloat16* src = (p < npix && co < a.Cout) ? a.gy + (size_t)p * a.Cout + co : nullptr;
      put_column8(S.a[st], 8 * g, kp, src);
    }
    // B_t: BN input channels x 64 pixels, one tile per tap of the group
    for (int j = 0; j < TG; ++j) {
      const int tap = t0 + j;
      const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
      const int yy = yh + dy, xx = xw + dx;
      const bool in = j < ntap && p < npix && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      for (int g = half; g < BN / 8; g += 2) {
        const int ci = c0 + 8 * g;
        const __nv_bfloat16* src =
            (in && ci < a.Cin) ? a.x + (((size_t)b * a.H + yy) * a.W + xx) * a.Cin + ci : nullptr;
        put_column8(S.b[st][j], 8 * g, kp, src);
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_addr(S.a[st]);
      for (int j = 0; j < ntap; ++j) {
        const uint32_t sb = tc::smem_addr(S.b[st][j]);
#pragma unroll
        for (int s = 0; s < 4; ++s)
          tc::mma_bf16(tmem + (uint32_t)(j * BN), tc::make_desc(sa + 256 * s, 128, 64 * 16),
                       tc::make_desc(sb + 256 * s, 128, 64 * 16), idesc, (c > 0 || s > 0) ? 1u : 0u);
      }
      tc::mma_commit(tc::smem_addr(&S.mbar[st]));
    }
    issued = c + 1;
  }
  if (issued > 0) {
    const int last = issued - 1;
    bool done = tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    done = __syncthreads_and(done);
    if (!done) tc::mbar_wait(tc::smem_addr(&S.mbar[last & 1]), (last >> 1) & 1, kWaitLimit);
    ok = ok && done;
  }
  if (!ok && t == 0) atomicCAS(&g_nn_error, 0, 1);
  tc::fence_after_sync();

  if (ok && issued > 0) {
    const int co = m0 + 32 * warp + (t & 31);
    for (int j = 0; j < ntap; ++j) {
      for (int col = 0; col < BN; col += 8) {
        float v[8];
        tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(j * BN + col), v);
        const int ci = c0 + col;
        if (co < a.Cout && ci < a.Cin) {
          float* dst = a.ws + (size_t)blockIdx.x * a.Cout * a.taps * a.Cin + ((size_t)co * a.taps + t0 + j) * a.Cin + ci;
          reinterpret_cast<float4*>(dst)[0] = make_float4(v[0], v[1], v[2], v[3]);
          reinterpret_cast<float4*>(dst)[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// gw[i] += sum over splits s (in order) of ws[s][i]
__global__ void k_wgrad_reduce(const float* __restrict__ ws, int splits, long long n, float* __restrict__ gw) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += ws[(size_t)k * n + i];
    gw[i] += s;
  }
}

// Pixel split of a weight-gradient launch: about two waves of CTAs, at least 8 chunks per
// CTA so the partial sums amortise.
template <int BN, int TG>
void wgrad_split(int B, int H, int W, int Cin, int Cout, int taps, int& splits, int& chunks_per_cta) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int npix = B * H * W;
  const int chunks = (npix + 63) / 64;
  const int tiles = ((Cout + 127) / 128) * ((Cin + BN - 1) / BN) * ((taps + TG - 1) / TG);
  splits = (2 * sms + tiles - 1) / tiles;
  splits = max(1, min(splits, (chunks + 7) / 8));
  chunks_per_cta = (chunks + splits - 1) / splits;
  splits = (chunks + chunks_per_cta - 1) / chunks_per_cta;
}

template <int BN, int TG>
cudaError_t launch_wgrad(WgradArgs a, float* gw, size_t ws_floats, cudaStream_t st) {
  const size_t smem = sizeof(WSmem<BN, TG>) + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad<BN, TG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int splits = 1;
  wgrad_split<BN, TG>(a.B, a.H, a.W, a.Cin, a.Cout, a.taps, splits, a.chunks_per_cta);
  const long long n = (long long)a.Cout * a.taps * a.Cin;
  if ((size_t)splits * (size_t)n > ws_floats) return cudaErrorInvalidValue;
  dim3 grid(splits, (a.Cout + 127) / 128, ((a.Cin + BN - 1) / BN) * ((a.taps + TG - 1) / TG));
  k_conv_wgrad<BN, TG><<<grid, kThreads, smem, st>>>(a);
  const long long blocks = (n + 255) / 256;
  k_wgrad_reduce<<<(int)(blocks < 1024 ? blocks : 1024), 256, 0, st>>>(a.ws, splits, n, gw);
  return cudaGetLastError();
}

template <int BN, int TG>
size_t wgrad_ws(int B, int H, int W, int Cin, int Cout, int taps) {
  int splits = 1, cpc = 1;
  wgrad_split<BN, TG>(B, H, W, Cin, Cout, taps, splits, cpc);
  return (size_t)splits * Cout * taps * Cin;
}

// wt[ci][8 - t][co] = w[co][t][ci] (taps 9) or wt[ci][0][co] = w[co][0][ci]: the weights
// of the input gradient as a forward convolution of the output gradient.
__global__ void k_flip_transpose(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt, int Cout,
                                 int taps, int Cin) {
  const int n = Cout * taps * Cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ci = i % Cin;
    const int rest = i / Cin;
    const int tp = rest % taps, co = rest / taps;
    wt[((size_t)ci * taps + (taps - 1 - tp)) * Cout + co] = w[i];
  }
}

}  // namespace

bool wgrad_args_ok(int B, int H, int W, int Cin, int Cout, int taps) {
  if (B < 1 || H < 1 || W < 1) return false;
  if (Cin < 8 || Cin % 8 != 0 || Cout < 8 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return false;
  return (long long)B * H * W < (1LL << 31);
}

size_t conv_wgrad_workspace(int B, int H, int W, int Cin, int Cout, int taps) {
  if (!wgrad_args_ok(B, H, W, Cin, Cout, taps)) return 0;
  if (taps == 1)
    return Cin <= 32 ? wgrad_ws<32, 1>(B, H, W, Cin, Cout, taps)
                     : Cin <= 64 ? wgrad_ws<64, 1>(B, H, W, Cin, Cout, taps) : wgrad_ws<128, 1>(B, H, W, Cin, Cout, taps);
  return Cin <= 32 ? wgrad_ws<32, 9>(B, H, W, Cin, Cout, taps)
                   : Cin <= 64 ? wgrad_ws<64, 3>(B, H, W, Cin, Cout, taps) : wgrad_ws<128, 3>(B, H, W, Cin, Cout, taps);
}

int conv_wgrad(const __nv_bfloat16* x, const __nv_bfloat16* gy, int B, int H, int W, int Cin, int Cout, int taps,
               float* gw, float* ws, size_t ws_floats, cudaStream_t st) {
  if (!x || !gy || !gw || !ws || !wgrad_args_ok(B, H, W, Cin, Cout, taps)) return 1;
  if (ws_floats < conv_wgrad_workspace(B, H, W, Cin, Cout, taps)) return 1;
  WgradArgs a{x, gy, ws, B, H, W, Cin, Cout, taps, 1};
  cudaError_t e;
  if (taps == 1)
    e = Cin <= 32 ? launch_wgrad<32, 1>(a, gw, ws_floats, st)
                  : Cin <= 64 ? launch_wgrad<64, 1>(a, gw, ws_floats, st) : launch_wgrad<128, 1>(a, gw, ws_floats, st);
  else
    e = Cin <= 32 ? launch_wgrad<32, 9>(a, gw, ws_floats, st)
                  : Cin <= 64 ? launch_wgrad<64, 3>(a, gw, ws_floats, st) : launch_wgrad<128, 3>(a, gw, ws_floats, st);
  return e == cudaSuccess ? 0 : 2;
}

int flip_transpose(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int taps, int Cin, cudaStream_t st) {
  if (!w || !wt || Cout < 1 || Cin < 1 || (taps != 1 && taps != 9)) return 1;
  const int n = Cout * taps * Cin;
  k_flip_transpose<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(w, wt, Cout, taps, Cin);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int take_error() {
  int v = 0, zero = 0;
  cudaDeviceSynchronize();
  cudaMemcpyFromSymbol(&v, g_nn_error, sizeof v);
  cudaMemcpyToSymbol(g_nn_error, &zero, sizeof zero);
  return v;
}

}  // namespace nn
}  // namespace stem

// the strip-persistent forward convolution (uses g_nn_error and make_map above)
#include "nn_conv_strip.cuh"
