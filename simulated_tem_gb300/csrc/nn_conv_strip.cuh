// Strip-persistent convolution for the corrector's wide, shallow layers (Cout <= 64,
// Cin <= 64: the full- and half-resolution levels of the U-Net).  A 96-channel input
// (dec0a) holds 231 KB here, one CTA per SM, and measured 6 % faster on the halo-tile
// kernel (two-row tiles, two CTAs per SM), which takes every wider input.
//
// A CTA walks down a band of image rows in one 128-pixel column strip, RP output rows per
// step.  Its weights (all taps, all input channels, BN <= 64 output channels) are loaded
// once by TMA and stay in shared memory.  Input rows live in a ring of 2 RP + 2 row slots,
// each holding all Cin channels of pixels x0 - 1 .. x0 + 128 as (Cin / 8) slabs of 130
// rows x 16 bytes: output rows y .. y + RP - 1 read input rows y - 1 .. y + RP from the
// ring, and the next step's RP new rows load meanwhile.  The nine taps read the slabs
// through descriptors shifted by 16 bytes per pixel (rows 16 bytes apart), as in the
// halo-tile kernel, and TMA zero-fills outside the image.
//
// With N = BN <= 64 one MMA is little work, and MMAs that accumulate into the same TMEM
// columns run one after another: the RP rows of a step have their own accumulators and
// their MMAs are interleaved, so consecutive MMAs are independent.
//
// Warp roles (224 threads): warp 4 lane 0 loads (TMA); warps 5 and 6, lane 0 each, issue
// the MMAs of the step's rows r = 0 and 1 (a thread waits tens of cycles per MMA it
// issues, and an N = 32 MMA takes less than that on the tensor pipe: two issuers keep it
// busy); warps 0-3 drain TMEM (warp w reads lanes 32w .. 32w + 31).  The issue loops add
// precomputed offsets to precomputed descriptors.  Two sets of accumulators: the epilogue
// of one step overlaps the MMAs of the next.  mbarriers: weights full; row slot full (TMA
// bytes) / empty (both issuers' commits after the last step that reads it); accumulators
// full (both issuers' commits) / empty (one arrival per epilogue warp).
//
// Every wait is bounded (about a second) and watches a shared abort flag, so a role that
// gives up stops the others quickly; the kernel then records an error in g_nn_error,
// waits (bounded) for its own loads and MMAs, and frees TMEM.
//
// Included by nn_conv.cu (one translation unit: the kernels share g_nn_error and the
// tensor-map helpers).
#pragma once

namespace stem {
namespace nn {
namespace strip {

constexpr int kThreads = 224;
constexpr int kIssuers = 2;  // MMA-issuing warps (5, 6); RP is a multiple of kIssuers
constexpr int kRingMax = 16;  // input row slots at most

struct StripArgs {
  const float* bias;
  const __nv_bfloat16* mask;
  void* y;
  int B, H, W, Cin, Cout, relu, y_fp32;
  int xtiles, bands, rows_per_band, n_strips;  // rows_per_band a multiple of RP
  int ring;                                    // input row slots
};

struct Bars {
  unsigned long long w_full, row_full[kRingMax], row_empty[kRingMax], acc_full[2], acc_empty[2], done;
  uint32_t tmem;
  int abort;
};

// bounded wait that gives up early when another role has aborted
__device__ __forceinline__ bool wait_bar(uint32_t mbar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    if (tc::mbar_try_wait(mbar, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// A strip's rows: output rows [y0, y1) of image img, column tile xt.
struct Strip {
  int xt, img, y0, y1;
};
__device__ __forceinline__ Strip strip_of(const StripArgs& a, int s) {
  Strip r;
  r.xt = s % a.xtiles;
  const int rest = s / a.xtiles;
  const int band = rest % a.bands;
  r.img = rest / a.bands;
  r.y0 = band * a.rows_per_band;
  r.y1 = min(a.H, r.y0 + a.rows_per_band);
  return r;
}

// NR = 3 (3 x 3 convolution) or 1 (1 x 1); RP output rows per step
template <int BN, int NR, int RP>
__global__ void __launch_bounds__(kThreads) k_conv_strip(const StripArgs a, const __grid_constant__ CUtensorMap tmx,
                                                         const __grid_constant__ CUtensorMap tmw) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - ((uintptr_t)smem_raw & 1023)) & 1023);
  static_assert(RP % kIssuers == 0, "rows per step shared by the issuers");
  constexpr int kTaps = NR == 3 ? 9 : 1;
  constexpr uint32_t kCols = 2 * RP * BN;  // two sets of RP accumulators
  const int G = a.Cin / 8;
  const int wbytes = kTaps * G * BN * 16;
  unsigned char* wsm = base;                               // [tap][g][BN][16 B]
  unsigned char* ring = base + ((wbytes + 1023) & ~1023);  // [slot][g][kSlab]
  const int R = a.ring;
  Bars& S = *reinterpret_cast<Bars*>(ring + R * G * kSlab);
  volatile int* abort = &S.abort;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  if (warp == 5) tc::tmem_alloc(tc::smem_addr(&S.tmem), kCols);
  if (t == 0) {
    tc::mbar_init(tc::smem_addr(&S.w_full), 1);
    for (int i = 0; i < R; ++i) {
      tc::mbar_init(tc::smem_addr(&S.row_full[i]), 1);
      tc::mbar_init(tc::smem_addr(&S.row_empty[i]), kIssuers);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(tc::smem_addr(&S.acc_full[i]), kIssuers);
      tc::mbar_init(tc::smem_addr(&S.acc_empty[i]), 4);
    }
    tc::mbar_init(tc::smem_addr(&S.done), kIssuers);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;

  if (warp == 4) {
    if (lane == 0) {
      // ---- producer: the weights once, then the strips' input rows in order
      const uint32_t wf = tc::smem_addr(&S.w_full);
      tc::mbar_arrive_expect_tx(wf, (uint32_t)wbytes);
      for (int tap = 0; tap < kTaps; ++tap)
        for (int g = 0; g < G; ++g)
          tc::tma_load_3d(tc::smem_addr(wsm + (tap * G + g) * BN * 16), &tmw, 8 * g, tap, 0, wf);
      int armed[kRingMax];
      for (int i = 0; i < kRingMax; ++i) armed[i] = 0;
      int li = 0;  // input rows loaded by this CTA (ring position)
      bool ok = true;
      for (int s = blockIdx.x; s < a.n_strips && ok; s += gridDim.x) {
        const Strip sp = strip_of(a, s);
        const int nsteps = (sp.y1 - sp.y0 + RP - 1) / RP;
        const int nin = nsteps * RP + NR - 1;
        for (int i = 0; i < nin; ++i, ++li) {
          const int slot = li % R;
          if (li >= R && !wait_bar(tc::smem_addr(&S.row_empty[slot]), (li / R - 1) & 1, abort)) {
            ok = false;
            break;
          }
          const uint32_t rf = tc::smem_addr(&S.row_full[slot]);
          tc::mbar_arrive_expect_tx(rf, (uint32_t)(G * kHalo * 16));
          ++armed[slot];
          const int yin = sp.y0 - (NR == 3 ? 1 : 0) + i;
          for (int g = 0; g < G; ++g)
            tc::tma_load_4d(tc::smem_addr(ring + (slot * G + g) * kSlab), &tmx, 8 * g, sp.xt * kTileX - 1, yin,
                            sp.img, rf);
        }
      }
      // every load issued has landed before the CTA may leave
      if (!tc::mbar_wait(wf, 0, kWaitLimit)) *abort = 1;
      for (int i = 0; i < R; ++i)
        if (armed[i] > 0 && !tc::mbar_wait(tc::smem_addr(&S.row_full[i]), (armed[i] - 1) & 1, kWaitLimit)) *abort = 1;
    }
  } else if (warp == 5 || warp == 6) {
    if (lane == 0) {
      // ---- MMA issuers: warp 5 + i issues rows r = i, i + kIssuers, ... of every step
      const int ri = warp - 5;
      constexpr uint32_t idesc = tc::make_idesc_bf16(128, BN);
      bool ok = wait_bar(tc::smem_addr(&S.w_full), 0, abort);
      tc::fence_after_sync();
      const uint32_t rb = tc::smem_addr(ring);
      const uint32_t row_bytes = (uint32_t)(G * kSlab);
      // descriptor of the weights of tap 0, chunk 0; per tap and per 16 channels the start
      // address (field bits 0-13, bytes / 16) moves by a fixed amount
      const uint64_t wdesc0 = tc::make_desc(tc::smem_addr(wsm), BN * 16, 128);
      const uint32_t wstep_tap = (uint32_t)(G * BN), wstep_k = (uint32_t)(2 * BN);  // in 16-byte units
      const uint32_t astep_k = (uint32_t)(2 * kSlab / 16);
      int li = 0;  // ring position of the strip's first input row
      int k = 0;   // steps issued by this CTA (accumulator set sequence)
      for (int s = blockIdx.x; s < a.n_strips && ok; s += gridDim.x) {
        const Strip sp = strip_of(a, s);
        const int nsteps = (sp.y1 - sp.y0 + RP - 1) / RP;
        for (int j = 0; j < nsteps && ok; ++j, ++k) {
          // input rows j RP .. j RP + RP + NR - 2 of the strip; the first step waits for all,
          // later ones for their RP new rows
          for (int d = (j == 0 ? 0 : NR - 1); d < RP + NR - 1; ++d) {
            const int q = li + j * RP + d;
            if (!wait_bar(tc::smem_addr(&S.row_full[q % R]), (q / R) & 1, abort)) {
              ok = false;
              break;
            }
          }
          const int buf = k & 1;
          if (ok && k >= 2 && !wait_bar(tc::smem_addr(&S.acc_empty[buf]), ((k >> 1) - 1) & 1, abort)) ok = false;
          if (!ok) break;
          tc::fence_after_sync();
          uint64_t rowdesc[RP + NR - 1];
#pragma unroll
          for (int d = 0; d < RP + NR - 1; ++d)
            rowdesc[d] = tc::make_desc(rb + (uint32_t)((li + j * RP + d) % R) * row_bytes, kSlab, 128);
#pragma unroll
          for (int r = ri; r < RP; r += kIssuers) {
            const uint32_t acc = tmem + (uint32_t)((buf * RP + r) * BN);
#pragma unroll
            for (int tap = 0; tap < kTaps; ++tap) {
              const int dy = NR == 3 ? tap / 3 : 0, dx = NR == 3 ? tap % 3 : 1;
              uint64_t ad = rowdesc[r + dy] + (uint64_t)dx;  // dx pixels = dx x 16 bytes
              uint64_t bd = wdesc0 + (uint64_t)(tap * wstep_tap);
              for (int s2 = 0; s2 < G / 2; ++s2) {
                tc::mma_bf16(acc, ad, bd, idesc, (tap == 0 && s2 == 0) ? 0u : 1u);
                ad += astep_k;
                bd += wstep_k;
              }
            }
          }
          tc::mma_commit(tc::smem_addr(&S.acc_full[buf]));
          // input rows j RP .. j RP + RP - 1 are read by no later step of this strip
#pragma unroll
          for (int r = 0; r < RP; ++r) tc::mma_commit(tc::smem_addr(&S.row_empty[(li + j * RP + r) % R]));
        }
        if (!ok) break;
        // the strip's last NR - 1 input rows
        for (int d = 0; d < NR - 1; ++d) tc::mma_commit(tc::smem_addr(&S.row_empty[(li + nsteps * RP + d) % R]));
        li += nsteps * RP + NR - 1;
      }
      tc::mma_commit(tc::smem_addr(&S.done));
      if (!tc::mbar_wait(tc::smem_addr(&S.done), 0, kWaitLimit)) *abort = 1;
    }
  } else {
    // ---- epilogue warps 0-3: TMEM lanes 32 warp .. 32 warp + 31 = pixels of the rows
    float bias[BN];
#pragma unroll
    for (int c = 0; c < BN; ++c) bias[c] = (a.bias && c < a.Cout) ? a.bias[c] : 0.f;
    int k = 0;
    bool ok = true;
    for (int s = blockIdx.x; s < a.n_strips && ok; s += gridDim.x) {
      const Strip sp = strip_of(a, s);
      const int nsteps = (sp.y1 - sp.y0 + RP - 1) / RP;
      const int xw = sp.xt * kTileX + 32 * warp + lane;
      for (int j = 0; j < nsteps; ++j, ++k) {
        const int buf = k & 1;
        if (!wait_bar(tc::smem_addr(&S.acc_full[buf]), (k >> 1) & 1, abort)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        for (int r = 0; r < RP; ++r) {
          float v[BN];
          {
            uint32_t reg[BN];
#pragma unroll
            for (int col = 0; col < BN; col += 32)
              tc::tmem_ld32_nowait(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)((buf * RP + r) * BN + col),
                                   reg + col);
            tc::tmem_wait_ld();
#pragma unroll
            for (int c = 0; c < BN; ++c) v[c] = __uint_as_float(reg[c]);
          }
          if (r == RP - 1) {  // the step's accumulators are free for the MMAs of step k + 2
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(tc::smem_addr(&S.acc_empty[buf]));
          }
          const int yy = sp.y0 + j * RP + r;
          if (xw < a.W && yy < sp.y1) {
            const size_t p = ((size_t)sp.img * a.H + yy) * a.W + xw;
#pragma unroll
            for (int col = 0; col < BN; col += 8) {
              const int n = col;
              if (n >= a.Cout) break;
              float* vv = v + col;
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                vv[i] += bias[n + i];
                if (a.relu) vv[i] = fmaxf(vv[i], 0.f);
              }
              if (a.mask) {
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
    (void)ok;
  }
  __syncthreads();
  if (t == 0 && S.abort) atomicCAS(&g_nn_error, 0, 1);
  tc::fence_after_sync();
  if (warp == 5) tc::tmem_dealloc(tmem, kCols);
}

template <int BN, int NR>
size_t strip_smem(int Cin, int ring) {
  const int G = Cin / 8;
  const size_t w = ((size_t)(NR == 3 ? 9 : 1) * G * BN * 16 + 1023) & ~(size_t)1023;
  return 1024 + w + (size_t)ring * G * kSlab + sizeof(Bars);
}

template <int BN, int NR, int RP>
int launch_strip(const __nv_bfloat16* x, const __nv_bfloat16* w, StripArgs a, cudaStream_t st) {
  const size_t per_sm = 232448;
  const int ring = 2 * RP + 2;  // RP + NR - 1 rows in use, RP loading
  const size_t need = strip_smem<BN, NR>(a.Cin, ring);
  if (need > per_sm - 1024) return -1;  // does not fit: the caller takes the halo-tile kernel
  a.ring = ring;
  CUtensorMap tmx, tmw;
  const int taps = NR == 3 ? 9 : 1;
  const cuuint64_t xd[4] = {(cuuint64_t)a.Cin, (cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.B};
  const cuuint64_t xs[3] = {(cuuint64_t)a.Cin * 2, (cuuint64_t)a.W * a.Cin * 2, (cuuint64_t)a.H * a.W * a.Cin * 2};
  const cuuint32_t xb[4] = {8, kHalo, 1, 1};
  const cuuint64_t wd[3] = {(cuuint64_t)a.Cin, (cuuint64_t)taps, (cuuint64_t)a.Cout};
  const cuuint64_t wsd[2] = {(cuuint64_t)a.Cin * 2, (cuuint64_t)taps * a.Cin * 2};
  const cuuint32_t wbx[3] = {8, 1, (cuuint32_t)BN};
  if (!make_map(&tmx, x, 4, xd, xs, xb) || !make_map(&tmw, w, 3, wd, wsd, wbx)) return 2;
  // CTAs per SM: shared memory, and TMEM (2 RP BN columns each, 512 per SM)
  int ctas = (int)(per_sm / (need + 1024));
  ctas = ctas < 1 ? 1 : ctas;
  if (ctas * 2 * RP * BN > 512) ctas = 512 / (2 * RP * BN);
  const size_t smem = per_sm / ctas - 1024 > need ? per_sm / ctas - 1024 : need;
  if (cudaFuncSetAttribute(k_conv_strip<BN, NR, RP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 2;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  a.xtiles = (a.W + kTileX - 1) / kTileX;
  const int slots = ctas * sms;
  int bands = (slots + a.xtiles * a.B - 1) / (a.xtiles * a.B);
  bands = bands < 1 ? 1 : bands > a.H ? a.H : bands;
  a.rows_per_band = ((a.H + bands - 1) / bands + RP - 1) / RP * RP;
  a.bands = (a.H + a.rows_per_band - 1) / a.rows_per_band;
  a.n_strips = a.xtiles * a.bands * a.B;
  const int grid = a.n_strips < slots ? a.n_strips : slots;
  k_conv_strip<BN, NR, RP><<<grid, kThreads, smem, st>>>(a, tmx, tmw);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace strip

int conv_fwd_strip(const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w, int Cout, int taps,
                   const float* bias, int relu, const __nv_bfloat16* mask, void* y, int y_fp32, cudaStream_t st) {
  if (Cout > 64 || Cin > 64 || Cin % 16 != 0 || Cout % 8 != 0 || (taps != 1 && taps != 9)) return -1;
  strip::StripArgs a{bias, mask, y, B, H, W, Cin, Cout, relu, y_fp32, 0, 0, 0, 0, 0};
  using namespace strip;
  // two rows per step (four measured no faster: fewer CTAs fit)
  if (taps == 9) return Cout <= 32 ? launch_strip<32, 3, 2>(x, w, a, st) : launch_strip<64, 3, 2>(x, w, a, st);
  return Cout <= 32 ? launch_strip<32, 1, 2>(x, w, a, st) : launch_strip<64, 1, 2>(x, w, a, st);
}

}  // namespace nn
}  // namespace stem
