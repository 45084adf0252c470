// Time-domain lag-GEMM form of the pair reduction, on the 5th-generation
// tensor cores (tcgen05.mma, TMEM accumulators, TMA-fed operands).
//
// For a short lag window (|d| <= shift, shift <= 256) the series
//   c_ij(d) = sum_k x_i[k] x_j[k-d]
// of a block of 128 events i against one event j is a GEMM:
//   D[i, n] = sum_k A[i, k] B_j[n, k],   A = events, B_j[n, k] = x_j[k - d(n)].
// With the lag order reversed inside a tile (n = shift - d), B_j is a Hankel
// matrix, B_j[n, k] = x_j[k + n - shift], so its 8x8 "core matrices" depend
// only on (row group + column group): core(g, h) = E_(g+h).  In the
// tensor core's no-swizzle K-major layout that is a descriptor with both the
// K-direction and the N-direction core-matrix strides equal to 128 bytes over
// a strip of (W + L)/8 distinct core matrices -- about 20 KB per event for
// the whole K range, built once per j in shared memory.
//
// Two forms (the kernel is instantiated per plane count NHL):
//  * FP32 accuracy from BF16 inputs: x = hi + lo with hi = bf16(x),
//    lo = bf16(x - hi); each lag product is hi_i hi_j + hi_i lo_j + lo_i hi_j
//    (three MMAs into the same FP32 accumulator; lo*lo ~ 2^-16 relative is
//    dropped);
//  * one FP16 plane of the samples scaled by 1/norm, one MMA per product.
// Norms and the final normalisation are FP64, as in the FFT form.  A second
// mode (RECT) correlates query events with catalog columns for the server.
//
// Work: persistent CTAs (one per SM: 512 TMEM columns and ~200 KB of shared
// memory each) walk items (I-block of 128 events, chunk of `jc` events j >=
// block start); j's are processed `jp` at a time (a "pass": jp accumulators
// of nt * wt columns).  The stages overlap: the Hankel strips are double
// buffered per (pass, channel) and TMEM holds two passes' accumulators when
// 2 jp wpad <= 512, so the strips of the next j are built and the previous
// pass's accumulators are reduced while the tensor cores run.  Warp roles:
//   warps 0-3  build the Hankel strips of the next (pass, channel);
//   warp 4     TMA producer of the A tiles (128 events x 64 samples per
//              plane, 128-byte swizzle) into a `stages`-deep ring;
//   warp 5     TMEM allocation and the MMA issue: the warp runs converged and
//              an elected lane issues the MMAs of a group of K-chunks, chunk
//              by chunk at each 16-sample K offset;
//   warps 6-9  epilogue: read TMEM (one lane quarter each, lane = event i),
//              reduce max/min + lags, write outputs.
// All mbarrier waits are bounded; a wait that runs out raises the shared
// abort flag and the device error flag, every role then unwinds, the CTA
// frees its TMEM and exits.
//
// Replaces the FFT-based inverseFFT/scan of Correlation_in_OMP/correlation_c.cpp:58-137
// for windows short enough that the direct lag sum is cheaper on tensor cores.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <climits>
#include <cstdio>
#include <cstdlib>

#include "../../include/seismic_gb300.h"
#include "energy.cuh"
#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma_host.cuh"

namespace seismic {

using tc::smem_u32;

constexpr int kLagM = 128;       // events per I-block (MMA M)
constexpr int kLagKC = 64;       // samples per A tile (one 128-byte swizzle row)
constexpr int kLagThreads = 320; // 10 warps
constexpr int kLagHistMax = 1024;
constexpr int kLagGroupMax = 4;  // K-chunks whose MMAs interleave

// ------------------------------------------------------------------ prep
// One warp per (event, channel) row: FP64 norm, then the hi/lo split of the
// (optionally 1/norm-scaled) samples into channel-major [C][N][Lp] arrays of
// 16-bit values: BF16 hi and lo (the three-product form), or FP16 hi only
// (the one-product form; xlo null).
template <bool F16>
__global__ void lag_prep_kernel(const float *__restrict__ ev, long long n, int C, int L, long long ev_stride,
                                long long ch_stride, int lp, int prescale, unsigned short *__restrict__ xhi,
                                unsigned short *__restrict__ xlo, double *__restrict__ norms) {
  const long long row = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n * C) return;
  const long long e = row / C;
  const int c = (int)(row % C);
  const float *src = ev + e * ev_stride + (long long)c * ch_stride;
  // energy as exact float-pair sums of power-of-two-scaled samples, FP64
  // only across the warp (energy.cuh)
  float m = 0.f;
  for (int k = lane; k < L; k += 32) m = fmaxf(m, fabsf(src[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int xe = energy_exponent(m);
  const EnergyScale sc(xe);
  float hi = 0.f, lo = 0.f;
  for (int k = lane; k < L; k += 32) add_square(sc(src[k]), hi, lo);
  double s = (double)hi + (double)lo;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const double nrm = sqrt(ldexp(s, 2 * xe));
  const float scale = prescale ? (nrm > 0.0 ? (float)(1.0 / nrm) : 0.f) : 1.f;
  unsigned short *dh = xhi + ((long long)c * n + e) * lp;
  unsigned short *dl = xlo ? xlo + ((long long)c * n + e) * lp : nullptr;
  for (int k = lane; k < lp; k += 32) {
    const float v = k < L ? src[k] * scale : 0.f;
    if constexpr (F16) {
      dh[k] = __half_as_ushort(__float2half_rn(v));
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      dh[k] = __bfloat16_as_ushort(h);
      dl[k] = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(h)));
    }
  }
  if (lane == 0) {
    norms[row] = nrm;
    inverse_norms_of(norms, n * C)[row] = split_double(nrm > 0.0 ? 1.0 / nrm : 0.0);
  }
}

// ------------------------------------------------------------------ main
struct LagArgs {
  const unsigned short *xhi, *xlo;  // A side [C][N][Lp] 16-bit (xlo unused with one product)
  const double *norms;              // [N*C], event-major
  long long n;
  // Rectangle mode (rect != 0): A = catalog events col_begin .. col_begin +
  // n_cols - 1 of the xhi/xlo arrays (n = catalog size), strips from the
  // query arrays qhi/qlo [C][n_query][Lp]; pair (query q, catalog e) at
  // outputs[q * n_cols + e - col_begin].  Triangle mode: strips from xhi/xlo.
  int rect;
  const unsigned short *qhi, *qlo;
  const double *q_norms;
  long long n_query, col_begin, n_cols;
  int C, L, lp;
  int shift;      // lags d = 1-shift .. shift
  int wpad;       // 2*shift rounded up to a multiple of 16*nt
  int nt, wt;     // N-tiles per j and their width (wt * nt == wpad)
  int jp;         // j's per pass (TMEM: nbuf * jp * wpad <= 512 columns)
  int nbuf;       // TMEM accumulator buffers (2 when they fit, else 1)
  int jc;         // j's per work item (multiple of jp)
  int nm;         // core matrices per Hankel strip = wpad/8 + lp/8 - 1
  int strip_bytes;
  int xs_len;     // staged x_j length (elements)
  int stages;
  int prescaled;
  float threshold;
  int n_hist;
  float delta_hist;
  float *vals_pos;
  int *lags_pos;
  float *vals_neg;
  int *lags_neg;
  int *max_hist, *min_hist;
  int *error_flag;
  int off_a, off_hank, off_xs, off_hist, off_bars, off_misc;  // shared-memory layout (host computed)
  // 16-bit planes per operand: 2 (BF16 hi, lo; products hi*hi + hi*lo +
  // lo*hi) or 1 (FP16 hi; hi*hi); the kernel is instantiated per value
  int nhl;
  int kgroup;     // K-chunks per MMA group (1 .. kLagGroupMax, at most stages / 2)
  long long blk_begin, blk_end;  // triangle: the 128-event blocks this launch walks
  unsigned wait_limit;  // polls of each bounded wait (0: kLagWaitPolls); SEISMIC_DEVICE_WAIT_POLLS
  int wait_probe;       // the TMA warp's first wait is on a barrier nothing completes (SEISMIC_DEVICE_WAIT_PROBE)
};

struct LagSmem {  // offsets into dynamic shared memory (base 1024-aligned)
  int a, hank, xs, hist, bars, misc, total;
};

static LagSmem lag_smem_layout(const LagArgs &a) {
  LagSmem s;
  int off = 0;
  s.a = off;
  off += a.stages * a.nhl * kLagM * kLagKC * 2;  // hi (+ lo) tiles per stage
  s.hank = off;
  off += 2 * a.jp * a.nhl * a.strip_bytes;  // two buffers of jp (hi [, lo]) strips
  s.xs = off;
  off += a.jp * a.nhl * ((a.xs_len * 2 + 15) / 16 * 16);
  s.hist = off;
  off += (a.n_hist > 0 && a.n_hist <= kLagHistMax) ? 2 * a.n_hist * 4 : 0;
  off = (off + 7) / 8 * 8;
  s.bars = off;
  off += (2 * a.stages + 9) * 8;
  s.misc = off;
  off += 24;  // TMEM address, abort flag, wait limit, the probe mbarrier (+16)
  s.total = off + 1024;  // room to align the base
  return s;
}

// Default poll limit of the lag-GEMM's waits (with back-off: about 2 s).
constexpr uint32_t kLagWaitPolls = 1u << 22;

// Bounded wait.  The CTA's poll limit (LagArgs::wait_limit, or the default)
// is the shared word right after its abort flag, read only when the barrier
// is not complete at the first poll (the MMA warp's waits sit on its issue
// path).
__device__ __forceinline__ bool lag_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err) {
  if (tc::mbar_try_wait(bar, parity)) return true;
  const uint32_t limit = reinterpret_cast<const volatile uint32_t *>(abort_flag)[1];
  for (uint32_t it = 0; it < limit; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (it > 64) __nanosleep(it > 4096 ? 512 : 32);
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return false;
}

// The same wait, answered alike on all 32 lanes of the calling warp (every
// lane must call it): a warp whose lanes took different exits would leave
// some lanes at a warp-synchronous instruction (tcgen05.ld, elect.sync,
// __syncwarp) that the others never reach.
__device__ __forceinline__ bool lag_wait_warp(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err) {
  const bool ok = lag_wait(bar, parity, abort_flag, err);
  return __all_sync(0xffffffffu, ok);
}

// AND of `ok` over the 128 strip-builder threads; also their barrier 1.
__device__ __forceinline__ bool builders_all(bool ok) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, 1, 128, pi;\n"
      " selp.u32 %0, 1, 0, po;\n}"
      : "=r"(r)
      : "r"((uint32_t)ok)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ int hist_bin_lag(float v, float delta, int n_hist) {
  if (v >= 1.0f) return n_hist - 1;
  int b = (int)(v / delta);
  return b > n_hist - 1 ? n_hist - 1 : (b < 0 ? 0 : b);
}

// Column n of a pass is lag shift - n (triangle: n increasing = lag
// decreasing, so among equal values the largest n is the first occurrence,
// the smallest lag) or lag n - (shift - 1) (rectangle: the smallest n).
// One scan chain over 16 columns n0 .. n0 + 15 (CHECK: only n < nvalid).
template <bool RECT, bool CHECK>
__device__ __forceinline__ void lag_scan16(const uint32_t (&r)[16], int n0, int nvalid, float &best, int &bn,
                                           float &worst, int &wn) {
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int n = n0 + k;
    const float v = __uint_as_float(r[k]);
    if (!CHECK || n < nvalid) {
      if (RECT ? v > best : v >= best) { best = v; bn = n; }
      if (RECT ? v < worst : v <= worst) { worst = v; wn = n; }
    }
  }
}
// Merge of two chains: does (v, n) win over (w, m)?  Larger (max) or
// smaller (min) value; on equal values the first occurrence.
template <bool RECT>
__device__ __forceinline__ bool lag_better(float v, int n, float w, int m, bool max) {
  if (max ? v > w : v < w) return true;
  return v == w && (RECT ? n < m : n > m);
}

// The MMAs of a group of G K-chunks (A tiles at descriptors dat[t], Hankel
// strips from dbg + t chunks): for each 16-sample K offset, the chunks' MMAs
// back to back for each of NC (j, N-tile) accumulators.  An MMA that opens a
// new K offset costs several times one that follows at the same offset with
// another B operand, so this order is much faster than chunk after chunk.
template <int NHL, int G, int NC>
__device__ __forceinline__ void lag_mma_group(const uint32_t (&dcol)[2], const uint32_t (&boff)[2],
                                              const uint64_t (&dat)[G], uint64_t dbg, uint32_t strip_u,
                                              uint32_t idesc, uint32_t acc_first) {
  constexpr uint32_t tile_u = kLagM * kLagKC * 2 / 16;
#pragma unroll
  for (int ks = 0; ks < kLagKC / 16; ++ks) {
#pragma unroll
    for (int t = 0; t < G; ++t) {
      const uint64_t dah = dat[t] + (uint64_t)(2 * ks);  // 32 bytes of K per step
      const uint64_t dbk = dbg + (uint64_t)((t * (kLagKC / 8) + 2 * ks) * 8);  // k core matrix
#pragma unroll
      for (int cb = 0; cb < NC; ++cb) {
        const uint64_t dbh = dbk + boff[cb];
        tc::mma_f16_elect(dcol[cb], dah, dbh, idesc, (ks | t) == 0 ? acc_first : 1u);
        if constexpr (NHL == 2) {  // hi*lo + lo*hi
          tc::mma_f16_elect(dcol[cb], dah, dbh + strip_u, idesc, 1u);
          tc::mma_f16_elect(dcol[cb], dah + tile_u, dbh, idesc, 1u);
        }
      }
    }
  }
}

// Items: row-block b (events [128b, 128b+128)) x chunk q of j's starting at
// 128b, each chunk `jc` events.  Advance (b, q) by `step` items.
// Rectangle mode: every block has the same n_query j's (pass n_rect = n_query).
__device__ __forceinline__ void advance_item(long long &b, long long &q, long long step, long long n, int jc,
                                             long long nblk, long long n_rect = 0) {
  while (step > 0 && b < nblk) {
    const long long rows_j = n_rect > 0 ? n_rect : n - b * kLagM;
    const long long chunks = (rows_j + jc - 1) / jc;
    const long long left = chunks - q;
    if (step < left) {
      q += step;
      return;
    }
    step -= left;
    ++b;
    q = 0;
  }
}

// NHL: 16-bit planes per operand (2: BF16 hi + lo, three products; 1: FP16
// hi, one product).  RECT: query x catalog rectangle instead of the triangle.
template <int NHL, bool RECT>
__global__ void __launch_bounds__(kLagThreads, 1)
    lag_gemm_kernel(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
                    LagArgs a) {
  constexpr int nhl = NHL;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  struct {
    int a, hank, xs, hist, bars, misc;
  } L = {a.off_a, a.off_hank, a.off_xs, a.off_hist, a.off_bars, a.off_misc};
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + L.bars);
  uint64_t *a_full = bars, *a_empty = bars + a.stages;
  uint64_t *hank_full = bars + 2 * a.stages, *hank_empty = hank_full + 2, *tmem_full = hank_full + 4,
           *tmem_empty = hank_full + 6, *mma_drain = hank_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(base + L.misc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(base + L.misc + 4);  // + the wait limit at misc + 8
  int *hist = reinterpret_cast<int *>(base + L.hist);
  const bool smem_hist = a.n_hist > 0 && a.n_hist <= kLagHistMax;

  const int tid = threadIdx.x;
  const int warp = tid / 32, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < a.stages; ++s) {
      tc::mbar_init(&a_full[s], 1);
      tc::mbar_init(&a_empty[s], 1);
    }
    for (int k = 0; k < 2; ++k) {
      tc::mbar_init(&hank_full[k], kLagM);  // the 128 builder threads
      tc::mbar_init(&hank_empty[k], 1);     // MMA commit
      tc::mbar_init(&tmem_full[k], 1);      // MMA commit
      tc::mbar_init(&tmem_empty[k], kLagM); // the 128 epilogue threads
    }
    tc::mbar_init(mma_drain, 1);
    tc::mbar_init(reinterpret_cast<uint64_t *>(base + L.misc + 16), 1);  // the probe: never completed
    *abort_flag = 0;
    reinterpret_cast<volatile uint32_t *>(abort_flag)[1] = a.wait_limit ? a.wait_limit : kLagWaitPolls;
    tc::fence_mbarrier_init();
  }
  if (smem_hist)
    for (int h = tid; h < 2 * a.n_hist; h += blockDim.x) hist[h] = 0;
  if (warp == 5) {
    tc::tmem_alloc(tmem_slot, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const long long N = a.n;
  // A-side events walked in blocks of 128: the triangle's rows, or the
  // catalog columns col_begin .. col_begin + n_cols - 1 of a rectangle
  const long long a_row0 = RECT ? a.col_begin : 0;
  // A-side blocks [blk_begin, nblk): all of them, or a chunk of the triangle
  const long long nblk = RECT ? (a.n_cols + kLagM - 1) / kLagM : a.blk_end;
  const long long n_rect = RECT ? a.n_query : 0;
  const long long n_j = RECT ? a.n_query : N;  // j's: triangle events or queries
  const int kchunks = a.lp / kLagKC;
  const int C = a.C;
  constexpr uint32_t tile_bytes = kLagM * kLagKC * 2;
  const uint32_t idesc = tc::idesc_f16_f32(kLagM, a.wt, NHL == 1);
  const uint32_t buf_cols = (uint32_t)(a.jp * a.wpad);  // TMEM columns of one pass

  long long b = RECT ? 0 : a.blk_begin, q = 0;
  advance_item(b, q, blockIdx.x, N, a.jc, nblk, n_rect);

  if (warp == 4) {
    // ================================================= TMA producer (A tiles)
    // converged loop; lane 0 issues the expect-tx arrive and the copies
    {
      int stage = 0;
      uint32_t phase = 0;
      long long it = 0;
      uint32_t issued_mask = 0, last_parity = 0;  // per stage: any load issued / parity of the latest
      // the test probe: a wait that nothing completes runs out before any load
      bool stop = a.wait_probe &&
                  !lag_wait_warp(reinterpret_cast<uint64_t *>(base + L.misc + 16), 0, abort_flag, a.error_flag);
      for (long long bb = b, qq = q; bb < nblk && !stop; advance_item(bb, qq, gridDim.x, N, a.jc, nblk, n_rect)) {
        const long long j_begin = (RECT ? 0 : bb * kLagM) + qq * a.jc;
        const long long j_end = min(j_begin + a.jc, n_j);
        for (long long j0 = j_begin; j0 < j_end && !stop; j0 += a.jp) {
          for (int c = 0; c < C && !stop; ++c) {
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
              if (it >= a.stages && !lag_wait_warp(&a_empty[stage], phase ^ 1, abort_flag, a.error_flag)) {
                stop = true;
                break;
              }
              if (lane == 0) {
                unsigned char *dst = base + L.a + stage * nhl * tile_bytes;
                tc::mbar_arrive_expect_tx(&a_full[stage], nhl * tile_bytes);
                const int row = (int)(c * N + a_row0 + bb * kLagM);
                tc::tma_load_2d(dst, &tm_hi, kc * kLagKC, row, &a_full[stage]);
                if (nhl > 1) tc::tma_load_2d(dst + tile_bytes, &tm_lo, kc * kLagKC, row, &a_full[stage]);
              }
              __syncwarp();
              issued_mask |= 1u << stage;
              last_parity = (last_parity & ~(1u << stage)) | (phase << stage);
              if (++stage == a.stages) {
                stage = 0;
                phase ^= 1;
              }
            }
          }
        }
      }
      // copies in flight land before the CTA may exit (bounded wait per stage)
      for (int st = 0; st < a.stages; ++st)
        if (issued_mask & (1u << st)) tc::mbar_wait(&a_full[st], (last_parity >> st) & 1u, 1u << 20);
    }
  } else if (warp == 5) {
    // ================================================= MMA issuer
    // The warp runs the loop converged and one elected lane issues each MMA
    // and commit (about 6 % faster than a lane-0-only loop).  The loop body
    // is kept to a few adds: descriptors are built once and advanced by their
    // start-address field (16-byte units; shared addresses stay below 2^18
    // bytes, so the field never carries), and the (j, N-tile) pairs of a pass
    // are a fixed table.
    {
      int stage = 0;
      uint32_t phase = 0;
      long long unit = 0, pass = 0;  // (pass, channel) strip units; passes
      const uint64_t da0 = tc::smem_desc(smem_u32(base + L.a), 16, 1024, 2);
      const uint64_t db0 = tc::smem_desc(smem_u32(base + L.hank), 128, 128, 0);
      constexpr uint32_t tile_u = tile_bytes >> 4;   // A tile, descriptor units
      const uint32_t strip_u = (uint32_t)a.strip_bytes >> 4;
      const int nnt = a.nt;
      constexpr int kFastGroup = NHL == 1 ? 4 : 2;  // K-chunks of the unrolled group
      bool stop = false;  // uniform over the warp
      for (long long bb = b, qq = q; bb < nblk && !stop; advance_item(bb, qq, gridDim.x, N, a.jc, nblk, n_rect)) {
        const long long j_begin = (RECT ? 0 : bb * kLagM) + qq * a.jc;
        const long long j_end = min(j_begin + a.jc, n_j);
        for (long long j0 = j_begin; j0 < j_end && !stop; j0 += a.jp, ++pass) {
          const int njp = (int)min((long long)a.jp, j_end - j0);
          const int tb = (int)(pass % a.nbuf);
          const long long tuse = pass / a.nbuf;
          if (tuse > 0 && !lag_wait_warp(&tmem_empty[tb], (uint32_t)((tuse - 1) & 1), abort_flag, a.error_flag)) {
            stop = true;
            break;
          }
          tc::fence_after_sync();
          const uint32_t tbase = tmem + (uint32_t)tb * buf_cols;
          // (j p, N-tile nt) pairs: TMEM column of the accumulator and the
          // strip offset of the tile's first core matrix (descriptor units)
          const int ncombo = njp * nnt;  // 1 or 2 (jp = 2 only with nt = 1)
          uint32_t dcol[2], boff[2];
#pragma unroll
          for (int cb = 0; cb < 2; ++cb) {
            const int p = nnt == 1 ? cb : cb >> 1, nt = nnt == 1 ? 0 : cb & 1;
            dcol[cb] = tbase + (uint32_t)(p * a.wpad + nt * a.wt);
            boff[cb] = (uint32_t)(p * nhl) * strip_u + (uint32_t)(nt * (a.wt / 8) * 8);
          }
          for (int c = 0; c < C && !stop; ++c, ++unit) {
            const int hb = (int)(unit & 1);
            if (!lag_wait_warp(&hank_full[hb], (uint32_t)((unit >> 1) & 1), abort_flag, a.error_flag)) {
              stop = true;
              break;
            }
            tc::fence_after_sync();
            const uint64_t dbu = db0 + (uint64_t)((uint32_t)(hb * a.jp * nhl) * strip_u);
            // K-chunks in groups of `kgroup` ring stages; within a group the
            // MMAs of one K-step offset are issued back to back for every
            // chunk (same accumulator, different operands), which keeps the
            // tensor pipe busier than one chunk's K-steps in a row
            for (int kc0 = 0; kc0 < kchunks && !stop; kc0 += a.kgroup) {
              const int g = min(a.kgroup, kchunks - kc0);
              bool ok = true;
              {
                int st = stage;
                uint32_t ph = phase;
                for (int t = 0; t < g; ++t) {
                  if (!lag_wait_warp(&a_full[st], ph, abort_flag, a.error_flag)) {
                    ok = false;
                    break;
                  }
                  if (++st == a.stages) {
                    st = 0;
                    ph ^= 1;
                  }
                }
              }
              if (!ok) {
                stop = true;
                break;
              }
              tc::fence_after_sync();
              if (g == kFastGroup && ncombo <= 2) {
                // the common cases, fully unrolled: a few adds per MMA
                uint64_t dat[kFastGroup];
                int st = stage;
#pragma unroll
                for (int t = 0; t < kFastGroup; ++t) {
                  dat[t] = da0 + (uint64_t)((uint32_t)(st * nhl) * tile_u);
                  if (++st == a.stages) st = 0;
                }
                const uint64_t dbg = dbu + (uint64_t)(kc0 * (kLagKC / 8) * 8);
                const uint32_t acc_first = (c | kc0) != 0 ? 1u : 0u;
                if (ncombo == 1)
                  lag_mma_group<NHL, kFastGroup, 1>(dcol, boff, dat, dbg, strip_u, idesc, acc_first);
                else
                  lag_mma_group<NHL, kFastGroup, 2>(dcol, boff, dat, dbg, strip_u, idesc, acc_first);
              } else {  // a group cut short by the end of the row (lp / 64 not a multiple)
#pragma unroll 1
                for (int ks = 0; ks < kLagKC / 16; ++ks) {
                  int st = stage;
#pragma unroll 1
                  for (int t = 0; t < g; ++t) {
                    const uint64_t dah = da0 + (uint64_t)((uint32_t)(st * nhl) * tile_u + 2 * ks);
                    const uint64_t dbk = dbu + (uint64_t)(((kc0 + t) * (kLagKC / 8) + 2 * ks) * 8);
                    const uint32_t acc0 = (c | kc0 | ks | t) != 0 ? 1u : 0u;
#pragma unroll 1
                    for (int cb = 0; cb < ncombo; ++cb) {
                      const uint64_t dbh = dbk + (cb == 0 ? boff[0] : boff[1]);
                      const uint32_t d = cb == 0 ? dcol[0] : dcol[1];
                      tc::mma_f16_elect(d, dah, dbh, idesc, acc0);
                      if constexpr (NHL == 2) {
                        tc::mma_f16_elect(d, dah, dbh + strip_u, idesc, 1u);
                        tc::mma_f16_elect(d, dah + tile_u, dbh, idesc, 1u);
                      }
                    }
                    if (++st == a.stages) st = 0;
                  }
                }
              }
              for (int t = 0; t < g; ++t) {
                tc::mma_commit_elect(&a_empty[stage]);
                if (++stage == a.stages) {
                  stage = 0;
                  phase ^= 1;
                }
              }
            }
            tc::mma_commit_elect(&hank_empty[hb]);  // this unit's strips are no longer read
          }
          tc::mma_commit_elect(&tmem_full[tb]);
        }
      }
      // every issued MMA has finished before TMEM is freed (bounded)
      tc::mma_commit_elect(mma_drain);
      tc::mbar_wait(mma_drain, 0, 1u << 20);
    }
  } else if (warp < 4) {
    // ================================================= Hankel strip builders (warps 0-3)
    const int e_lane = tid;  // 0..127
    const int xs_stride = (a.xs_len * 2 + 15) / 16 * 16;
    // xs[u] = x[u - off]: off = shift, or shift - 1 in the rectangle, whose
    // pairs are (j, i) (the lag of pair (query, catalog event) is the negated
    // lag of the GEMM).  The planes hold zeros from L to lp, so each pass
    // copies the lp samples of a row to xs[off ..]; the rest of xs stays zero
    // from here on.
    const int off = RECT ? a.shift - 1 : a.shift;
    for (int w = e_lane; w < a.jp * nhl * xs_stride / 4; w += kLagM)
      reinterpret_cast<uint32_t *>(base + L.xs)[w] = 0u;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const int n8 = a.lp / 8;  // 16-byte chunks per row
    long long unit = 0;
    bool stop = false;  // uniform over the 128 builders
    for (long long bb = b, qq = q; bb < nblk && !stop; advance_item(bb, qq, gridDim.x, N, a.jc, nblk, n_rect)) {
      const long long j_begin = (RECT ? 0 : bb * kLagM) + qq * a.jc;
      const long long j_end = min(j_begin + a.jc, n_j);
      for (long long j0 = j_begin; j0 < j_end && !stop; j0 += a.jp) {
        const int njp = (int)min((long long)a.jp, j_end - j0);
        for (int c = 0; c < C && !stop; ++c, ++unit) {
          const int hb = (int)(unit & 1);
          // wait until the MMAs of the unit two back (same buffer) no longer
          // read it; its outcome is shared by all builders at the barrier
          // below (xs, written before it, is the builders' own)
          const bool ready =
              unit < 2 || lag_wait(&hank_empty[hb], (uint32_t)(((unit >> 1) - 1) & 1), abort_flag, a.error_flag);
          // rows of the j side (triangle events, or the rectangle's queries):
          // chunks f = ((p * nhl + hl) * n8 + ch), four per thread in flight
          const long long row0 = (long long)c * n_j + j0;
          const int n_f = njp * nhl * n8;
          for (int f0 = e_lane; f0 < n_f; f0 += 4 * kLagM) {
            uint4 v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int f = f0 + t * kLagM;
              if (f < n_f) {
                const int ph = f / n8, ch = f - ph * n8;
                const int p = ph / nhl, hl = ph - p * nhl;
                const unsigned short *plane = hl == 0 ? (RECT ? a.qhi : a.xhi) : (RECT ? a.qlo : a.xlo);
                v[t] = __ldg(reinterpret_cast<const uint4 *>(plane + (row0 + p) * a.lp) + ch);
              }
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const int f = f0 + t * kLagM;
              if (f < n_f) {
                const int ph = f / n8, ch = f - ph * n8;
                unsigned short *xs = reinterpret_cast<unsigned short *>(base + L.xs + ph * xs_stride) + off + 8 * ch;
                if ((off & 7) == 0) {
                  *reinterpret_cast<uint4 *>(xs) = v[t];
                } else if ((off & 1) == 0) {
                  uint32_t *x2 = reinterpret_cast<uint32_t *>(xs);
                  x2[0] = v[t].x;
                  x2[1] = v[t].y;
                  x2[2] = v[t].z;
                  x2[3] = v[t].w;
                } else {
                  const uint32_t wv[4] = {v[t].x, v[t].y, v[t].z, v[t].w};
#pragma unroll
                  for (int k = 0; k < 4; ++k) {
                    xs[2 * k] = (unsigned short)(wv[k] & 0xFFFFu);
                    xs[2 * k + 1] = (unsigned short)(wv[k] >> 16);
                  }
                }
              }
            }
          }
          if (!builders_all(ready)) {  // also the barrier before the strips are built
            stop = true;
            break;
          }
          for (int p = 0; p < njp; ++p) {
#pragma unroll
            for (int hl = 0; hl < nhl; ++hl) {
              const uint32_t *xw = reinterpret_cast<const uint32_t *>(base + L.xs + (p * nhl + hl) * xs_stride);
              uint4 *strip =
                  reinterpret_cast<uint4 *>(base + L.hank + ((hb * a.jp + p) * nhl + hl) * a.strip_bytes);
              // core matrix m, row r = xs[o .. o + 7], o = 8m + r: five 32-bit
              // words from xs[o & ~1], shifted by one sample when o is odd
              for (int o = e_lane; o < a.nm * 8; o += kLagM) {
                const uint32_t *src = xw + (o >> 1);
                const uint32_t sh = 16u * (uint32_t)(o & 1);
                uint32_t wd[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) wd[k] = src[k];
                uint32_t w[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) w[k] = __funnelshift_r(wd[k], wd[k + 1], sh);
                strip[o] = make_uint4(w[0], w[1], w[2], w[3]);
              }
            }
          }
          asm volatile("bar.sync 1, 128;" ::: "memory");  // xs is rewritten by the next unit
          tc::fence_proxy_async_smem();
          tc::mbar_arrive(&hank_full[hb]);
        }
      }
    }
  } else {
    // ================================================= epilogue (warps 6-9)
    const int quarter = warp & 3;                 // TMEM lanes 32 quarter .. 32 quarter + 31
    const int e_lane = 32 * quarter + lane;       // event within the block
    const uint32_t lane_addr = (uint32_t)(32 * quarter) << 16;
    long long pass = 0;
    bool stop = false;  // uniform over the warp
    for (long long bb = b, qq = q; bb < nblk && !stop; advance_item(bb, qq, gridDim.x, N, a.jc, nblk, n_rect)) {
      const long long j_begin = (RECT ? 0 : bb * kLagM) + qq * a.jc;
      const long long j_end = min(j_begin + a.jc, n_j);
      for (long long j0 = j_begin; j0 < j_end && !stop; j0 += a.jp, ++pass) {
        const int njp = (int)min((long long)a.jp, j_end - j0);
        const int tb = (int)(pass % a.nbuf);
        if (!lag_wait_warp(&tmem_full[tb], (uint32_t)((pass / a.nbuf) & 1), abort_flag, a.error_flag)) {
          stop = true;
          break;
        }
        tc::fence_after_sync();
        const long long i = a_row0 + bb * kLagM + e_lane;  // A-side event
        // extrema of the (up to two) j's of the pass, then the TMEM buffer
        // goes back to the MMA before the normalisation and the stores
        float bestp[2], worstp[2];
        int bnp[2], wnp[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          if (p < njp) {
            const uint32_t col0 = (uint32_t)tb * buf_cols + (uint32_t)(p * a.wpad);
            // four scan chains (one per 16-column slice of each 64-column
            // block), merged below: chains of 1/4 the length
            float best[4] = {0.f, 0.f, 0.f, 0.f}, worst[4] = {0.f, 0.f, 0.f, 0.f};
            int bn[4] = {0, 0, 0, 0}, wn[4] = {0, 0, 0, 0};
            for (int c0 = 0; c0 < a.wpad; c0 += 64) {
              // up to four 16-column loads in flight, one wait
              uint32_t r[4][16];
              const int nl = min(4, (a.wpad - c0) / 16);
#pragma unroll
              for (int h = 0; h < 4; ++h)
                if (h < nl) tc::tmem_ld16_issue(tmem + lane_addr + col0 + (uint32_t)(c0 + 16 * h), r[h]);
              tc::tmem_ld_wait();
              if (c0 + 64 <= 2 * a.shift) {  // every column of the block is a lag
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                  tc::tmem_regs_ready(r[h]);
                  lag_scan16<RECT, false>(r[h], c0 + 16 * h, 0, best[h], bn[h], worst[h], wn[h]);
                }
              } else {
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                  if (h < nl) {
                    tc::tmem_regs_ready(r[h]);
                    lag_scan16<RECT, true>(r[h], c0 + 16 * h, 2 * a.shift, best[h], bn[h], worst[h], wn[h]);
                  }
                }
              }
            }
#pragma unroll
            for (int h = 1; h < 4; ++h) {
              if (lag_better<RECT>(best[h], bn[h], best[0], bn[0], true)) { best[0] = best[h]; bn[0] = bn[h]; }
              if (lag_better<RECT>(worst[h], wn[h], worst[0], wn[0], false)) { worst[0] = worst[h]; wn[0] = wn[h]; }
            }
            bestp[p] = best[0];
            bnp[p] = bn[0];
            worstp[p] = worst[0];
            wnp[p] = wn[0];
          }
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&tmem_empty[tb]);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const long long j = j0 + p;
          if (p < njp && (RECT ? (i < a.col_begin + a.n_cols && i < N) : (i < N && j >= i))) {
            const float best = bestp[p], worst = worstp[p];
            const int bn = bnp[p], wn = wnp[p];
            // final normalisation in FP64: per-event 1/norm (FP64, kept as hi + lo)
            const float2 *inv = inverse_norms_of(a.norms, N * C);  // A side
            const float2 *inv_j = RECT ? inverse_norms_of(a.q_norms, a.n_query * C) : inv;
            double scale;
            bool live = false;
            if (a.prescaled) {
              for (int cc = 0; cc < C; ++cc) live |= (inv[i * C + cc].x > 0.f) && (inv_j[j * C + cc].x > 0.f);
              scale = 1.0 / (double)C;
            } else {
              const float2 ni = inv[i * C], nj = inv_j[j * C];
              live = ni.x > 0.f && nj.x > 0.f;
              scale = ((double)ni.x + (double)ni.y) * ((double)nj.x + (double)nj.y);
            }
            float vp = 0.f, vn = 0.f;
            int lp = 0, ln = 0;
            if (live) {
              vp = (float)((double)best * scale);
              vn = (float)((double)worst * scale);
              const int lag0 = RECT ? 1 - a.shift : a.shift;  // lag at n = 0
              const int dir = RECT ? 1 : -1;                  // lag step per n
              lp = best > 0.f ? lag0 + dir * bn : 0;
              ln = worst < 0.f ? lag0 + dir * wn : 0;
              if (a.n_hist > 0) {
                const int hp = hist_bin_lag(vp, a.delta_hist, a.n_hist);
                const int hn = hist_bin_lag(-vn, a.delta_hist, a.n_hist);
                if (smem_hist) {
                  atomicAdd(&hist[hp], 1);
                  atomicAdd(&hist[a.n_hist + hn], 1);
                } else {
                  atomicAdd(&a.max_hist[hp], 1);
                  atomicAdd(&a.min_hist[hn], 1);
                }
              }
              if (!(vp > a.threshold)) { vp = 0.f; lp = 0; }
              if (!(vn < -a.threshold)) { vn = 0.f; ln = 0; }
            }
            const long long idx = RECT ? j * a.n_cols + (i - a.col_begin) : i * N - i * (i - 1) / 2 + (j - i);
            a.vals_pos[idx] = vp;
            a.lags_pos[idx] = lp;
            a.vals_neg[idx] = vn;
            a.lags_neg[idx] = ln;
          }
        }
      }
    }
  }

  // ---- teardown: every role is past its loop; flush histograms, free TMEM
  tc::fence_before_sync();
  __syncthreads();
  if (smem_hist) {
    for (int h = tid; h < a.n_hist; h += blockDim.x) {
      if (hist[h]) atomicAdd(&a.max_hist[h], hist[h]);
      if (hist[a.n_hist + h]) atomicAdd(&a.min_hist[h], hist[a.n_hist + h]);
    }
  }
  if (warp == 5) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------------------------ host
// Set by a kernel whose bounded wait ran out (never by a fault).
__device__ int g_device_error;

int *device_error_flag() {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) return nullptr;
  return static_cast<int *>(p);
}

// 2-D map of a [rows][lp] plane of 16-bit values (copied bit for bit; BF16
// or FP16 is the MMA's business).
static bool make_map(CUtensorMap *m, const void *ptr, long long rows, int lp) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)lp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)lp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kLagKC, (cuuint32_t)kLagM};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 16-bit planes per event row of a lag form: BF16 hi + lo (three products) or
// FP16 hi (one product).
int lag_planes(int form) { return form == SEISMIC_FORM_LAGGEMM_FP16 ? 1 : 2; }

// Samples are always scaled by 1/norm before rounding to 16 bits: the
// multichannel mean needs it, FP16's range (+-65504) needs it, and it keeps
// every lag sum within [-1, 1], so raw amplitudes near the ends of FP32's
// range cannot overflow or underflow the FP32 accumulators.
constexpr int kLagPrescaled = 1;

LagPlan lag_plan(long long n_events, int n_channels, int length, int shift, int n_hist, int nhl) {
  LagPlan pl{};
  pl.ok = false;
  if (shift < 1 || 2 * shift > 512 || length < 1 || (nhl != 1 && nhl != 2)) return pl;
  pl.lp = (length + kLagKC - 1) / kLagKC * kLagKC;
  const int w = 2 * shift;
  pl.nt = w > 256 ? 2 : 1;
  pl.wt = ((w + pl.nt - 1) / pl.nt + 15) / 16 * 16;
  pl.wpad = pl.nt * pl.wt;
  // two TMEM buffers of jp accumulators when they fit in 512 columns
  pl.nbuf = 2 * pl.wpad <= 512 ? 2 : 1;
  pl.jp = 512 / pl.nbuf / pl.wpad >= 2 ? 2 : 1;
  pl.nm = pl.wpad / 8 + pl.lp / 8 - 1;
  pl.strip_bytes = (pl.nm + 1) * 128;
  pl.xs_len = pl.wpad + pl.lp + 16;
  pl.jc = 32;
  LagArgs t{};
  t.nhl = nhl;
  t.jp = pl.jp;
  t.strip_bytes = pl.strip_bytes;
  t.xs_len = pl.xs_len;
  t.n_hist = n_hist;
  // A-tile ring: as deep as shared memory allows, up to 8 stages (4, 8 and
  // 10 stages of one plane ran at the same speed; SEISMIC_LAG_STAGES sets
  // another cap, 2 .. 12)
  int max_stages = 8;
  if (const char *env = getenv("SEISMIC_LAG_STAGES")) {
    const int v = atoi(env);
    if (v >= 2 && v <= 12) max_stages = v;
  }
  for (pl.stages = max_stages; pl.stages >= 2; --pl.stages) {
    t.stages = pl.stages;
    pl.smem = lag_smem_layout(t).total;
    if (pl.smem <= 227 * 1024) break;
  }
  pl.ok = pl.smem <= 227 * 1024;
  // MMA groups of up to four K-chunks, with at least as many stages again
  // in the ring for the TMA to fill meanwhile (SEISMIC_LAG_KGROUP overrides).
  // With three BF16 stages (lags +-256) a group of two leaving one stage to
  // refill ran 6 % slower than groups of one (serving, 16.6 vs 15.7 ms).
  pl.kgroup = pl.stages / 2 < kLagGroupMax ? pl.stages / 2 : kLagGroupMax;
  if (const char *env = getenv("SEISMIC_LAG_KGROUP")) {
    const int v = atoi(env);
    if (v >= 1 && v <= kLagGroupMax && v <= pl.stages) pl.kgroup = v;
  }
  if (pl.kgroup < 1) pl.kgroup = 1;
  (void)n_events;
  (void)n_channels;
  return pl;
}

// Workspace of a lag form for n events: [hi planes][lo planes if nhl == 2][norms].
static size_t lag_plane_bytes(long long n, int C, int lp) { return ((size_t)n * C * lp * 2 + 255) / 256 * 256; }

size_t lag_workspace_bytes(long long n, int C, int length, int nhl) {
  const int lp = (length + kLagKC - 1) / kLagKC * kLagKC;
  return nhl * lag_plane_bytes(n, C, lp) + norms_buffer_bytes(n * C) + 256;
}

cudaError_t lag_prepare(const float *events, long long n, int C, int length, long long ev_stride,
                        long long ch_stride, int form, void *ws, cudaStream_t s) {
  const int nhl = lag_planes(form);
  const int lp = (length + kLagKC - 1) / kLagKC * kLagKC;
  const size_t xb = lag_plane_bytes(n, C, lp);
  unsigned short *xhi = reinterpret_cast<unsigned short *>(ws);
  unsigned short *xlo = nhl > 1 ? reinterpret_cast<unsigned short *>(reinterpret_cast<char *>(ws) + xb) : nullptr;
  double *norms = reinterpret_cast<double *>(reinterpret_cast<char *>(ws) + nhl * xb);
  const long long rows = n * C;
  const unsigned grid = (unsigned)((rows + 7) / 8);
  if (nhl == 1)
    lag_prep_kernel<true><<<grid, 256, 0, s>>>(events, n, C, length, ev_stride, ch_stride, lp, kLagPrescaled,
                                               xhi, nullptr, norms);
  else
    lag_prep_kernel<false><<<grid, 256, 0, s>>>(events, n, C, length, ev_stride, ch_stride, lp,
                                                kLagPrescaled, xhi, xlo, norms);
  return cudaGetLastError();
}

// Shared set-up and launch of lag_gemm_kernel once `a` holds the operands.
static cudaError_t launch_lag_kernel(LagArgs &a, const LagPlan &pl, const unsigned short *a_hi,
                                     const unsigned short *a_lo, long long a_rows, long long items, int sm_count,
                                     cudaStream_t s) {
  CUtensorMap mhi, mlo;
  if (!make_map(&mhi, a_hi, a_rows, pl.lp)) return cudaErrorInvalidValue;
  if (!make_map(&mlo, a_lo ? a_lo : a_hi, a_rows, pl.lp)) return cudaErrorInvalidValue;
  a.lp = pl.lp;
  a.wpad = pl.wpad;
  a.nt = pl.nt;
  a.wt = pl.wt;
  a.jp = pl.jp;
  a.nbuf = pl.nbuf;
  a.nm = pl.nm;
  a.strip_bytes = pl.strip_bytes;
  a.xs_len = pl.xs_len;
  a.stages = pl.stages;
  a.kgroup = pl.kgroup;
  a.prescaled = kLagPrescaled;
  a.delta_hist = a.n_hist > 0 ? (float)(1.0 / a.n_hist) : 0.f;
  {
    const LagSmem lay = lag_smem_layout(a);
    a.off_a = lay.a;
    a.off_hank = lay.hank;
    a.off_xs = lay.xs;
    a.off_hist = lay.hist;
    a.off_bars = lay.bars;
    a.off_misc = lay.misc;
  }
  void (*kern)(const CUtensorMap, const CUtensorMap, LagArgs) =
      a.nhl == 1 ? (a.rect ? lag_gemm_kernel<1, true> : lag_gemm_kernel<1, false>)
                 : (a.rect ? lag_gemm_kernel<2, true> : lag_gemm_kernel<2, false>);
  {
    cudaError_t e = ensure_dynamic_smem((const void *)kern, 227 * 1024);
    if (e != cudaSuccess) return e;
  }
  if (items <= 0) return cudaSuccess;
  const long long grid = items < sm_count ? items : sm_count;
  kern<<<(unsigned)grid, kLagThreads, pl.smem, s>>>(mhi, mlo, a);
  return cudaGetLastError();
}

long long lag_blocks(long long n) { return (n + kLagM - 1) / kLagM; }

long long lag_block_row(long long b, long long n) { return b * kLagM < n ? b * kLagM : n; }

cudaError_t launch_lag_blocks(const void *ws, long long n, int C, int length, int shift, float threshold,
                              int n_hist, float *vp, int *lp, float *vn, int *ln, int *hmax, int *hmin,
                              int *error_flag, int sm_count, cudaStream_t s, int form, long long blk_begin,
                              long long blk_end) {
  const int nhl = lag_planes(form);
  const LagPlan pl = lag_plan(n, C, length, shift, n_hist, nhl);
  const long long nblk = lag_blocks(n);
  if (!pl.ok || blk_begin < 0 || blk_end > nblk || blk_begin > blk_end) return cudaErrorInvalidValue;
  const size_t xb = lag_plane_bytes(n, C, pl.lp);
  const unsigned short *xhi = reinterpret_cast<const unsigned short *>(ws);
  const unsigned short *xlo =
      nhl > 1 ? reinterpret_cast<const unsigned short *>(reinterpret_cast<const char *>(ws) + xb) : nullptr;
  LagArgs a{};
  a.xhi = xhi;
  a.xlo = xlo;
  a.norms = reinterpret_cast<const double *>(reinterpret_cast<const char *>(ws) + nhl * xb);
  a.n = n;
  a.C = C;
  a.L = length;
  a.shift = shift;
  a.nhl = nhl;
  a.jc = pl.jc;
  a.threshold = threshold;
  a.n_hist = n_hist;
  a.vals_pos = vp;
  a.lags_pos = lp;
  a.vals_neg = vn;
  a.lags_neg = ln;
  a.max_hist = hmax;
  a.min_hist = hmin;
  a.error_flag = error_flag;
  a.wait_limit = device_wait_polls();
  a.wait_probe = device_wait_probe();
  a.blk_begin = blk_begin;
  a.blk_end = blk_end;
  long long items = 0;
  for (long long bb = blk_begin; bb < blk_end; ++bb) items += (n - bb * kLagM + pl.jc - 1) / pl.jc;
  return launch_lag_kernel(a, pl, xhi, xlo, n * C, items, sm_count, s);
}

cudaError_t launch_lag_gemm(const float *events, long long n, int C, int length, long long ev_stride,
                            long long ch_stride, int shift, float threshold, int n_hist, float *vp, int *lp,
                            float *vn, int *ln, int *hmax, int *hmin, void *ws, int *error_flag, int sm_count,
                            cudaStream_t s, int *launches, int form) {
  if (!lag_plan(n, C, length, shift, n_hist, lag_planes(form)).ok) return cudaErrorInvalidValue;
  cudaError_t e = lag_prepare(events, n, C, length, ev_stride, ch_stride, form, ws, s);
  if (e != cudaSuccess) return e;
  ++*launches;
  e = launch_lag_blocks(ws, n, C, length, shift, threshold, n_hist, vp, lp, vn, ln, hmax, hmin, error_flag,
                        sm_count, s, form, 0, lag_blocks(n));
  if (e == cudaSuccess) ++*launches;
  return e;
}

cudaError_t launch_lag_rect(const void *cat_ws, long long n_cat, const void *q_ws, long long n_query, int C,
                            int length, int shift, long long col_begin, long long n_cols, float threshold, int form,
                            float *vp, int *lp, float *vn, int *ln, int *error_flag, int sm_count, cudaStream_t s) {
  const int nhl = lag_planes(form);
  LagPlan pl = lag_plan(n_cat, C, length, shift, 0, nhl);
  if (!pl.ok || col_begin < 0 || n_cols < 1 || col_begin + n_cols > n_cat || n_query < 1)
    return cudaErrorInvalidValue;
  pl.jc = 8;  // queries per item: more items than SMs for a 64-query request (4 and 8 measured equal, 16 slower)
  if (const char *env = getenv("SEISMIC_LAG_RECT_JC")) {  // 1 .. 64, a multiple of jp
    const int v = atoi(env);
    if (v >= 1 && v <= 64 && v % pl.jp == 0) pl.jc = v;
  }
  const size_t cb = lag_plane_bytes(n_cat, C, pl.lp), qb = lag_plane_bytes(n_query, C, pl.lp);
  const char *cw = static_cast<const char *>(cat_ws), *qw = static_cast<const char *>(q_ws);
  LagArgs a{};
  a.rect = 1;
  a.xhi = reinterpret_cast<const unsigned short *>(cw);
  a.xlo = nhl > 1 ? reinterpret_cast<const unsigned short *>(cw + cb) : nullptr;
  a.norms = reinterpret_cast<const double *>(cw + nhl * cb);
  a.qhi = reinterpret_cast<const unsigned short *>(qw);
  a.qlo = nhl > 1 ? reinterpret_cast<const unsigned short *>(qw + qb) : nullptr;
  a.q_norms = reinterpret_cast<const double *>(qw + nhl * qb);
  a.n = n_cat;
  a.n_query = n_query;
  a.col_begin = col_begin;
  a.n_cols = n_cols;
  a.C = C;
  a.L = length;
  a.shift = shift;
  a.nhl = nhl;
  a.jc = pl.jc;
  a.threshold = threshold;
  a.vals_pos = vp;
  a.lags_pos = lp;
  a.vals_neg = vn;
  a.lags_neg = ln;
  a.error_flag = error_flag;
  a.wait_limit = device_wait_polls();
  a.wait_probe = device_wait_probe();
  const long long nblk = (n_cols + kLagM - 1) / kLagM;
  const long long items = nblk * ((n_query + pl.jc - 1) / pl.jc);
  return launch_lag_kernel(a, pl, a.xhi, a.xlo, n_cat * C, items, sm_count, s);
}

}  // namespace seismic
