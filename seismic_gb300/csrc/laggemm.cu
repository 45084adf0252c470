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
// FP32 accuracy from BF16 inputs: x = hi + lo with hi = bf16(x),
// lo = bf16(x - hi); each lag product is hi_i hi_j + hi_i lo_j + lo_i hi_j
// (three MMAs into the same FP32 accumulator; lo*lo ~ 2^-16 relative is
// dropped).  Norms and the final normalisation are FP64, as in the FFT form.
//
// Work: persistent CTAs (one per SM: 512 TMEM columns and ~200 KB of shared
// memory each) walk items (I-block of 128 events, chunk of `jc` events j >=
// block start); j's are processed `jp` at a time (a "pass": jp accumulators
// of nt * wt columns).  The stages overlap: the Hankel strips are double
// buffered per (pass, channel) and TMEM holds two passes' accumulators when
// 2 jp wpad <= 512, so the strips of the next j are built and the previous
// pass's accumulators are reduced while the tensor cores run.  Warp roles:
//   warps 0-3  build the Hankel strips of the next (pass, channel);
//   warp 4     TMA producer of the A tiles (128 events x 64 samples, hi and
//              lo, 128-byte swizzle) into a `stages`-deep ring;
//   warp 5     TMEM allocation and the single MMA-issuing thread;
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

#include <climits>
#include <cstdio>

#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma_host.cuh"

namespace seismic {

using tc::smem_u32;

constexpr int kLagM = 128;       // events per I-block (MMA M)
constexpr int kLagKC = 64;       // samples per A tile (one 128-byte swizzle row)
constexpr int kLagThreads = 320; // 10 warps
constexpr int kLagHistMax = 1024;

// ------------------------------------------------------------------ prep
// One warp per (event, channel) row: FP64 norm, then hi/lo BF16 split of the
// (optionally 1/norm-scaled) samples into channel-major [C][N][Lp] arrays.
__global__ void lag_prep_kernel(const float *__restrict__ ev, long long n, int C, int L, long long ev_stride,
                                long long ch_stride, int lp, int prescale, __nv_bfloat16 *__restrict__ xhi,
                                __nv_bfloat16 *__restrict__ xlo, double *__restrict__ norms) {
  const long long row = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n * C) return;
  const long long e = row / C;
  const int c = (int)(row % C);
  const float *src = ev + e * ev_stride + (long long)c * ch_stride;
  double s = 0.0;
  for (int k = lane; k < L; k += 32) {
    const double v = src[k];
    s += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const double nrm = sqrt(s);
  const float scale = prescale ? (nrm > 0.0 ? (float)(1.0 / nrm) : 0.f) : 1.f;
  __nv_bfloat16 *dh = xhi + ((long long)c * n + e) * lp;
  __nv_bfloat16 *dl = xlo + ((long long)c * n + e) * lp;
  for (int k = lane; k < lp; k += 32) {
    const float v = k < L ? src[k] * scale : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    dh[k] = h;
    dl[k] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
  if (lane == 0) {
    norms[row] = nrm;
    inverse_norms_of(norms, n * C)[row] = nrm > 0.0 ? (float)(1.0 / nrm) : 0.f;
  }
}

// ------------------------------------------------------------------ main
struct LagArgs {
  const __nv_bfloat16 *xhi, *xlo;  // [C][N][Lp]
  const double *norms;             // [N*C], event-major
  long long n;
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
};

struct LagSmem {  // offsets into dynamic shared memory (base 1024-aligned)
  int a, hank, xs, hist, bars, misc, total;
};

static LagSmem lag_smem_layout(const LagArgs &a) {
  LagSmem s;
  int off = 0;
  s.a = off;
  off += a.stages * 2 * kLagM * kLagKC * 2;  // hi + lo tiles per stage
  s.hank = off;
  off += 2 * a.jp * 2 * a.strip_bytes;  // two buffers of jp (hi, lo) strips
  s.xs = off;
  off += a.jp * 2 * ((a.xs_len * 2 + 15) / 16 * 16);
  s.hist = off;
  off += (a.n_hist > 0 && a.n_hist <= kLagHistMax) ? 2 * a.n_hist * 4 : 0;
  off = (off + 7) / 8 * 8;
  s.bars = off;
  off += (2 * a.stages + 9) * 8;
  s.misc = off;
  off += 16;
  s.total = off + 1024;  // room to align the base
  return s;
}

__device__ __forceinline__ bool lag_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err) {
  for (uint32_t it = 0; it < (1u << 22); ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (it > 64) __nanosleep(it > 4096 ? 512 : 32);
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ int hist_bin_lag(float v, float delta, int n_hist) {
  if (v >= 1.0f) return n_hist - 1;
  int b = (int)(v / delta);
  return b > n_hist - 1 ? n_hist - 1 : (b < 0 ? 0 : b);
}

// Items: row-block b (events [128b, 128b+128)) x chunk q of j's starting at
// 128b, each chunk `jc` events.  Advance (b, q) by `step` items.
__device__ __forceinline__ void advance_item(long long &b, long long &q, long long step, long long n, int jc,
                                             long long nblk) {
  while (step > 0 && b < nblk) {
    const long long rows_j = n - b * kLagM;
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

__global__ void __launch_bounds__(kLagThreads, 1)
    lag_gemm_kernel(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
                    LagArgs a) {
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
  volatile int *abort_flag = reinterpret_cast<volatile int *>(base + L.misc + 4);
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
    *abort_flag = 0;
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
  const long long nblk = (N + kLagM - 1) / kLagM;
  const int kchunks = a.lp / kLagKC;
  const int C = a.C;
  const uint32_t tile_bytes = kLagM * kLagKC * 2;
  const uint32_t idesc = tc::idesc_bf16_f32(kLagM, a.wt);
  const uint32_t buf_cols = (uint32_t)(a.jp * a.wpad);  // TMEM columns of one pass

  long long b = 0, q = 0;
  advance_item(b, q, blockIdx.x, N, a.jc, nblk);

  if (warp == 4) {
    // ================================================= TMA producer (A tiles)
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      long long it = 0;
      uint32_t issued_mask = 0, last_parity = 0;  // per stage: any load issued / parity of the latest
      for (long long bb = b, qq = q; bb < nblk && !*abort_flag; advance_item(bb, qq, gridDim.x, N, a.jc, nblk)) {
        const long long j_begin = bb * kLagM + qq * a.jc;
        const long long j_end = min(j_begin + a.jc, N);
        for (long long j0 = j_begin; j0 < j_end && !*abort_flag; j0 += a.jp) {
          for (int c = 0; c < C && !*abort_flag; ++c) {
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
              if (it >= a.stages && !lag_wait(&a_empty[stage], phase ^ 1, abort_flag, a.error_flag)) break;
              unsigned char *dst = base + L.a + stage * 2 * tile_bytes;
              tc::mbar_arrive_expect_tx(&a_full[stage], 2 * tile_bytes);
              const int row = (int)(c * N + bb * kLagM);
              tc::tma_load_2d(dst, &tm_hi, kc * kLagKC, row, &a_full[stage]);
              tc::tma_load_2d(dst + tile_bytes, &tm_lo, kc * kLagKC, row, &a_full[stage]);
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
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      long long unit = 0, pass = 0;  // (pass, channel) strip units; passes
      for (long long bb = b, qq = q; bb < nblk && !*abort_flag; advance_item(bb, qq, gridDim.x, N, a.jc, nblk)) {
        const long long j_begin = bb * kLagM + qq * a.jc;
        const long long j_end = min(j_begin + a.jc, N);
        for (long long j0 = j_begin; j0 < j_end && !*abort_flag; j0 += a.jp, ++pass) {
          const int njp = (int)min((long long)a.jp, j_end - j0);
          const int tb = (int)(pass % a.nbuf);
          const long long tuse = pass / a.nbuf;
          if (tuse > 0 && !lag_wait(&tmem_empty[tb], (uint32_t)((tuse - 1) & 1), abort_flag, a.error_flag)) break;
          tc::fence_after_sync();
          const uint32_t tbase = tmem + (uint32_t)tb * buf_cols;
          for (int c = 0; c < C && !*abort_flag; ++c, ++unit) {
            const int hb = (int)(unit & 1);
            if (!lag_wait(&hank_full[hb], (uint32_t)((unit >> 1) & 1), abort_flag, a.error_flag)) break;
            tc::fence_after_sync();
            for (int kc = 0; kc < kchunks; ++kc) {
              if (!lag_wait(&a_full[stage], phase, abort_flag, a.error_flag)) break;
              tc::fence_after_sync();
              const uint32_t a_hi = smem_u32(base + L.a + stage * 2 * tile_bytes);
              const uint32_t a_lo = a_hi + tile_bytes;
#pragma unroll
              for (int ks = 0; ks < kLagKC / 16; ++ks) {
                const uint64_t dah = tc::smem_desc(a_hi + 32 * ks, 16, 1024, 2);
                const uint64_t dal = tc::smem_desc(a_lo + 32 * ks, 16, 1024, 2);
                const int h0 = kc * (kLagKC / 8) + 2 * ks;  // k core-matrix index
                for (int p = 0; p < njp; ++p) {
                  const uint32_t s_hi = smem_u32(base + L.hank + ((hb * a.jp + p) * 2 + 0) * a.strip_bytes);
                  const uint32_t s_lo = s_hi + a.strip_bytes;
                  for (int nt = 0; nt < a.nt; ++nt) {
                    const uint32_t coff = (uint32_t)((nt * (a.wt / 8) + h0) * 128);
                    const uint64_t dbh = tc::smem_desc(s_hi + coff, 128, 128, 0);
                    const uint64_t dbl = tc::smem_desc(s_lo + coff, 128, 128, 0);
                    const uint32_t d = tbase + (uint32_t)(p * a.wpad + nt * a.wt);
                    const uint32_t acc0 = (c > 0 || kc > 0 || ks > 0) ? 1u : 0u;
                    tc::mma_bf16(d, dah, dbh, idesc, acc0);
                    tc::mma_bf16(d, dah, dbl, idesc, 1u);
                    tc::mma_bf16(d, dal, dbh, idesc, 1u);
                  }
                }
              }
              tc::mma_commit(&a_empty[stage]);
              if (++stage == a.stages) {
                stage = 0;
                phase ^= 1;
              }
            }
            tc::mma_commit(&hank_empty[hb]);  // this unit's strips are no longer read
          }
          tc::mma_commit(&tmem_full[tb]);
        }
      }
      // every issued MMA has finished before TMEM is freed (bounded)
      tc::mma_commit(mma_drain);
      tc::mbar_wait(mma_drain, 0, 1u << 20);
    }
  } else if (warp < 4) {
    // ================================================= Hankel strip builders (warps 0-3)
    const int e_lane = tid;  // 0..127
    long long unit = 0;
    for (long long bb = b, qq = q; bb < nblk && !*abort_flag; advance_item(bb, qq, gridDim.x, N, a.jc, nblk)) {
      const long long j_begin = bb * kLagM + qq * a.jc;
      const long long j_end = min(j_begin + a.jc, N);
      for (long long j0 = j_begin; j0 < j_end && !*abort_flag; j0 += a.jp) {
        const int njp = (int)min((long long)a.jp, j_end - j0);
        for (int c = 0; c < C && !*abort_flag; ++c, ++unit) {
          const int hb = (int)(unit & 1);
          // wait until the MMAs of the unit two back (same buffer) no longer read it
          if (unit >= 2 && !lag_wait(&hank_empty[hb], (uint32_t)(((unit >> 1) - 1) & 1), abort_flag, a.error_flag))
            break;
          const int xs_stride = (a.xs_len * 2 + 15) / 16 * 16;
          for (int p = 0; p < njp; ++p) {
            const long long j = j0 + p;
            const __nv_bfloat16 *srcs[2] = {a.xhi + ((long long)c * N + j) * a.lp,
                                            a.xlo + ((long long)c * N + j) * a.lp};
#pragma unroll
            for (int hl = 0; hl < 2; ++hl) {
              unsigned short *xs = reinterpret_cast<unsigned short *>(base + L.xs + (p * 2 + hl) * xs_stride);
              const unsigned short *src = reinterpret_cast<const unsigned short *>(srcs[hl]);
              // xs[u] = x[u - shift] (zero outside [0, L))
              for (int u = e_lane; u < a.xs_len; u += kLagM) {
                const int k = u - a.shift;
                xs[u] = (k >= 0 && k < a.L) ? src[k] : (unsigned short)0;
              }
            }
          }
          asm volatile("bar.sync 1, 128;" ::: "memory");
          for (int p = 0; p < njp; ++p) {
#pragma unroll
            for (int hl = 0; hl < 2; ++hl) {
              const unsigned short *xs =
                  reinterpret_cast<const unsigned short *>(base + L.xs + (p * 2 + hl) * xs_stride);
              uint4 *strip =
                  reinterpret_cast<uint4 *>(base + L.hank + ((hb * a.jp + p) * 2 + hl) * a.strip_bytes);
              // core matrix m, row r = xs[8m + r .. 8m + r + 7]
              for (int rowi = e_lane; rowi < a.nm * 8; rowi += kLagM) {
                const int o = rowi;  // 8m + r
                uint32_t w[4];
#pragma unroll
                for (int qd = 0; qd < 4; ++qd)
                  w[qd] = (uint32_t)xs[o + 2 * qd] | ((uint32_t)xs[o + 2 * qd + 1] << 16);
                strip[rowi] = make_uint4(w[0], w[1], w[2], w[3]);
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
    for (long long bb = b, qq = q; bb < nblk && !*abort_flag; advance_item(bb, qq, gridDim.x, N, a.jc, nblk)) {
      const long long j_begin = bb * kLagM + qq * a.jc;
      const long long j_end = min(j_begin + a.jc, N);
      for (long long j0 = j_begin; j0 < j_end && !*abort_flag; j0 += a.jp, ++pass) {
        const int njp = (int)min((long long)a.jp, j_end - j0);
        const int tb = (int)(pass % a.nbuf);
        if (!lag_wait(&tmem_full[tb], (uint32_t)((pass / a.nbuf) & 1), abort_flag, a.error_flag)) break;
        tc::fence_after_sync();
        const long long i = bb * kLagM + e_lane;
        for (int p = 0; p < njp; ++p) {
          const long long j = j0 + p;
          float best = 0.f, worst = 0.f;
          int bn = 0, wn = 0;
          const uint32_t col0 = (uint32_t)tb * buf_cols + (uint32_t)(p * a.wpad);
          for (int c0 = 0; c0 < a.wpad; c0 += 64) {
            // up to four 16-column loads in flight, one wait
            uint32_t r[4][16];
            const int nl = min(4, (a.wpad - c0) / 16);
#pragma unroll
            for (int h = 0; h < 4; ++h)
              if (h < nl) tc::tmem_ld16_issue(tmem + lane_addr + col0 + (uint32_t)(c0 + 16 * h), r[h]);
            tc::tmem_ld_wait();
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              if (h < nl) {
                tc::tmem_regs_ready(r[h]);
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                  const int n = c0 + 16 * h + k;
                  const float v = __uint_as_float(r[h][k]);
                  if (n < 2 * a.shift) {
                    // n increasing = lag decreasing: ">=" keeps the largest n among
                    // equal values, i.e. the smallest lag (first occurrence)
                    if (v >= best) { best = v; bn = n; }
                    if (v <= worst) { worst = v; wn = n; }
                  }
                }
              }
            }
          }
          if (i < N && j >= i) {
            // per-event 1/norm factors come from FP64 (prep kernel); per pair FP32
            const float *inv = inverse_norms_of(a.norms, N * C);
            float scale;
            bool live = false;
            if (a.prescaled) {
              for (int cc = 0; cc < C; ++cc) live |= (inv[i * C + cc] > 0.f) && (inv[j * C + cc] > 0.f);
              scale = 1.0f / (float)C;
            } else {
              const float ni = inv[i * C], nj = inv[j * C];
              live = ni > 0.f && nj > 0.f;
              scale = ni * nj;
            }
            float vp = 0.f, vn = 0.f;
            int lp = 0, ln = 0;
            if (live) {
              vp = best * scale;
              vn = worst * scale;
              lp = best > 0.f ? a.shift - bn : 0;
              ln = worst < 0.f ? a.shift - wn : 0;
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
            const long long idx = i * N - i * (i - 1) / 2 + (j - i);
            a.vals_pos[idx] = vp;
            a.lags_pos[idx] = lp;
            a.vals_neg[idx] = vn;
            a.lags_neg[idx] = ln;
          }
        }
        tc::fence_before_sync();
        tc::mbar_arrive(&tmem_empty[tb]);
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

LagPlan lag_plan(long long n_events, int n_channels, int length, int shift, int n_hist) {
  LagPlan pl{};
  pl.ok = false;
  if (shift < 1 || 2 * shift > 512 || length < 1) return pl;
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
  t.stages = 4;
  t.jp = pl.jp;
  t.strip_bytes = pl.strip_bytes;
  t.xs_len = pl.xs_len;
  t.n_hist = n_hist;
  for (pl.stages = 4; pl.stages >= 2; --pl.stages) {
    t.stages = pl.stages;
    pl.smem = lag_smem_layout(t).total;
    if (pl.smem <= 227 * 1024) break;
  }
  pl.ok = pl.smem <= 227 * 1024;
  (void)n_events;
  (void)n_channels;
  return pl;
}

size_t lag_workspace_bytes(long long n, int C, int length) {
  const int lp = (length + kLagKC - 1) / kLagKC * kLagKC;
  const size_t x = (size_t)n * C * lp * 2;
  return 2 * ((x + 255) / 256 * 256) + norms_buffer_bytes(n * C) + 256;
}

cudaError_t launch_lag_gemm(const float *events, long long n, int C, int length, long long ev_stride,
                            long long ch_stride, int shift, float threshold, int n_hist, float *vp, int *lp,
                            float *vn, int *ln, int *hmax, int *hmin, void *ws, int *error_flag, int sm_count,
                            cudaStream_t s, int *launches) {
  const LagPlan pl = lag_plan(n, C, length, shift, n_hist);
  if (!pl.ok) return cudaErrorInvalidValue;
  const size_t x = (size_t)n * C * pl.lp * 2;
  const size_t xb = (x + 255) / 256 * 256;
  __nv_bfloat16 *xhi = reinterpret_cast<__nv_bfloat16 *>(ws);
  __nv_bfloat16 *xlo = reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(ws) + xb);
  double *norms = reinterpret_cast<double *>(reinterpret_cast<char *>(ws) + 2 * xb);
  const long long rows = n * C;
  lag_prep_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, s>>>(events, n, C, length, ev_stride, ch_stride, pl.lp,
                                                             C > 1 ? 1 : 0, xhi, xlo, norms);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  ++*launches;

  CUtensorMap mhi, mlo;
  if (!make_map(&mhi, xhi, rows, pl.lp) || !make_map(&mlo, xlo, rows, pl.lp)) return cudaErrorInvalidValue;
  LagArgs a{};
  a.xhi = xhi;
  a.xlo = xlo;
  a.norms = norms;
  a.n = n;
  a.C = C;
  a.L = length;
  a.lp = pl.lp;
  a.shift = shift;
  a.wpad = pl.wpad;
  a.nt = pl.nt;
  a.wt = pl.wt;
  a.jp = pl.jp;
  a.nbuf = pl.nbuf;
  a.jc = pl.jc;
  a.nm = pl.nm;
  a.strip_bytes = pl.strip_bytes;
  a.xs_len = pl.xs_len;
  a.stages = pl.stages;
  a.prescaled = C > 1 ? 1 : 0;
  a.threshold = threshold;
  a.n_hist = n_hist;
  a.delta_hist = n_hist > 0 ? (float)(1.0 / n_hist) : 0.f;
  a.vals_pos = vp;
  a.lags_pos = lp;
  a.vals_neg = vn;
  a.lags_neg = ln;
  a.max_hist = hmax;
  a.min_hist = hmin;
  a.error_flag = error_flag;
  {
    const LagSmem lay = lag_smem_layout(a);
    a.off_a = lay.a;
    a.off_hank = lay.hank;
    a.off_xs = lay.xs;
    a.off_hist = lay.hist;
    a.off_bars = lay.bars;
    a.off_misc = lay.misc;
  }
  static int configured = 0;
  if (configured < pl.smem) {
    e = cudaFuncSetAttribute(lag_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return e;
    configured = 227 * 1024;
  }
  const long long nblk = (n + kLagM - 1) / kLagM;
  long long items = 0;
  for (long long bb = 0; bb < nblk; ++bb) items += (n - bb * kLagM + pl.jc - 1) / pl.jc;
  const long long grid = items < sm_count ? items : sm_count;
  lag_gemm_kernel<<<(unsigned)grid, kLagThreads, pl.smem, s>>>(mhi, mlo, a);
  e = cudaGetLastError();
  if (e == cudaSuccess) ++*launches;
  return e;
}

}  // namespace seismic
