// Kernels (b) + (c), staged form: the pair-tile kernel with its spectra
// staged into shared memory by TMA.  Same results as the direct form
// (pairs.cu); replaces the same reference code:
//   ElementWiseMultiplication  Correlation_in_OMP/correlation_c.cpp:188-193
//   inverseFFT                 Correlation_in_OMP/correlation_c.cpp:58-137
//   the dynamic row loop       Correlation_in_OMP/correlation_c.cpp:251-293
//
// Work item = TI consecutive events i0 .. i0+TI-1 and TJ = 2 NG / TI
// consecutive events j0 .. j0+TJ-1 (StagedGeom); group g of the CTA's NG FFT
// groups takes the couple (i0 + g / (TJ/2); j0 + 2 (g % (TJ/2)), +1) -- the
// same couples as the direct form, so both forms give bit-identical results.
// The items of the upper triangle tile squares of TS = lcm(TI, TJ) events,
// walked in row bands of `band_tiles` tile rows so the i spectra of a band
// stay in L2 while every column to its right passes over it once (and a
// band's outputs are contiguous packed rows); the rectangle (query x
// catalog) walks column blocks of TJ events, all query blocks per column
// block.
//
// Pipeline.  Each item's spectra are cut into units (channel c, chunk r):
// bins [r S, (r+1) S) of the TI rows i0.. and the TJ rows j0.., exactly the
// bins ca + r S and cb + r S every FFT thread reads at step r
// (pair_core.cuh).  A producer warp (one elected thread) streams units into
// a ring of K shared-memory slots: two 3-D TMA boxes {S bins, 1 channel, TI
// or TJ events} (rows past the last event are zero-filled by the TMA unit),
// completing on the slot's `full` mbarrier; the FFT warps conj-multiply
// from the slot and release it on its `empty` mbarrier.  While the groups
// run their inverse FFTs the producer fills the ring with the next item's
// units, so spectra reads leave the critical path.  A unit stages TI + TJ
// rows for TI TJ pairs, each row shared by all the groups that use it: with
// 24 groups, TI = 6 stages 14 rows per 48 pairs where one i per item (TI =
// 1) stages 49, so the ring holds a whole item of the overlap-save form and
// the FFT threads no longer wait for units at the start of an item.
//
// Bounded waits and the abort path.  The producer's waits (for a slot to be
// released) are bounded by PairArgs::wait_limit polls; one that runs out sets
// the device error flag (the host reports SEISMIC_ERR_DEVICE_TIMEOUT; the
// outputs are then incomplete) and the CTA's abort flag, and the producer
// issues nothing more.  Before it leaves, the producer waits for every copy
// it issued to land (copies from valid memory always complete; this wait is
// bounded too), so the CTA never exits with a copy still writing its shared
// memory.  The FFT threads poll their `full` barrier and give up only when a
// unit's copies have not landed AND the abort flag is set, i.e. at a unit
// the producer never issued; a group leaves its item loop only by a vote of
// all its threads, so no thread is left waiting at a group barrier.
// (This header holds the kernel and its launch templates; pairs_staged.cu and
// pairs_staged_large.cu instantiate them for P = 512, 1024 and 2048, 4096, two
// translation units that compile in parallel.)
#pragma once
#include <cstdlib>
#include <cstring>

#include "pair_core.cuh"
#include "tcgen05.cuh"
#include "tma_host.cuh"

namespace seismic {

constexpr int kStagedHistMax = 1024;  // larger histograms use global atomics
constexpr int kStagedRingMax = 16;
// Decoded items published by the producer; it runs at most kStagedRingMax
// units (>= 2 per item) ahead of the slowest FFT thread, so 16 entries never
// wrap onto an item still being read.
constexpr int kItemRing = 16;
constexpr size_t kStagedSmemBudget = 227 * 1024;

template <int P, int NWARP, int RU, int ST> struct Staged {  // RU: chunks r per ring slot, ST: spectra type
  static constexpr int G = P / 32;
  static constexpr int NG = NWARP * 32 / G;  // FFT groups per CTA
  static constexpr int S = P / 16;
  static constexpr int NW = (G + 31) / 32;
  static constexpr int CONSUMERS = NWARP * 32;  // FFT threads
  static constexpr int THREADS = CONSUMERS + 32;  // + the producer warp
  // exchange buffer of one group.  P = 4096 with FP32 spectra runs its
  // exchanges in two halves (inverse_fft_group_split) and leaves the other
  // half to the ring: N=4096 C=3 94.6 -> 102.3 M pairs/s.  Elsewhere the
  // extra barriers cost more than the ring gains (measured, M pairs/s,
  // full / split exchange): FP16 spectra at that shape 102.5 / 92.0; the
  // overlap-save Q=512 x 4 form 831 / 813; Q=1024 x 2 with three channels
  // 340 / 336; plain P=2048 one channel 268 / 262 -- only plain P=2048 with
  // three channels gained (198 / 211).
  static constexpr bool SPLIT_EX = P == 4096 && ST == 0;
  static constexpr int EX_LEN = SPLIT_EX ? padded_len<P / 2>() : padded_len<P>();
  static constexpr size_t EX_BYTES = (size_t)NG * EX_LEN * sizeof(float2);
  static constexpr size_t RED_BYTES = (size_t)NG * NW * 8 * sizeof(unsigned);
  static constexpr size_t PROD_OFF = (EX_BYTES + RED_BYTES + 15) / 16 * 16;
  // producer area: cursor (48 B), abort flag (+48), probe mbarrier (+56),
  // item ring of kItemRing (i, j0)
  static constexpr size_t ITEMS_OFF = PROD_OFF + 64;
  static constexpr size_t RING_OFF = (ITEMS_OFF + kItemRing * 16 + 127) / 128 * 128;
};

// Item geometry: TI i events x TJ = 2 NG / TI j events per item (TI divides
// NG), square tiles of TS = lcm(TI, TJ) events holding (TS / TI) x (TS / TJ)
// items, row-major.  TI = 1 is one i per item (TS = TJ = 2 NG).
struct StagedGeom {
  int ti, tj, ts;
  int jpt;        // items along a tile row: TS / TJ
  long long ipt;  // items per tile
};
__host__ __device__ __forceinline__ StagedGeom staged_geom(int ng, int ti) {
  StagedGeom g;
  g.ti = ti;
  g.tj = 2 * ng / ti;
  int x = g.ti, y = g.tj;  // gcd
  while (y) {
    const int r = x % y;
    x = y;
    y = r;
  }
  g.ts = g.ti / x * g.tj;
  g.jpt = g.ts / g.tj;
  g.ipt = (long long)(g.ts / g.ti) * g.jpt;
  return g;
}

// Item w -> (i0, j0).  Triangle: tile x = w / ipt in band order, item k =
// w % ipt at row k / jpt, column k % jpt of the tile's items.  Rectangle:
// column block w / ceil(n_query / TI), query block w % that.
__host__ __device__ __forceinline__ void staged_decode(const PairArgs &a, const StagedGeom &gm, long long w,
                                                       long long &i0, long long &j0) {
  if (a.rect) {
    const long long nqb = (a.n_query + gm.ti - 1) / gm.ti;
    const long long blk = (w < 0x7fffffffLL && nqb < 0x7fffffffLL)
                              ? (long long)((unsigned)w / (unsigned)nqb) : w / nqb;
    i0 = (w - blk * nqb) * gm.ti;
    j0 = a.col_begin + blk * gm.tj;
    return;
  }
  const long long nb = (a.n_events + gm.ts - 1) / gm.ts;
  // 32-bit division when it fits (a 64-bit one is a long software routine)
  const long long x = (w < 0x7fffffffLL) ? (long long)((unsigned)w / (unsigned)gm.ipt) : w / gm.ipt;
  const int k = (int)(w - x * gm.ipt);
  long long bi, bj;
  band_tile(x, nb, a.band_tiles, bi, bj);
  i0 = bi * gm.ts + (long long)(k / gm.jpt) * gm.ti;
  j0 = bj * gm.ts + (long long)(k % gm.jpt) * gm.tj;
}

// Producer side: bounded wait; on running out it raises the abort and error flags.
__device__ __forceinline__ bool producer_wait(uint64_t *bar, uint32_t parity, uint32_t limit,
                                              volatile int *abort_flag, int *err) {
  if (tc::mbar_wait(bar, parity, limit)) return true;
  *abort_flag = 1;
  if (err) atomicExch(err, 1);
  return false;
}

// FFT-thread side: true once the phase completed; false only when it has not
// and the producer has aborted (so it never will).  The phase is tested
// before the flag: a thread never gives up on a unit that has landed.
__device__ __forceinline__ bool consumer_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  for (uint32_t it = 0;; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return tc::mbar_try_wait(bar, parity);
    if (it > 64) __nanosleep(it > 4096 ? 256 : 32);
  }
}


// Default poll limit of the producer's waits (with back-off: seconds).
constexpr uint32_t kStagedWaitPolls = 1u << 24;

// Cursor of the next unit to stage (shared memory, used by the producer only).
struct StagedCursor {
  long long w, i, j0;
  int c, r;
  unsigned seq;  // items decoded so far by this CTA
};
struct StagedItem {
  long long i, j0;
};

template <int P, int NWARP, int RU, int ST>
__device__ __forceinline__ void staged_issue(const PairArgs &a, const StagedGeom &gm, const CUtensorMap *imap,
                                             const CUtensorMap *jmap, StagedCursor *cur, StagedItem *items,
                                             unsigned char *dst, uint64_t *full, uint32_t sub_bytes) {
  using SH = Staged<P, NWARP, RU, ST>;
  using ST_T = typename SpecT<ST>::T;
  constexpr int S = SH::S;
  const uint32_t ibytes = (uint32_t)(gm.ti * S * sizeof(ST_T));
  const int C = spectrum_rows(a);
  const int c = cur->c, r = cur->r;
  tc::mbar_arrive_expect_tx(full, RU * sub_bytes);
#pragma unroll
  for (int h = 0; h < RU; ++h) {
    unsigned char *d = dst + h * sub_bytes;
    tc::tma_load_3d(d, imap, (r + h) * S, c, (int)cur->i, full);
    tc::tma_load_3d(d + ibytes, jmap, (r + h) * S, c, (int)cur->j0, full);
  }
  cur->r += RU;
  if (cur->r == 8) {
    cur->r = 0;
    if (++cur->c == C) {
      cur->c = 0;
      cur->w += gridDim.x;
      if (cur->w < a.couple_end) {
        staged_decode(a, gm, cur->w, cur->i, cur->j0);
        // published before the item's first unit is armed: that arrive
        // releases it to the FFT threads that wait on the unit
        items[++cur->seq % kItemRing] = StagedItem{cur->i, cur->j0};
      }
    }
  }
}

// KTI: the item's i events TI as a compile-time constant (0: the runtime
// PairArgs::item_i).  The default geometry of each CTA shape runs with KTI
// set: its unit strides and row offsets become immediates, a few integer
// instructions less per staged bin (overlap-save Q=512 x 4: 840 -> 889 M
// pairs/s).
template <int P, int NWARP, int RU, int ST, int KTI>
__global__ void __launch_bounds__(NWARP * 32 + 32, 1)
    staged_pair_kernel(const PairArgs a, const __grid_constant__ CUtensorMap jmap,
                       const __grid_constant__ CUtensorMap imap) {
  using SH = Staged<P, NWARP, RU, ST>;
  using ST_T = typename SpecT<ST>::T;
  constexpr int G = SH::G, S = SH::S, NW = SH::NW;
  constexpr int KTJ = KTI ? 2 * SH::NG / KTI : 0;
  static_assert(KTI == 0 || (SH::NG % KTI == 0 && KTJ % 2 == 0), "staged_pair_kernel: KTI must divide the groups");
  // per-item constants: compile-time with KTI, else from the kernel
  // parameters (PairArgs::item_*), not registers held across the FFT
  const uint32_t UNIT = KTI ? (uint32_t)(RU * (KTI + KTJ) * S * sizeof(ST_T)) : a.unit_bytes;

  extern __shared__ __align__(128) unsigned char smem[];
  float2 *bufs = reinterpret_cast<float2 *>(smem);
  unsigned *reds = reinterpret_cast<unsigned *>(smem + SH::EX_BYTES);
  StagedCursor *cur = reinterpret_cast<StagedCursor *>(smem + SH::PROD_OFF);
  volatile int *s_abort = reinterpret_cast<volatile int *>(smem + SH::PROD_OFF + 48);
  uint64_t *probe = reinterpret_cast<uint64_t *>(smem + SH::PROD_OFF + 56);  // never completed
  StagedItem *items = reinterpret_cast<StagedItem *>(smem + SH::ITEMS_OFF);
  unsigned char *ring = smem + SH::RING_OFF;
  const int K = a.ring;
  uint64_t *full = reinterpret_cast<uint64_t *>(ring + (size_t)K * UNIT);
  uint64_t *empty = full + K;
  int *hist = reinterpret_cast<int *>(empty + K);
  const bool smem_hist = a.n_hist > 0 && a.n_hist <= kStagedHistMax;
  const int C = spectrum_rows(a);  // spectrum rows per event: channels, times blocks in the overlap-save form
  const long long N = a.n_events;

  if (threadIdx.x == 0) {
    *s_abort = 0;
    tc::mbar_init(probe, 1);
    for (int k = 0; k < K; ++k) {
      tc::mbar_init(&full[k], 1);
      tc::mbar_init(&empty[k], SH::CONSUMERS);
    }
    tc::fence_mbarrier_init();
    tc::fence_proxy_async_smem();
  }
  if (smem_hist)
    for (int h = threadIdx.x; h < 2 * a.n_hist; h += blockDim.x) hist[h] = 0;
  __syncthreads();

  if (threadIdx.x >= SH::CONSUMERS) {
    // ------------------------------------------------------------ producer
    if (threadIdx.x == SH::CONSUMERS) {
      const StagedGeom gm = staged_geom(SH::NG, KTI ? KTI : a.item_i);
      const uint32_t sub_bytes = UNIT / RU;
      const long long units_total =
          ((a.couple_end - a.couple_begin - blockIdx.x + gridDim.x - 1) / gridDim.x) * C * (8 / RU);
      cur->w = a.couple_begin + blockIdx.x;
      cur->c = 0;
      cur->r = 0;
      staged_decode(a, gm, cur->w, cur->i, cur->j0);
      cur->seq = 0;
      items[0] = StagedItem{cur->i, cur->j0};
      int slot = 0;
      uint32_t phase = 0;
      const uint32_t limit = a.wait_limit ? a.wait_limit : kStagedWaitPolls;
      long long issued = 0;
      // the test probe: a wait that nothing completes runs out before any issue
      const bool probed = a.wait_probe && !producer_wait(probe, 0, limit, s_abort, a.error_flag);
      for (long long u = 0; u < units_total && !probed; ++u) {
        if (u >= K && !producer_wait(&empty[slot], phase ^ 1u, limit, s_abort, a.error_flag)) break;
        staged_issue<P, NWARP, RU, ST>(a, gm, &imap, &jmap, cur, items, ring + (size_t)slot * UNIT, &full[slot],
                                       sub_bytes);
        ++issued;
        if (++slot == K) {
          slot = 0;
          phase ^= 1u;
        }
      }
      // drain: the last arming of every slot has landed before the CTA may
      // exit (immediate when the FFT threads consumed everything)
      for (int k = 0; k < K && k < issued; ++k) {
        const long long last = k + ((issued - 1 - k) / K) * K;  // last unit issued into slot k
        if (!tc::mbar_wait(&full[k], (uint32_t)((last / K) & 1), kStagedWaitPolls)) {
          *s_abort = 1;
          if (a.error_flag) atomicExch(a.error_flag, 1);
        }
      }
    }
  } else {
    // ---------------------------------------------------------- FFT groups
    const int g = threadIdx.x / G;
    const int t = threadIdx.x % G;
    float2 *buf = bufs + g * SH::EX_LEN;
    unsigned *red = reds + g * NW * 8;
    TwiddleRoots<P, 1> roots;
    roots.load(t, a.twiddles);
    const uint32_t wmask = window_mask<P>(t, a.shift);
    const int ca = (t == 0) ? 0 : t;
    const int cb = (t == 0) ? S / 2 : S - t;
    int slot = 0;
    uint32_t phase = 0;
    unsigned seq = 0;
    for (long long w = a.couple_begin + blockIdx.x; w < a.couple_end; w += gridDim.x, ++seq) {
      // the item's first unit being full also publishes its (i, j0); if it
      // never landed, the entry read below is stale, and nothing indexes
      // memory with it before the group's vote after the unit loop
      bool stop = !consumer_wait(&full[slot], phase, s_abort);
      const StagedItem it = items[seq % kItemRing];
      // the group's i row gi and couple column gc within the item
      const int ti = KTI ? KTI : a.item_i, tjh = KTI ? KTJ / 2 : (a.item_j >> 1);
      const int gi = KTI ? g / (KTJ / 2) : (int)(((unsigned)g * a.item_magic) >> 16), gc = g - gi * tjh;
      const int ri = gi * S, rows = KTI ? KTI + KTJ : a.item_i + a.item_j;
      const long long i = it.i + gi, j0 = it.j0;
      long long ja = j0 + 2 * gc, jb = ja + 1;
      bool live, out_b;
      if (!a.rect) {
        const bool v1 = i < N && ja < N && ja >= i;
        const bool v2 = i < N && jb < N && jb >= i;
        live = v1 || v2;
        out_b = v1 && v2;
        if (!v1) ja = jb;
        if (jb >= N) jb = ja;
      } else {
        live = i < a.n_query && ja - a.col_begin < a.n_cols;
        out_b = jb - a.col_begin < a.n_cols;
        if (!out_b) jb = ja;
      }
      const int ra = (ti + (int)(ja - j0)) * S, rb = (ti + (int)(jb - j0)) * S;  // rows of ja, jb in a chunk
      CoupleAcc y;
      y.zero();
      for (int c = 0; c < C && !stop; ++c) {
#pragma unroll
        for (int rp = 0; rp < 8; rp += RU) {
          if (!consumer_wait(&full[slot], phase, s_abort)) {
            stop = true;
            break;
          }
          const ST_T *u = reinterpret_cast<const ST_T *>(ring + (size_t)slot * UNIT);
#pragma unroll
          for (int h = 0; h < RU; ++h) {
            const ST_T *uh = u + h * (rows * S);
            if (live)
              y.add<ST>(rp + h, uh[ri + ca], uh[ra + ca], uh[rb + ca], uh[ri + cb], uh[ra + cb], uh[rb + cb]);
          }
          tc::mbar_arrive(&empty[slot]);
          if (++slot == K) {
            slot = 0;
            phase ^= 1u;
          }
        }
      }
      // an abort inside the item: the group leaves together, by the vote
      // folded into the inverse FFT's first barrier (or a vote of its own
      // for a group without a pair in this item)
      if (live) {  // uniform over the group
        float2 v[32];
        assemble_couple(y, t, v);
        if constexpr (SH::SPLIT_EX)
          inverse_fft_group_split<P>(v, buf, t, g, ca, cb, roots, &stop);
        else
          inverse_fft_group<P>(v, buf, t, g, ca, cb, a.twiddles, roots, &stop);
        if (stop) break;
        scan_and_write<P, kLivenessVote<P, ST>, kScanRowSkip<P, ST>>(a, v, i, ja, i, jb, out_b, t, g, red, hist, smem_hist, wmask, buf);
      } else if (group_sync_any<G>(g, stop)) {
        break;
      }
    }
  }
  __syncthreads();
  if (smem_hist) {
    for (int h = threadIdx.x; h < a.n_hist; h += blockDim.x) {
      if (hist[h]) atomicAdd(&a.max_hist[h], hist[h]);
      if (hist[a.n_hist + h]) atomicAdd(&a.min_hist[h], hist[a.n_hist + h]);
    }
  }
}

// ------------------------------------------------------------------ host
static bool staged_disabled() {
  const char *e = getenv("SEISMIC_PAIR_KERNEL");
  return e && strcmp(e, "direct") == 0;
}

constexpr int kStagedWarps = 12;  // FFT warps per CTA, plus the producer warp

// The widest FFT-warp count whose CTA (plus the producer warp) still gets 128
// registers a thread: at most 4 warps per SM sub-partition, i.e. 16 warps,
// in whole groups of P/32 threads.
constexpr int staged_wide_warps(int P) { return P >= 4096 ? 12 : (P == 2048 ? 14 : 15); }

// CTA shape of a launch: FFT warps per CTA and chunks per ring slot.  In
// order: a shape the autotuner forces while timing, SEISMIC_STAGED_WARPS
// ("12", "wide") / SEISMIC_STAGED_RU ("2", "4"), the tuner's cached choice
// for exactly (P, spectrum rows), else the built-in rule: the wide CTA (the
// most FFT warps that keep 128 registers a thread) with 4-chunk slots.
// Measured with items of TI x TJ events, FP32, M pairs/s, 12 warps / wide:
// overlap-save Q=512 x 4 rows 710 / 825, Q=1024 x 2 rows 451 / 516, P=512
// one channel 977 / 1128, P=1024 523 / 585, P=1024 three channels 380 /
// 469, P=2048 219 / 274, P=2048 three channels 192 / 195 (P=4096: the same
// CTA).  Half-precision spectra always take 4-chunk slots; an FP32 launch
// whose item rows leave no room for two 4-chunk slots takes 2
// (launch_staged_p).
struct StagedShape {
  int nwarp, ru;
};
static StagedShape staged_shape(int P, const PairArgs &a) {
  const int rows = spectrum_rows(a);
  int w = a.staged_warps, ru = a.staged_ru;
  if (!w) {
    const char *e = getenv("SEISMIC_STAGED_WARPS");
    if (e && strcmp(e, "wide") == 0) w = staged_wide_warps(P);
    if (e && strcmp(e, "12") == 0) w = kStagedWarps;
  }
  if (!ru) {
    const char *e = getenv("SEISMIC_STAGED_RU");
    if (e && strcmp(e, "2") == 0) ru = 2;
    if (e && strcmp(e, "4") == 0) ru = 4;
  }
  int tw = 0, tru = 0;
  if ((!w || !ru) && tune_staged_lookup(P, rows, &tw, &tru)) {
    if (!w) w = tw;
    if (!ru) ru = tru;
  }
  if (!w) w = staged_wide_warps(P);
  w = (w == kStagedWarps) ? kStagedWarps : staged_wide_warps(P);
  ru = (a.stype != 0 || ru != 2) ? 4 : 2;
  return StagedShape{w, ru};
}

bool staged_enabled();

// i events per item (TI, a divisor of the NG groups): SEISMIC_STAGED_TI if it
// divides NG, else the TI of least estimated time per pair,
//   (query rows covered / query rows) x (1 + 0.18 (TI + TJ) / (2 NG)):
// the first factor is the FFT work of groups left without a query on the
// rectangle (1 on the triangle), the second the staging of TI + TJ rows per
// 2 NG pairs (one i per item, 49 rows per 48 pairs, measured 13 % slower than
// 14 rows per 48 on the overlap-save form).  The triangle takes the fewest
// rows; a one-query request keeps TI = 1.
static int staged_item_rows(int ng, const PairArgs &a) {
  if (const char *e = getenv("SEISMIC_STAGED_TI")) {
    const int v = atoi(e);
    if (v >= 1 && v <= ng && ng % v == 0) return v;
  }
  int best = 1;
  double best_cost = 0.0;
  for (int d = 1; d <= ng; ++d) {
    if (ng % d) continue;
    const double rows = d + 2.0 * ng / d;
    const double pad = (a.rect && a.n_query > 0) ? (double)((a.n_query + d - 1) / d * d) / (double)a.n_query : 1.0;
    const double cost = pad * (1.0 + 0.18 * rows / (2.0 * ng));
    if (d == 1 || cost < best_cost) {
      best = d;
      best_cost = cost;
    }
  }
  return best;
}

// Ring slots of a launch: the shared memory left beside the FFT exchange
// buffers (and room for the largest shared histogram), in slots of RU chunks
// of the item's TI + TJ rows; at most kStagedRingMax.
template <int P, int NWARP, int RU, int ST> static int staged_ring_slots(const PairArgs &a, size_t *unit_bytes) {
  using SH = Staged<P, NWARP, RU, ST>;
  const StagedGeom gm = staged_geom(SH::NG, staged_item_rows(SH::NG, a));
  const size_t unit = (size_t)RU * (gm.ti + gm.tj) * SH::S * sizeof(typename SpecT<ST>::T);
  if (unit_bytes) *unit_bytes = unit;
  const size_t hist_reserve = (size_t)2 * kStagedHistMax * sizeof(int);
  const int K = (int)((kStagedSmemBudget - SH::RING_OFF - hist_reserve) / (unit + 2 * sizeof(uint64_t)));
  return K > kStagedRingMax ? kStagedRingMax : K;
}

template <int P, int NWARP, int RU, int ST, int KTI>
static cudaError_t launch_staged_t(const PairArgs &a0, int sm_count, cudaStream_t s) {
  using SH = Staged<P, NWARP, RU, ST>;
  using ST_T = typename SpecT<ST>::T;
  PairArgs a = a0;
  a.item_i = staged_item_rows(SH::NG, a);
  if (KTI && a.item_i != KTI) return cudaErrorInvalidConfiguration;  // the caller picks KTI from this rule
  const StagedGeom gm = staged_geom(SH::NG, a.item_i);
  a.item_j = gm.tj;
  // g / (TJ/2) = (g * ceil(2^16 / (TJ/2))) >> 16 exactly while g * TJ/2 < 2^16
  a.item_magic = (unsigned)((65536 + gm.tj / 2 - 1) / (gm.tj / 2));
  size_t unit = 0;
  const int K = staged_ring_slots<P, NWARP, RU, ST>(a, &unit);
  a.unit_bytes = (unsigned)unit;
  if (K < 2) return cudaErrorInvalidConfiguration;
  a.ring = K;
  const size_t hist_bytes = (a.n_hist > 0 && a.n_hist <= kStagedHistMax) ? (size_t)2 * a.n_hist * sizeof(int) : 0;
  const size_t smem = SH::RING_OFF + (size_t)K * unit + (size_t)2 * K * sizeof(uint64_t) + hist_bytes;
  {
    cudaError_t e =
        ensure_dynamic_smem((const void *)staged_pair_kernel<P, NWARP, RU, ST, KTI>, (int)kStagedSmemBudget);
    if (e != cudaSuccess) return e;
  }
  a.band_tiles = l2_band_tiles(spectrum_rows(a), P, (int)sizeof(ST_T), gm.ts);
  a.wait_limit = device_wait_polls();
  a.wait_probe = device_wait_probe();

  // Tensor maps of the j and the i spectra: dims {P/2 bins, C spectrum rows,
  // events}, boxes {S bins, 1 row, TJ or TI events}.
  CUtensorMap map, imap;
  const void *spec_i = a.spectra_i ? a.spectra_i : (a.rect ? a.spectra_q : a.spectra);
  const long long n_i = a.rect ? a.n_query : a.n_events;
  const cuuint64_t strides[2] = {(cuuint64_t)(P / 2) * sizeof(ST_T),
                                 (cuuint64_t)spectrum_rows(a) * (P / 2) * sizeof(ST_T)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = sizeof(ST_T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  for (int side = 0; side < 2; ++side) {
    const cuuint64_t dims[3] = {(cuuint64_t)(P / 2), (cuuint64_t)spectrum_rows(a),
                                (cuuint64_t)(side == 0 ? a.n_events : n_i)};
    const cuuint32_t box[3] = {(cuuint32_t)SH::S, 1u, (cuuint32_t)(side == 0 ? gm.tj : gm.ti)};
    if (tensor_map_encoder()(side == 0 ? &map : &imap, dt, 3, const_cast<void *>(side == 0 ? a.spectra : spec_i),
                             dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  const long long items = a.couple_end - a.couple_begin;
  if (items <= 0) return cudaSuccess;
  const int grid = (int)(items < sm_count ? items : sm_count);
  staged_pair_kernel<P, NWARP, RU, ST, KTI><<<grid, SH::THREADS, smem, s>>>(a, map, imap);
  return cudaGetLastError();
}

// The triangle's item geometry for ng groups: the fewest staged rows TI +
// 2 ng / TI (smallest TI on ties), as staged_item_rows picks it.
constexpr int default_item_rows(int ng) {
  int best = 1, best_rows = 1 + 2 * ng;
  for (int d = 2; d <= ng; ++d)
    if (ng % d == 0 && d + 2 * ng / d < best_rows) {
      best = d;
      best_rows = d + 2 * ng / d;
    }
  return best;
}

template <int P> static cudaError_t launch_staged_p(const PairArgs &a, int sm_count, cudaStream_t s) {
  const StagedShape sh = staged_shape(P, a);
  constexpr int WW = staged_wide_warps(P);
  constexpr int KT = default_item_rows(WW * 32 / (P / 32));
  const bool wide = sh.nwarp == WW;
  // the default CTA with its default item geometry: the compile-time form
  const bool ct = wide && staged_item_rows(WW * 32 / (P / 32), a) == KT;
  switch (a.stype) {
    case 0:
      if (wide) {
        if (sh.ru == 4 && staged_ring_slots<P, WW, 4, 0>(a, nullptr) >= 2)
          return ct ? launch_staged_t<P, WW, 4, 0, KT>(a, sm_count, s) : launch_staged_t<P, WW, 4, 0, 0>(a, sm_count, s);
        return launch_staged_t<P, WW, 2, 0, 0>(a, sm_count, s);
      }
      return (sh.ru == 4 && staged_ring_slots<P, kStagedWarps, 4, 0>(a, nullptr) >= 2)
                 ? launch_staged_t<P, kStagedWarps, 4, 0, 0>(a, sm_count, s)
                 : launch_staged_t<P, kStagedWarps, 2, 0, 0>(a, sm_count, s);
    case 1:
      if (wide)
        return ct ? launch_staged_t<P, WW, 4, 1, KT>(a, sm_count, s) : launch_staged_t<P, WW, 4, 1, 0>(a, sm_count, s);
      return launch_staged_t<P, kStagedWarps, 4, 1, 0>(a, sm_count, s);
    case 2:
      if (wide)
        return ct ? launch_staged_t<P, WW, 4, 2, KT>(a, sm_count, s) : launch_staged_t<P, WW, 4, 2, 0>(a, sm_count, s);
      return launch_staged_t<P, kStagedWarps, 4, 2, 0>(a, sm_count, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
