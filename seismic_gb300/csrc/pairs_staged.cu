// Kernels (b) + (c), staged form: the pair-tile kernel with its spectra
// staged into shared memory by TMA.  Same results as the direct form
// (pairs.cu); replaces the same reference code:
//   ElementWiseMultiplication  Correlation_in_OMP/correlation_c.cpp:188-193
//   inverseFFT                 Correlation_in_OMP/correlation_c.cpp:58-137
//   the dynamic row loop       Correlation_in_OMP/correlation_c.cpp:251-293
//
// Work item = one event i and a block of T = 2 NG consecutive events
// j0 .. j0+T-1; group g of the CTA's NG FFT groups takes the couple
// (i; j0+2g, j0+2g+1) -- the same couples as the direct form, so both forms
// give bit-identical results.  The items of the upper triangle are square
// tiles of T x T events (T items per tile, one per i), walked in row bands
// of `band_tiles` tile rows so the i spectra of a band stay in L2 while
// every column to its right passes over it once (and a band's outputs are
// contiguous packed rows); the rectangle (query x catalog) walks column
// blocks, all queries per block.
//
// Pipeline.  Each item's spectra are cut into units (channel c, chunk r):
// bins [r S, (r+1) S) of row i and of the T rows j0..j0+T-1, exactly the
// bins ca + r S and cb + r S every FFT thread reads at step r
// (pair_core.cuh).  A producer warp (one elected thread) streams units into
// a ring of K shared-memory slots: a 1-D bulk copy for row i's chunk and one
// 3-D TMA box {S bins, 1 channel, T events} for the j rows (rows past the
// catalog are zero-filled by the TMA unit), completing on the slot's `full`
// mbarrier; the FFT warps conj-multiply from the slot and release it on its
// `empty` mbarrier.  While the groups run their inverse FFTs the producer
// fills the ring with the next item's first units, so spectra reads leave
// the critical path.  Row i is staged once per unit for all NG groups:
// 1 + T rows per T pairs instead of 3 rows per 2.
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

template <int P, int NWARP, int RU> struct Staged {  // RU: chunks r per ring slot
  static constexpr int G = P / 32;
  static constexpr int NG = NWARP * 32 / G;  // FFT groups per CTA
  static constexpr int T = 2 * NG;           // j events per item = tile side; T items per tile
  static constexpr int ROWS = 1 + T;         // staged rows per unit: i, j0 .. j0+T-1
  static constexpr int S = P / 16;
  static constexpr int NW = (G + 31) / 32;
  static constexpr int CONSUMERS = NWARP * 32;  // FFT threads
  static constexpr int THREADS = CONSUMERS + 32;  // + the producer warp
  static constexpr size_t EX_BYTES = (size_t)NG * padded_len<P>() * sizeof(float2);
  static constexpr size_t RED_BYTES = (size_t)NG * NW * 8 * sizeof(unsigned);
  static constexpr size_t PROD_OFF = (EX_BYTES + RED_BYTES + 15) / 16 * 16;
  // producer area: cursor (48 B), abort flag (+48), probe mbarrier (+56),
  // item ring of kItemRing (i, j0)
  static constexpr size_t ITEMS_OFF = PROD_OFF + 64;
  static constexpr size_t RING_OFF = (ITEMS_OFF + kItemRing * 16 + 127) / 128 * 128;
  // one chunk r of every staged row, and a ring slot of RU chunks
  template <int ST> static constexpr size_t sub_bytes() { return (size_t)ROWS * S * sizeof(typename SpecT<ST>::T); }
  template <int ST> static constexpr size_t unit_bytes() { return RU * sub_bytes<ST>(); }
};

// Item w -> (i, j0).  Triangle: tile x = w / T in band order, i = bi T + w % T.
__host__ __device__ __forceinline__ void staged_decode(const PairArgs &a, int T, long long w, long long &i,
                                                       long long &j0) {
  if (a.rect) {
    const long long blk = (w < 0x7fffffffLL && a.n_query < 0x7fffffffLL)
                              ? (long long)((unsigned)w / (unsigned)a.n_query) : w / a.n_query;
    i = w - blk * a.n_query;
    j0 = a.col_begin + blk * T;
    return;
  }
  const long long nb = (a.n_events + T - 1) / T;
  const long long x = w / T;
  long long bi, bj;
  band_tile(x, nb, a.band_tiles, bi, bj);
  i = bi * T + (w - x * T);
  j0 = bj * T;
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
__device__ __forceinline__ void staged_issue(const PairArgs &a, const CUtensorMap *jmap, StagedCursor *cur,
                                             StagedItem *items, unsigned char *dst, uint64_t *full) {
  using SH = Staged<P, NWARP, RU>;
  using ST_T = typename SpecT<ST>::T;
  constexpr int S = SH::S, H = P / 2;
  constexpr uint32_t CHUNK = (uint32_t)(S * sizeof(ST_T));
  const int C = spectrum_rows(a);
  const ST_T *spec_i = reinterpret_cast<const ST_T *>(a.spectra_i ? a.spectra_i : (a.rect ? a.spectra_q : a.spectra));
  const long long n_i = a.rect ? a.n_query : a.n_events;
  const long long i = cur->i < n_i ? cur->i : n_i - 1;  // ragged last tile row: staged but unused
  const int c = cur->c, r = cur->r;
  tc::mbar_arrive_expect_tx(full, (uint32_t)SH::template unit_bytes<ST>());
#pragma unroll
  for (int h = 0; h < RU; ++h) {
    unsigned char *d = dst + h * SH::template sub_bytes<ST>();
    tc::bulk_load(d, spec_i + (i * C + c) * (long long)H + (r + h) * S, CHUNK, full);
    tc::tma_load_3d(d + CHUNK, jmap, (r + h) * S, c, (int)cur->j0, full);
  }
  cur->r += RU;
  if (cur->r == 8) {
    cur->r = 0;
    if (++cur->c == C) {
      cur->c = 0;
      cur->w += gridDim.x;
      if (cur->w < a.couple_end) {
        staged_decode(a, SH::T, cur->w, cur->i, cur->j0);
        // published before the item's first unit is armed: that arrive
        // releases it to the FFT threads that wait on the unit
        items[++cur->seq % kItemRing] = StagedItem{cur->i, cur->j0};
      }
    }
  }
}

template <int P, int NWARP, int RU, int ST>
__global__ void __launch_bounds__(NWARP * 32 + 32, 1)
    staged_pair_kernel(const PairArgs a, const __grid_constant__ CUtensorMap jmap) {
  using SH = Staged<P, NWARP, RU>;
  using ST_T = typename SpecT<ST>::T;
  constexpr int G = SH::G, T = SH::T, S = SH::S, NW = SH::NW;
  constexpr uint32_t UNIT = (uint32_t)SH::template unit_bytes<ST>();

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
      const long long units_total =
          ((a.couple_end - a.couple_begin - blockIdx.x + gridDim.x - 1) / gridDim.x) * C * (8 / RU);
      cur->w = a.couple_begin + blockIdx.x;
      cur->c = 0;
      cur->r = 0;
      staged_decode(a, T, cur->w, cur->i, cur->j0);
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
        staged_issue<P, NWARP, RU, ST>(a, &jmap, cur, items, ring + (size_t)slot * UNIT, &full[slot]);
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
    float2 *buf = bufs + g * padded_len<P>();
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
      const long long i = it.i, j0 = it.j0;
      long long ja = j0 + 2 * g, jb = ja + 1;
      bool live, out_b;
      if (!a.rect) {
        const bool v1 = i < N && ja < N && ja >= i;
        const bool v2 = i < N && jb < N && jb >= i;
        live = v1 || v2;
        out_b = v1 && v2;
        if (!v1) ja = jb;
        if (jb >= N) jb = ja;
      } else {
        live = ja - a.col_begin < a.n_cols;
        out_b = jb - a.col_begin < a.n_cols;
        if (!out_b) jb = ja;
      }
      const int ra = (1 + (int)(ja - j0)) * S, rb = (1 + (int)(jb - j0)) * S;  // rows of ja, jb in a unit
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
            const ST_T *uh = u + h * (SH::ROWS * S);
            if (live) y.add<ST>(rp + h, uh[ca], uh[ra + ca], uh[rb + ca], uh[cb], uh[ra + cb], uh[rb + cb]);
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
        inverse_fft_group<P>(v, buf, t, g, ca, cb, a.twiddles, roots, &stop);
        if (stop) break;
        scan_and_write<P>(a, v, i, ja, i, jb, out_b, t, g, red, hist, smem_hist, wmask);
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
// order: a shape the autotuner forces while timing, SEISMIC_STAGED_WARPS /
// SEISMIC_STAGED_RU, the tuner's cached choice for exactly (P, spectrum
// rows), else the built-in rule: the wide CTA (more FFT warps, a smaller
// ring) where one spectrum row's item fits it -- one channel at P = 2048
// (FP32 spectra 263 vs 230 M pairs/s measured, FP16 256 vs 233, BF16 255 vs
// 237; with three channels 175 vs 184) -- and 4-chunk slots otherwise.  The
// wide FP32 CTA has room for 2-chunk slots only; half-precision spectra
// always take 4.
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
  }
  int tw = 0, tru = 0;
  if ((!w || !ru) && tune_staged_lookup(P, rows, &tw, &tru)) {
    if (!w) w = tw;
    if (!ru) ru = tru;
  }
  if (!w) w = (P == 2048 && rows == 1) ? staged_wide_warps(P) : kStagedWarps;
  w = (w == kStagedWarps) ? kStagedWarps : staged_wide_warps(P);
  if (a.stype != 0) ru = 4;                       // half spectra: 4-chunk slots
  else if (w != kStagedWarps) ru = 2;             // the wide FP32 CTA: 2-chunk slots
  else ru = (ru == 2) ? 2 : 4;
  return StagedShape{w, ru};
}

// The staged form serves P = 512 .. 4096: there the three rows of a couple
// (3 x C x 4P bytes) outgrow what L1 keeps and the direct form waits on L2
// (measured, staged vs direct M pairs/s: P=512 C=1 973 vs 926, P=1024 C=1
// 549 vs 496, C=3 379 vs 339).  SEISMIC_PAIR_KERNEL=direct forces the direct
// form everywhere.
bool staged_enabled() { return !staged_disabled() && tensor_map_encoder() != nullptr; }

bool staged_supported(int P, const PairArgs &a) {
  if (P < 512 || P > 4096 || staged_disabled()) return false;
  if (a.stype < 0 || a.stype > 2) return false;
  if ((reinterpret_cast<uintptr_t>(a.spectra) & 15u) != 0) return false;
  if (a.rect && (reinterpret_cast<uintptr_t>(a.spectra_q) & 15u) != 0) return false;
  if (a.spectra_i && (reinterpret_cast<uintptr_t>(a.spectra_i) & 15u) != 0) return false;
  return tensor_map_encoder() != nullptr;
}

int staged_tile_side(int P, const PairArgs &a) { return 2 * (staged_shape(P, a).nwarp * 32 / (P / 32)); }

long long staged_items_total(int P, const PairArgs &a) {
  const long long T = staged_tile_side(P, a);
  if (a.rect) return a.n_query * ((a.n_cols + T - 1) / T);
  const long long nb = (a.n_events + T - 1) / T;
  return T * (nb * (nb + 1) / 2);
}

template <int P, int NWARP, int RU, int ST>
static cudaError_t launch_staged_t(const PairArgs &a0, int sm_count, cudaStream_t s) {
  using SH = Staged<P, NWARP, RU>;
  using ST_T = typename SpecT<ST>::T;
  PairArgs a = a0;
  const size_t unit = SH::template unit_bytes<ST>();
  const size_t hist_reserve = (size_t)2 * kStagedHistMax * sizeof(int);
  int K = (int)((kStagedSmemBudget - SH::RING_OFF - hist_reserve) / (unit + 2 * sizeof(uint64_t)));
  if (K > kStagedRingMax) K = kStagedRingMax;
  if (K < 2) return cudaErrorInvalidConfiguration;
  a.ring = K;
  const size_t hist_bytes = (a.n_hist > 0 && a.n_hist <= kStagedHistMax) ? (size_t)2 * a.n_hist * sizeof(int) : 0;
  const size_t smem = SH::RING_OFF + (size_t)K * unit + (size_t)2 * K * sizeof(uint64_t) + hist_bytes;
  {
    cudaError_t e = ensure_dynamic_smem((const void *)staged_pair_kernel<P, NWARP, RU, ST>, (int)kStagedSmemBudget);
    if (e != cudaSuccess) return e;
  }
  a.band_tiles = l2_band_tiles(spectrum_rows(a), P, (int)sizeof(ST_T), SH::T);
  a.wait_limit = device_wait_polls();
  a.wait_probe = device_wait_probe();

  // Tensor map of the j spectra: dims {P/2 bins, C channels, N events},
  // box {S bins, 1 channel, T events}.
  CUtensorMap map;
  const cuuint64_t dims[3] = {(cuuint64_t)(P / 2), (cuuint64_t)spectrum_rows(a), (cuuint64_t)a.n_events};
  const cuuint64_t strides[2] = {(cuuint64_t)(P / 2) * sizeof(ST_T),
                                 (cuuint64_t)spectrum_rows(a) * (P / 2) * sizeof(ST_T)};
  const cuuint32_t box[3] = {(cuuint32_t)SH::S, 1u, (cuuint32_t)SH::T};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = sizeof(ST_T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  if (tensor_map_encoder()(&map, dt, 3, const_cast<void *>(a.spectra), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  const long long items = a.couple_end - a.couple_begin;
  if (items <= 0) return cudaSuccess;
  const int grid = (int)(items < sm_count ? items : sm_count);
  staged_pair_kernel<P, NWARP, RU, ST><<<grid, SH::THREADS, smem, s>>>(a, map);
  return cudaGetLastError();
}

template <int P> static cudaError_t launch_staged_p(const PairArgs &a, int sm_count, cudaStream_t s) {
  const StagedShape sh = staged_shape(P, a);
  const bool wide = sh.nwarp != kStagedWarps;
  switch (a.stype) {
    case 0:
      if (wide) return launch_staged_t<P, staged_wide_warps(P), 2, 0>(a, sm_count, s);
      return sh.ru == 2 ? launch_staged_t<P, kStagedWarps, 2, 0>(a, sm_count, s)
                        : launch_staged_t<P, kStagedWarps, 4, 0>(a, sm_count, s);
    case 1:
      return wide ? launch_staged_t<P, staged_wide_warps(P), 4, 1>(a, sm_count, s)
                  : launch_staged_t<P, kStagedWarps, 4, 1>(a, sm_count, s);
    case 2:
      return wide ? launch_staged_t<P, staged_wide_warps(P), 4, 2>(a, sm_count, s)
                  : launch_staged_t<P, kStagedWarps, 4, 2>(a, sm_count, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_pairs_staged(int P, const PairArgs &a, int sm_count, cudaStream_t s) {
  switch (P) {
    case 512: return launch_staged_p<512>(a, sm_count, s);
    case 1024: return launch_staged_p<1024>(a, sm_count, s);
    case 2048: return launch_staged_p<2048>(a, sm_count, s);
    case 4096: return launch_staged_p<4096>(a, sm_count, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
