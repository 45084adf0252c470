// Kernels (b) + (c): fused pair-tile correlation with an upper-triangle tile
// scheduler (direct-load form; staged_core.cuh holds the TMA-staged form).
//
// Replaces, per pair (i, j >= i) of the packed upper triangle:
//   ElementWiseMultiplication  Correlation_in_OMP/correlation_c.cpp:188-193
//   inverseFFT (c2r + window scan + normalise + histogram + threshold)
//                              Correlation_in_OMP/correlation_c.cpp:58-137
//   the dynamic row loop       Correlation_in_OMP/correlation_c.cpp:251-293
// and the GPU chunk loop EWM_Linear -> cuFFT C2R -> FE_Linear of
// Correlation_in_CUDA/correlation_cuda.cu:409-505, without any lag series
// or product spectrum ever written to global memory.
//
// Work decomposition.  Events are cut into square tiles of `tile` events;
// tiles (bi, bj >= bi) of the upper triangle are enumerated in row bands
// of `band_tiles` tile rows (band_tile; 0 = one band).  A tile holds tile*tile/2 couples (pair_core.cuh); couples
// are dealt to groups of G = P/32 threads round-robin, the groups of one CTA
// taking neighbouring couples of the same tile, whose spectra they read
// straight from global memory (L2).  This form serves every size P and the
// batched launch; staged_core.cuh stages the spectra through shared memory.
#include <algorithm>
#include "pair_core.cuh"

namespace seismic {

long long rect_couples_total(long long n_query, long long n_cols, int tile) {
  const long long cols = (n_cols + 1) / 2;
  const long long chunks = (cols + tile - 1) / tile;
  return chunks * tile * n_query;
}

long long pair_couples_total(long long n_events, int tile) {
  const long long nb = (n_events + tile - 1) / tile;
  return nb * (nb + 1) / 2 * ((long long)tile * tile / 2);
}

int pair_tile_for(int P) { return P <= 2048 ? 8 : (P == 4096 ? 4 : 2); }

template <int P, int ST>
__device__ __forceinline__ void pair_body(const PairArgs &a, long long w_first, long long w_stride, long long w_end,
                                          unsigned char *smem_raw, int *hist, bool smem_hist);

// Shared-memory layout of a 256-thread CTA working at size P: NG exchange
// buffers, NG reduction slots, then the histogram (2 * n_hist ints).
template <int P> __device__ __forceinline__ int *pair_hist_smem(unsigned char *smem_raw) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int NW = (G + 31) / 32;
  return reinterpret_cast<int *>(smem_raw + (size_t)NG * padded_len<P>() * sizeof(float2) +
                                 (size_t)NG * NW * 8 * sizeof(unsigned));
}

// 256 threads (two CTAs per SM), or one FFT group of P/32 threads where that
// is more (P = 16384: 512 threads, 139 KB of exchange buffer, one CTA per SM).
template <int P, int ST>
__global__ void __launch_bounds__((P / 32 > 256 ? P / 32 : 256), (P / 32 > 256 ? 1 : 2)) pair_kernel(PairArgs a) {
  constexpr int NG = (256 / (P / 32)) > 0 ? (256 / (P / 32)) : 1;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  int *hist = pair_hist_smem<P>(smem_raw);
  const bool smem_hist = a.n_hist > 0 && a.n_hist <= kSmemHistMax;
  if (smem_hist) {
    for (int h = threadIdx.x; h < 2 * a.n_hist; h += blockDim.x) hist[h] = 0;
  }
  __syncthreads();
  const int g = threadIdx.x / (P / 32);
  pair_body<P, ST>(a, a.couple_begin + (long long)blockIdx.x * NG + g, (long long)gridDim.x * NG, a.couple_end,
                   smem_raw, hist, smem_hist);
  if (smem_hist) {
    __syncthreads();
    for (int h = threadIdx.x; h < a.n_hist; h += blockDim.x) {
      if (hist[h]) atomicAdd(&a.max_hist[h], hist[h]);
      if (hist[a.n_hist + h]) atomicAdd(&a.min_hist[h], hist[a.n_hist + h]);
    }
  }
}

// Couples w = w_first, w_first + w_stride, ... < w_end of the triangle of
// `a`, processed by this thread's group (G = P/32 threads).  `hist` is the
// CTA's shared histogram (2 * n_hist ints) when smem_hist, else unused.
template <int P, int ST>
__device__ __forceinline__ void pair_body(const PairArgs &a, long long w_first, long long w_stride, long long w_end,
                                          unsigned char *smem_raw, int *hist, bool smem_hist) {
  using ST_T = typename SpecT<ST>::T;
  const ST_T *spectra = reinterpret_cast<const ST_T *>(a.spectra);
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int S = P / 16;
  constexpr int H = P / 2;
  constexpr int NW = (G + 31) / 32;
  float2 *bufs = reinterpret_cast<float2 *>(smem_raw);
  unsigned *reds = reinterpret_cast<unsigned *>(bufs + NG * padded_len<P>());
  const int g = threadIdx.x / G;
  const int t = threadIdx.x % G;
  float2 *buf = bufs + g * padded_len<P>();
  unsigned *red = reds + g * NW * 8;

  const long long N = a.n_events;
  const int C = a.n_channels;
  const long long T = a.tile;
  const long long nb = (N + T - 1) / T;
  const long long cpt = T * T / 2;
  // Twiddle roots of the radix-16 passes depend only on the thread: load once.
  TwiddleRoots<P, 1> roots;
  roots.load(t, a.twiddles);
  const uint32_t wmask = window_mask<P>(t, a.shift);

  const int ca = (t == 0) ? 0 : t;
  const int cb = (t == 0) ? S / 2 : S - t;

  const ST_T *spectra_i = a.rect ? reinterpret_cast<const ST_T *>(a.spectra_q) : spectra;
  for (long long w = w_first; w < w_end; w += w_stride) {
    long long i, ja, jb;
    bool out_b;
    if (!a.rect) {
      // 32-bit division where it fits (a 64-bit one is a long software routine)
      const long long tile = w < 0x7fffffffLL ? (long long)((unsigned)w / (unsigned)cpt) : w / cpt;
      const int lc2 = (int)(2 * (w - tile * cpt));
      long long bi, bj;
      band_tile(tile, nb, a.band_tiles, bi, bj);
      const long long ii = lc2 / (int)T, jj = lc2 - (int)ii * (int)T;
      i = bi * T + ii;
      const long long j1 = bj * T + jj, j2 = j1 + 1;
      const bool v1 = i < N && j1 < N && j1 >= i;
      const bool v2 = i < N && j2 < N && j2 >= i;
      if (!v1 && !v2) continue;  // uniform over the group
      ja = v1 ? j1 : j2;
      jb = j2 < N ? j2 : ja;
      out_b = v1 && v2;
    } else {
      // chunk of T couple-columns x all queries; j are subset columns
      const long long per_chunk = a.n_query * T;
      const long long chunk = (w < 0x7fffffffLL && per_chunk < 0x7fffffffLL)
                                  ? (long long)((unsigned)w / (unsigned)per_chunk) : w / per_chunk;
      const long long r = w - chunk * per_chunk;
      i = r < 0x7fffffffLL ? (long long)((unsigned)r / (unsigned)T) : r / T;
      const long long j1 = 2 * (chunk * T + (r - i * T)), j2 = j1 + 1;
      if (j1 >= a.n_cols) continue;  // uniform over the group
      out_b = j2 < a.n_cols;
      ja = a.col_begin + j1;          // catalog event indices
      jb = out_b ? ja + 1 : ja;
    }

    // ---- conj products, accumulated over channels, for this thread's 16 bins
    CoupleAcc y;
    y.zero();
    for (int c = 0; c < C; ++c) {
      const ST_T *Xi = spectra_i + (i * C + c) * (long long)H;
      const ST_T *X1 = spectra + (ja * C + c) * (long long)H;
      const ST_T *X2 = spectra + (jb * C + c) * (long long)H;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int ka = ca + r * S, kb = cb + r * S;
        y.add<ST>(r, __ldg(Xi + ka), __ldg(X1 + ka), __ldg(X2 + ka), __ldg(Xi + kb), __ldg(X1 + kb),
                  __ldg(X2 + kb));
      }
    }
    float2 v[32];
    assemble_couple(y, t, v);
    inverse_fft_group<P>(v, buf, t, g, ca, cb, a.twiddles, roots);
    scan_and_write<P, kLivenessVote<P, ST>, kScanRowSkip<P, ST>>(a, v, i, ja, i, jb, out_b, t, g, red, hist, smem_hist, wmask, buf);
  }
}

// ----------------------------------------------------------- batched form
// One CTA-sized item of one catalog: the CTA's groups take its couples.
// Inlined: as a call per item (which moves the mixed-size kernel's 1,000
// bytes of register spills out of it) the batched launch ran 9 % slower.
template <int P>
__device__ __forceinline__ void batched_pair_item(const PairArgs &a, long long begin, long long end,
                                                  unsigned char *smem_raw) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  int *hist = pair_hist_smem<P>(smem_raw);
  const bool smem_hist = a.n_hist > 0 && a.n_hist <= kSmemHistMax;
  if (smem_hist)
    for (int h = threadIdx.x; h < 2 * a.n_hist; h += blockDim.x) hist[h] = 0;
  __syncthreads();
  pair_body<P, 0>(a, begin + threadIdx.x / G, NG, end, smem_raw, hist, smem_hist);
  __syncthreads();
  if (smem_hist) {
    for (int h = threadIdx.x; h < a.n_hist; h += blockDim.x) {
      if (hist[h]) atomicAdd(&a.max_hist[h], hist[h]);
      if (hist[a.n_hist + h]) atomicAdd(&a.min_hist[h], hist[a.n_hist + h]);
    }
  }
}

// Persistent over every catalog of transform size P: CTAs pull work items
// from a global counter until the list is exhausted; items are pre-sorted by
// cost (largest first).  One such launch per size present in a batch; the
// batch graph runs them as concurrent branches.
template <int P>
__global__ void __launch_bounds__(256, 2)
    batched_pair_kernel(const BatchCatalog *__restrict__ cats, const BatchItem *__restrict__ items, long long n_items,
                        unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ BatchItem s_w;
  __shared__ __align__(16) PairArgs s_args;  // the item's catalog descriptor, read from shared memory
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = (long long)atomicAdd(counter, 1ULL);
      if (s_item < n_items) {
        s_w = items[s_item];
        s_args = cats[s_w.cat].pairs;
      }
    }
    __syncthreads();
    const long long it = s_item;
    if (it >= n_items) break;
    batched_pair_item<P>(s_args, s_w.begin, s_w.end, smem_raw);
    __syncthreads();  // s_item and the shared buffers are reused by the next item
  }
}

// Persistent over every catalog of a batch whatever its transform size: the
// item's catalog descriptor names P, and the CTA's 256 threads run that
// size's groups for the item (every size uses 256 threads x 32 values and
// the same shared-memory footprint).  One launch covers the whole batch, and
// the items of all sizes, sorted by cost, balance across the SMs together.
__global__ void __launch_bounds__(256, 2)
    batched_pair_kernel_mixed(const BatchCatalog *__restrict__ cats, const BatchItem *__restrict__ items,
                              long long n_items, unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ BatchItem s_w;
  __shared__ int s_p;
  __shared__ __align__(16) PairArgs s_args;
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = (long long)atomicAdd(counter, 1ULL);
      if (s_item < n_items) {
        s_w = items[s_item];
        s_args = cats[s_w.cat].pairs;
        s_p = cats[s_w.cat].P;
      }
    }
    __syncthreads();
    if (s_item >= n_items) break;
    switch (s_p) {  // uniform over the CTA
      case 64: batched_pair_item<64>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 128: batched_pair_item<128>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 256: batched_pair_item<256>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 512: batched_pair_item<512>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 1024: batched_pair_item<1024>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 2048: batched_pair_item<2048>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 4096: batched_pair_item<4096>(s_args, s_w.begin, s_w.end, smem_raw); break;
      case 8192: batched_pair_item<8192>(s_args, s_w.begin, s_w.end, smem_raw); break;
      default: break;
    }
    __syncthreads();  // s_item and the shared buffers are reused by the next item
  }
}

template <int P> static size_t batched_pair_smem_t(int max_hist) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int NW = (G + 31) / 32;
  size_t s = (size_t)NG * padded_len<P>() * sizeof(float2) + (size_t)NG * NW * 8 * sizeof(unsigned);
  if (max_hist > 0 && max_hist <= kSmemHistMax) s += (size_t)2 * max_hist * sizeof(int);
  return s;
}

template <int P> static int batched_ctas_t(int max_hist) {
  int n = 0;
  ensure_dynamic_smem((const void *)batched_pair_kernel<P>, (int)batched_pair_smem_t<P>(kSmemHistMax));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batched_pair_kernel<P>, 256,
                                                    batched_pair_smem_t<P>(max_hist)) != cudaSuccess)
    n = 1;
  return n > 0 ? n : 1;
}

template <int P>
static cudaError_t launch_batched_t(const BatchCatalog *cats, const BatchItem *items, long long n_items,
                                    unsigned long long *counter, int grid, int max_hist, cudaStream_t s) {
  // the shared-memory attribute was set by batched_pairs_ctas_per_sm during planning,
  // so nothing but the launch happens here (it may be inside a stream capture)
  batched_pair_kernel<P><<<grid, 256, batched_pair_smem_t<P>(max_hist), s>>>(cats, items, n_items, counter);
  return cudaGetLastError();
}

static size_t batched_mixed_smem(int max_hist) {
  return std::max({batched_pair_smem_t<64>(max_hist), batched_pair_smem_t<128>(max_hist),
                   batched_pair_smem_t<256>(max_hist), batched_pair_smem_t<512>(max_hist),
                   batched_pair_smem_t<1024>(max_hist), batched_pair_smem_t<2048>(max_hist),
                   batched_pair_smem_t<4096>(max_hist), batched_pair_smem_t<8192>(max_hist)});
}

int batched_mixed_ctas_per_sm(int max_hist) {
  int n = 0;
  ensure_dynamic_smem((const void *)batched_pair_kernel_mixed, (int)batched_mixed_smem(kSmemHistMax));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batched_pair_kernel_mixed, 256,
                                                    batched_mixed_smem(max_hist)) != cudaSuccess)
    n = 1;
  return n > 0 ? n : 1;
}

cudaError_t launch_batched_pairs_mixed(const BatchCatalog *cats, const BatchItem *items, long long n_items,
                                       unsigned long long *counter, int grid, int max_hist, cudaStream_t s) {
  // attribute set by batched_mixed_ctas_per_sm during planning (no API call here: may be captured)
  batched_pair_kernel_mixed<<<grid, 256, batched_mixed_smem(max_hist), s>>>(cats, items, n_items, counter);
  return cudaGetLastError();
}

int batched_pairs_ctas_per_sm(int P, int max_hist) {
  switch (P) {
    case 64: return batched_ctas_t<64>(max_hist);
    case 128: return batched_ctas_t<128>(max_hist);
    case 256: return batched_ctas_t<256>(max_hist);
    case 512: return batched_ctas_t<512>(max_hist);
    case 1024: return batched_ctas_t<1024>(max_hist);
    case 2048: return batched_ctas_t<2048>(max_hist);
    case 4096: return batched_ctas_t<4096>(max_hist);
    case 8192: return batched_ctas_t<8192>(max_hist);
    default: return 1;
  }
}

cudaError_t launch_batched_pairs(int P, const BatchCatalog *cats, const BatchItem *items, long long n_items,
                                 unsigned long long *counter, int grid, int max_hist, cudaStream_t s) {
  switch (P) {
    case 64: return launch_batched_t<64>(cats, items, n_items, counter, grid, max_hist, s);
    case 128: return launch_batched_t<128>(cats, items, n_items, counter, grid, max_hist, s);
    case 256: return launch_batched_t<256>(cats, items, n_items, counter, grid, max_hist, s);
    case 512: return launch_batched_t<512>(cats, items, n_items, counter, grid, max_hist, s);
    case 1024: return launch_batched_t<1024>(cats, items, n_items, counter, grid, max_hist, s);
    case 2048: return launch_batched_t<2048>(cats, items, n_items, counter, grid, max_hist, s);
    case 4096: return launch_batched_t<4096>(cats, items, n_items, counter, grid, max_hist, s);
    case 8192: return launch_batched_t<8192>(cats, items, n_items, counter, grid, max_hist, s);
    default: return cudaErrorInvalidValue;
  }
}

int groups_per_cta(int P) { return (256 / (P / 32)) > 0 ? (256 / (P / 32)) : 1; }

template <int P> static size_t pair_smem_bytes(int n_hist) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int NW = (G + 31) / 32;
  size_t s = (size_t)NG * padded_len<P>() * sizeof(float2) + (size_t)NG * NW * 8 * sizeof(unsigned);
  if (n_hist > 0 && n_hist <= kSmemHistMax) s += (size_t)2 * n_hist * sizeof(int);
  return s;
}

template <int P, int ST> static cudaError_t launch_pairs_st(const PairArgs &a, int grid, cudaStream_t s) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  const size_t smem = pair_smem_bytes<P>(a.n_hist);
  cudaError_t e = ensure_dynamic_smem((const void *)pair_kernel<P, ST>, (int)pair_smem_bytes<P>(kSmemHistMax));
  if (e != cudaSuccess) return e;
  if (a.couple_end <= a.couple_begin) return cudaSuccess;
  pair_kernel<P, ST><<<grid, NG * G, smem, s>>>(a);
  return cudaGetLastError();
}

template <int P> static cudaError_t launch_pairs_t(const PairArgs &a, int grid, cudaStream_t s) {
  switch (a.stype) {
    case 0: return launch_pairs_st<P, 0>(a, grid, s);
    case 1: return launch_pairs_st<P, 1>(a, grid, s);
    case 2: return launch_pairs_st<P, 2>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int P> static int ctas_per_sm_t() {
  int n = 0;
  const size_t smem = pair_smem_bytes<P>(64);
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  ensure_dynamic_smem((const void *)pair_kernel<P, 0>, (int)pair_smem_bytes<P>(kSmemHistMax));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pair_kernel<P, 0>, NG * G, smem) != cudaSuccess) n = 1;
  return n > 0 ? n : 1;
}

int pair_ctas_per_sm(int P) {
  switch (P) {
    case 64: return ctas_per_sm_t<64>();
    case 128: return ctas_per_sm_t<128>();
    case 256: return ctas_per_sm_t<256>();
    case 512: return ctas_per_sm_t<512>();
    case 1024: return ctas_per_sm_t<1024>();
    case 2048: return ctas_per_sm_t<2048>();
    case 4096: return ctas_per_sm_t<4096>();
    case 8192: return ctas_per_sm_t<8192>();
    case 16384: return ctas_per_sm_t<16384>();
    default: return 1;
  }
}

cudaError_t launch_pairs(int P, const PairArgs &a, int grid, cudaStream_t s) {
  switch (P) {
    case 64: return launch_pairs_t<64>(a, grid, s);
    case 128: return launch_pairs_t<128>(a, grid, s);
    case 256: return launch_pairs_t<256>(a, grid, s);
    case 512: return launch_pairs_t<512>(a, grid, s);
    case 1024: return launch_pairs_t<1024>(a, grid, s);
    case 2048: return launch_pairs_t<2048>(a, grid, s);
    case 4096: return launch_pairs_t<4096>(a, grid, s);
    case 8192: return launch_pairs_t<8192>(a, grid, s);
    case 16384: return launch_pairs_t<16384>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
