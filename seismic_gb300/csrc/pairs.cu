// Kernels (b) + (c): fused pair-tile correlation with an upper-triangle tile
// scheduler.
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
// tiles (bi, bj >= bi) are enumerated row-major over the upper triangle
// (decode_tile).  A tile holds tile*tile/2 "couples": two pairs (i, j) and
// (i, j+1) that share event i.  One couple is one size-P complex inverse FFT:
//   Z = Y1 + i Y2,  Y1 = sum_c X_ic conj X_jc,  Y2 = sum_c X_ic conj X_(j+1)c,
// and, because both lag series are real, Re z and Im z are the two series.
// Couples are dealt to groups of G = P/32 threads round-robin; the groups of
// one CTA take neighbouring couples of the same tile, so the tile's spectra
// are re-read from L1.
//
// Lag semantics.  z[m] is the circular correlation sum_k x_i[k] x_j[k-d] at
// d = m (mod P).  The reference scans corr_t[L + t], t = -shift .. shift-1,
// reporting lag t+1 (correlation_c.cpp:102-111); corr_t[L+t] equals the
// circular correlation at d = t+1, so lag d is read at m = d mod P, and the
// first-occurrence rule becomes "largest value, ties to the smallest d".
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <climits>

#include "fft_core.cuh"
#include "kernels.cuh"

namespace seismic {

constexpr int kSmemHistMax = 4096;

__host__ __device__ __forceinline__ long long tri_start(long long b, long long nb) {
  return b * nb - b * (b - 1) / 2;
}

// Row-major decode of tile index x over the upper triangle of nb x nb tiles:
// a single-precision estimate of the row, corrected exactly in integers.
__device__ __forceinline__ void decode_tile(long long x, long long nb, long long &bi, long long &bj) {
  const float twonb1 = 2.0f * (float)nb + 1.0f;
  long long b = (long long)((twonb1 - sqrtf(fmaxf(twonb1 * twonb1 - 8.0f * (float)x, 0.f))) * 0.5f);
  if (b < 0) b = 0;
  if (b > nb - 1) b = nb - 1;
  while (b + 1 < nb && tri_start(b + 1, nb) <= x) ++b;
  while (b > 0 && tri_start(b, nb) > x) --b;
  bi = b;
  bj = b + (x - tri_start(b, nb));
}

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

// Spectrum storage types: 0 float2 (FP32 form), 1 half2, 2 bfloat162.  For
// the half types the pointwise product a * conj(b) runs in the storage type
// (HMUL2) and is accumulated over channels in FP32.
template <int ST> struct SpecT;
template <> struct SpecT<0> {
  using T = float2;
  __device__ static __forceinline__ void cmac_conj(float2 &y, float2 a, float2 b) {
    y.x = fmaf(a.x, b.x, fmaf(a.y, b.y, y.x));
    y.y = fmaf(a.y, b.x, fmaf(-a.x, b.y, y.y));
  }
  __device__ static __forceinline__ float2 f2(float2 a) { return a; }
};
template <> struct SpecT<1> {
  using T = __half2;
  __device__ static __forceinline__ void cmac_conj(float2 &y, __half2 a, __half2 b) {
    const float2 p = __half22float2(__hmul2(a, b));                        // (ax bx, ay by)
    const float2 q = __half22float2(__hmul2(a, __lowhigh2highlow(b)));     // (ax by, ay bx)
    y.x += p.x + p.y;
    y.y += q.y - q.x;
  }
  __device__ static __forceinline__ float2 f2(__half2 a) { return __half22float2(a); }
};
template <> struct SpecT<2> {
  using T = __nv_bfloat162;
  __device__ static __forceinline__ void cmac_conj(float2 &y, __nv_bfloat162 a, __nv_bfloat162 b) {
    const float2 p = __bfloat1622float2(__hmul2(a, b));
    const float2 q = __bfloat1622float2(__hmul2(a, __lowhigh2highlow(b)));
    y.x += p.x + p.y;
    y.y += q.y - q.x;
  }
  __device__ static __forceinline__ float2 f2(__nv_bfloat162 a) { return __bfloat1622float2(a); }
};

__device__ __forceinline__ int hist_bin(float v, float delta, int n_hist) {
  if (v >= 1.0f) return n_hist - 1;
  int b = (int)(v / delta);
  return b > n_hist - 1 ? n_hist - 1 : (b < 0 ? 0 : b);
}

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

template <int P, int ST>
__global__ void __launch_bounds__(256, 2) pair_kernel(PairArgs a) {
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
  using SP = SpecT<ST>;
  using ST_T = typename SP::T;
  const ST_T *spectra = reinterpret_cast<const ST_T *>(a.spectra);
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int S = P / 16;
  constexpr int H = P / 2;
  constexpr int NW = (G + 31) / 32;
  using PL = FftPlan<P>;
  constexpr int RL = PL::R4 ? PL::R4 : (PL::R3 ? PL::R3 : PL::R2);
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
  const int d0 = 1 - a.shift;
  const bool full_window = 2LL * a.shift >= P;  // every index m is inside the lag window
  const int span = full_window ? P : 2 * a.shift - 1;  // inside iff (m - d0) mod P <= span
  const unsigned gmask = group_lane_mask<G>();
  // Twiddle roots of the radix-16 passes depend only on the thread: load once.
  TwiddleRoots<P, 1> roots;
  roots.load(t, a.twiddles);

  const int ca = (t == 0) ? 0 : t;
  const int cb = (t == 0) ? S / 2 : S - t;

  const ST_T *spectra_i = a.rect ? reinterpret_cast<const ST_T *>(a.spectra_q) : spectra;
  for (long long w = w_first; w < w_end; w += w_stride) {
    long long i, ja, jb;
    bool out_b;
    if (!a.rect) {
      const long long tile = w / cpt;
      const long long lc = w - tile * cpt;
      long long bi, bj;
      decode_tile(tile, nb, bi, bj);
      const long long ii = (2 * lc) / T, jj = (2 * lc) % T;
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
      const long long chunk = w / per_chunk, r = w - chunk * per_chunk;
      i = r / T;
      const long long j1 = 2 * (chunk * T + (r - i * T)), j2 = j1 + 1;
      if (j1 >= a.n_cols) continue;  // uniform over the group
      out_b = j2 < a.n_cols;
      ja = a.col_begin + j1;          // catalog event indices
      jb = out_b ? ja + 1 : ja;
    }

    // ---- conj products, accumulated over channels, for this thread's 16 bins
    float2 ya1[8], ya2[8], yb1[8], yb2[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      ya1[r] = ya2[r] = yb1[r] = yb2[r] = make_float2(0.f, 0.f);
    }
    float dc1 = 0.f, dc2 = 0.f, nq1 = 0.f, nq2 = 0.f;
    for (int c = 0; c < C; ++c) {
      const ST_T *Xi = spectra_i + (i * C + c) * (long long)H;
      const ST_T *X1 = spectra + (ja * C + c) * (long long)H;
      const ST_T *X2 = spectra + (jb * C + c) * (long long)H;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int ka = ca + r * S, kb = cb + r * S;
        const ST_T xa = __ldg(Xi + ka), pa = __ldg(X1 + ka), qa = __ldg(X2 + ka);
        const ST_T xb = __ldg(Xi + kb), pb = __ldg(X1 + kb), qb = __ldg(X2 + kb);
        SP::cmac_conj(ya1[r], xa, pa);
        SP::cmac_conj(ya2[r], xa, qa);
        SP::cmac_conj(yb1[r], xb, pb);
        SP::cmac_conj(yb2[r], xb, qb);
        if (r == 0) {  // slot 0 packs the two real bins DC and Nyquist
          const float2 fx = SP::f2(xa), fp = SP::f2(pa), fq = SP::f2(qa);
          dc1 = fmaf(fx.x, fp.x, dc1);
          nq1 = fmaf(fx.y, fp.y, nq1);
          dc2 = fmaf(fx.x, fq.x, dc2);
          nq2 = fmaf(fx.y, fq.y, nq2);
        }
      }
    }

    // ---- assemble Z = Y1 + i Y2 over the full Hermitian range for columns a, b
    float2 v[32];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float2 A1 = ya1[r], A2 = ya2[r], B1 = yb1[r], B2 = yb2[r];
      // Y1 + i Y2  and  conj(Y1) + i conj(Y2)
      const float2 za = make_float2(A1.x - A2.y, A1.y + A2.x);
      const float2 zac = make_float2(A1.x + A2.y, A2.x - A1.y);
      const float2 zb = make_float2(B1.x - B2.y, B1.y + B2.x);
      const float2 zbc = make_float2(B1.x + B2.y, B2.x - B1.y);
      v[16 + r] = zb;
      if (t != 0) {
        v[r] = za;
        v[16 + 15 - r] = zac;
        v[15 - r] = zbc;
      } else {
        v[16 + 15 - r] = zbc;
        if (r == 0) {
          v[0] = make_float2(dc1, dc2);
          v[8] = make_float2(nq1, nq2);
        } else {
          v[r] = za;
          v[16 - r] = zac;
        }
      }
    }

    // ---- pass 1 (radix 16, no twiddles) on both columns, then Stockham passes
    dft<16, 1>(&v[0]);
    dft<16, 1>(&v[16]);
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      buf[pad16(ca * 16 + r)] = v[r];
      buf[pad16(cb * 16 + r)] = v[16 + r];
    }
    group_sync<G>(g);
    pass_read<P, PL::R2>(buf, v, t);
    group_sync<G>(g);
    pass_compute<P, PL::R2, 16, 1>(v, t, a.twiddles, roots.template get<2>());
    if constexpr (PL::R3 != 0) {
      pass_write<P, PL::R2, 16>(buf, v, t);
      group_sync<G>(g);
      pass_read<P, PL::R3>(buf, v, t);
      group_sync<G>(g);
      pass_compute<P, PL::R3, 16 * PL::R2, 1>(v, t, a.twiddles, roots.template get<3>());
      if constexpr (PL::R4 != 0) {
        pass_write<P, PL::R3, 16 * PL::R2>(buf, v, t);
        group_sync<G>(g);
        pass_read<P, PL::R4>(buf, v, t);
        group_sync<G>(g);
        pass_compute<P, PL::R4, 16 * PL::R2 * PL::R3, 1>(v, t, a.twiddles, roots.template get<4>());
      }
    }

    // ---- window scan, phase A: per-thread max / min of both series.
    //      Values outside the lag window are zeroed (0 never wins: only a
    //      strictly positive maximum / strictly negative minimum counts).
#pragma unroll
    for (int q = 0; q < 32 / RL; ++q) {
#pragma unroll
      for (int r = 0; r < RL; ++r) {
        if (!full_window) {
          const int m = last_pass_index<P, RL>(t, q, r);
          if (((m - d0) & (P - 1)) > span) v[q * RL + r] = make_float2(0.f, 0.f);
        }
      }
    }
    float mx0 = 0.f, mn0 = 0.f, mx1 = 0.f, mn1 = 0.f;
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      mx0 = fmaxf(mx0, v[e].x);
      mn0 = fminf(mn0, v[e].x);
      mx1 = fmaxf(mx1, v[e].y);
      mn1 = fminf(mn1, v[e].y);
    }
    // ---- phase B: group maxima of the four magnitudes (float bits of values
    //      >= 0 order like unsigned integers)
    const unsigned own[4] = {__float_as_uint(mx0), __float_as_uint(-mn0) & 0x7fffffffu, __float_as_uint(mx1),
                             __float_as_uint(-mn1) & 0x7fffffffu};
    unsigned key[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) key[k] = __reduce_max_sync(gmask, own[k]);
    if constexpr (NW > 1) {
      if ((t & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) red[(t >> 5) * 8 + k] = key[k];
      }
      group_sync<G>(g);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        unsigned mk = red[k];
#pragma unroll
        for (int wv = 1; wv < NW; ++wv) mk = max(mk, red[wv * 8 + k]);
        key[k] = mk;
      }
    }
    // ---- phase C: threads holding a winning value find its smallest lag
    //      (first occurrence in increasing lag, as the reference's scan)
    int lag[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
    const bool owner = (key[0] && own[0] == key[0]) || (key[1] && own[1] == key[1]) ||
                       (key[2] && own[2] == key[2]) || (key[3] && own[3] == key[3]);
    if (owner) {
#pragma unroll
      for (int q = 0; q < 32 / RL; ++q) {
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          const int m = last_pass_index<P, RL>(t, q, r);
          const int d = d0 + ((m - d0) & (P - 1));
          const float2 z = v[q * RL + r];
          if (__float_as_uint(z.x) == key[0]) lag[0] = min(lag[0], d);
          if (__float_as_uint(-z.x) == key[1]) lag[1] = min(lag[1], d);
          if (__float_as_uint(z.y) == key[2]) lag[2] = min(lag[2], d);
          if (__float_as_uint(-z.y) == key[3]) lag[3] = min(lag[3], d);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) lag[k] = __reduce_min_sync(gmask, lag[k]);
    if constexpr (NW > 1) {
      if ((t & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) red[(t >> 5) * 8 + 4 + k] = (unsigned)lag[k];
      }
      group_sync<G>(g);
      if (t == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
          for (int wv = 0; wv < NW; ++wv) lag[k] = min(lag[k], (int)red[wv * 8 + 4 + k]);
        }
      }
    }

    // ---- epilogue: normalise, histogram, threshold, packed write.  The
    //      per-event factors 1/norm were computed in FP64 by the spectra
    //      kernel and rounded once; the per-pair scaling is FP32 (<= 4 ulp),
    //      which keeps the slow FP64 pipe out of the pair loop.
    if (t == 0) {
      const float *inv_i = a.rect ? a.inv_norms_q : a.inv_norms;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        if (p == 1 && !out_b) break;
        const long long j = p == 0 ? ja : jb;
        const unsigned kp = key[2 * p], kn = key[2 * p + 1];
        float scale;
        bool live = false;
        if (a.prescaled) {  // spectra already carry 1/norm: mean over channels
          for (int c = 0; c < C; ++c) live |= (inv_i[i * C + c] > 0.f) && (a.inv_norms[j * C + c] > 0.f);
          scale = 1.0f / ((float)P * (float)C);
        } else {
          const float ni = inv_i[i * C], nj = a.inv_norms[j * C];
          live = ni > 0.f && nj > 0.f;
          scale = (ni * nj) * (1.0f / (float)P);
        }
        float vp = 0.f, vn = 0.f;
        int lp = 0, ln = 0;
        if (live) {
          vp = __uint_as_float(kp) * scale;
          vn = -(__uint_as_float(kn) * scale);
          lp = kp ? lag[2 * p] : 0;
          ln = kn ? lag[2 * p + 1] : 0;
          if (a.n_hist > 0) {
            const int hp = hist_bin(vp, a.delta_hist, a.n_hist);
            const int hn = hist_bin(-vn, a.delta_hist, a.n_hist);
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
        const long long idx = a.rect ? i * a.n_cols + (j - a.col_begin) : i * N - i * (i - 1) / 2 + (j - i);
        a.vals_pos[idx] = vp;
        a.lags_pos[idx] = lp;
        a.vals_neg[idx] = vn;
        a.lags_neg[idx] = ln;
      }
    }
  }
}

// ----------------------------------------------------------- batched form
// One CTA-sized item of one catalog: the CTA's groups take its couples.
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
  cudaFuncSetAttribute(batched_pair_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)batched_pair_smem_t<P>(kSmemHistMax));
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
  static int configured_bytes = 0;
  if ((int)smem > configured_bytes) {
    const int want = (int)pair_smem_bytes<P>(kSmemHistMax);
    cudaError_t e = cudaFuncSetAttribute(pair_kernel<P, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, want);
    if (e != cudaSuccess) return e;
    configured_bytes = want;
  }
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
  cudaFuncSetAttribute(pair_kernel<P, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)pair_smem_bytes<P>(kSmemHistMax));
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
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
