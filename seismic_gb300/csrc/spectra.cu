// Kernel (a): forward real FFT of every (event, channel) row plus its FP64
// energy norm, run once per row.
//
// Replaces the reference's ComputeNorms (Correlation_in_OMP/correlation_c.cpp:195-204,
// float accumulation) and its two r2c FFT sets of the events and of the
// time-reversed events (ComputeFFT, correlation_c.cpp:32-49; cuFFT R2C x2 in
// Correlation_in_CUDA/correlation_cuda.cu:619-636).  Only the forward spectra
// are built: the reversed-event spectrum is conj(X) times a linear phase, and
// the pair kernel uses conj(X_j) directly.
//
// One group of G = P/32 threads transforms two rows at once as the real and
// imaginary parts of one complex size-P FFT:
//   z = a + i b,  Z = FFT(z),  A[k] = (Z[k] + conj Z[P-k]) / 2,
//   B[k] = (Z[k] - conj Z[P-k]) / (2i).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "energy.cuh"
#include "fft_core.cuh"
#include "kernels.cuh"

namespace seismic {

// exp(+2 pi i k / kMaxP); read by every kernel through a pointer argument.
__device__ float2 g_twiddle[kMaxP];

__global__ void twiddle_init_kernel() {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < kMaxP) {
    double s, c;
    sincospi(2.0 * (double)k / (double)kMaxP, &s, &c);
    g_twiddle[k] = make_float2((float)c, (float)s);
  }
}

cudaError_t init_twiddles(cudaStream_t s) {
  twiddle_init_kernel<<<kMaxP / 256, 256, 0, s>>>();
  return cudaGetLastError();
}

const float2 *twiddle_table() {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_twiddle) != cudaSuccess) return nullptr;
  return reinterpret_cast<const float2 *>(p);
}

__device__ __forceinline__ void store_spectrum(void *base, int stype, long long idx, float2 v) {
  if (stype == 0)
    reinterpret_cast<float2 *>(base)[idx] = v;
  else if (stype == 1)
    reinterpret_cast<__half2 *>(base)[idx] = __float22half2_rn(v);
  else
    reinterpret_cast<__nv_bfloat162 *>(base)[idx] = __float22bfloat162_rn(v);
}

// Sum over the group of G threads of float pairs (hi, lo) by exact TwoSum
// steps (energy.cuh): the group's energy without FP64 shuffles.  `red` is
// the group's scratch (2 * ceil(G / 32) doubles); thread 0's result is the
// one used.
template <int G> __device__ __forceinline__ void group_sum_pair(float &hi, float &lo, double *red, int g, int t) {
#pragma unroll
  for (int o = (G < 32 ? G : 32) / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(group_lane_mask<G>(), hi, o);
    const float l2 = __shfl_xor_sync(group_lane_mask<G>(), lo, o);
    add_pair(hi, lo, h2, l2);
  }
  if constexpr (G > 32) {
    float2 *rf = reinterpret_cast<float2 *>(red);
    if ((t & 31) == 0) rf[t >> 5] = make_float2(hi, lo);
    group_sync<G>(g);
    hi = 0.f;
    lo = 0.f;
#pragma unroll
    for (int w = 0; w < G / 32; ++w) add_pair(hi, lo, rf[w].x, rf[w].y);
    group_sync<G>(g);
  }
}

// Maximum over the group of G threads (same scratch and barriers as
// group_sum_pair).
template <int G> __device__ __forceinline__ float group_max_float(float v, double *red, int g, int t) {
#pragma unroll
  for (int o = (G < 32 ? G : 32) / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(group_lane_mask<G>(), v, o));
  if constexpr (G > 32) {
    if ((t & 31) == 0) red[t >> 5] = (double)v;
    group_sync<G>(g);
    float m = 0.f;
#pragma unroll
    for (int w = 0; w < G / 32; ++w) m = fmaxf(m, (float)red[w]);
    group_sync<G>(g);
    return m;
  } else {
    return v;
  }
}

template <int P> __device__ __forceinline__ void spectra_body(const SpectraArgs &a, long long pair_index,
                                                              unsigned char *smem_raw);

template <int P>
__global__ void __launch_bounds__(P / 32 > 256 ? P / 32 : 256) spectra_kernel(SpectraArgs a) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  spectra_body<P>(a, (long long)blockIdx.x * NG + threadIdx.x / G, smem_raw);
}

// Rows 2*pair_index and 2*pair_index+1 of `a`, by this thread's group.
template <int P> __device__ __forceinline__ void spectra_body(const SpectraArgs &a, long long pair_index,
                                                              unsigned char *smem_raw) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int S = P / 16;
  constexpr int H = P / 2;
  float2 *bufs = reinterpret_cast<float2 *>(smem_raw);
  double *reds = reinterpret_cast<double *>(bufs + NG * padded_len<P>());

  const int g = threadIdx.x / G;
  const int t = threadIdx.x % G;
  float2 *buf = bufs + g * padded_len<P>();
  double *red = reds + g * 2 * ((G + 31) / 32);

  const long long rows = a.n_events * (long long)a.n_channels;
  const long long row_a = 2 * pair_index;
  if (row_a >= rows) return;  // whole group leaves together
  const long long row_b = row_a + 1;
  const bool has_b = row_b < rows;

  const float *src_a = a.events + (row_a / a.n_channels) * a.ev_stride + (row_a % a.n_channels) * a.ch_stride;
  const float *src_b = has_b ? a.events + (row_b / a.n_channels) * a.ev_stride + (row_b % a.n_channels) * a.ch_stride
                             : src_a;

  // ---- pass 1: columns c0 = t and c1 = t + S/2, samples c + r*S
  float2 v[32];
  float ma = 0.f, mb = 0.f;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const int c = t + half * (S / 2);
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int s = c + r * S;
      float xa = 0.f, xb = 0.f;
      if (s < a.length) {
        xa = __ldg(src_a + s);
        xb = has_b ? __ldg(src_b + s) : 0.f;
      }
      ma = fmaxf(ma, fabsf(xa));
      mb = fmaxf(mb, fabsf(xb));
      v[half * 16 + r] = make_float2(xa, xb);
    }
  }
  // energies: samples scaled by a power of two below the row's largest
  // magnitude (exact; no overflow or loss of the large terms to FP32's
  // range), summed as float pairs, the exponent put back in FP64
  const int xea = energy_exponent(group_max_float<G>(ma, red, g, t));
  const int xeb = energy_exponent(group_max_float<G>(mb, red, g, t));
  const EnergyScale sca(xea), scb(xeb);
  float eah = 0.f, eal = 0.f, ebh = 0.f, ebl = 0.f;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    add_square(sca(v[k].x), eah, eal);
    add_square(scb(v[k].y), ebh, ebl);
  }
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    dft<16, -1>(&v[half * 16]);
    const int c = t + half * (S / 2);
#pragma unroll
    for (int r = 0; r < 16; ++r) buf[pad16(c * 16 + r)] = v[half * 16 + r];
  }
  group_sum_pair<G>(eah, eal, red, g, t);
  group_sum_pair<G>(ebh, ebl, red, g, t);
  // FP64 once per group: norms, inverse norms rounded once, and the
  // spectrum scale factors, handed to the group through `red`
  if (t == 0) {
    const double na = sqrt(ldexp((double)eah + (double)eal, 2 * xea));
    const double nb = sqrt(ldexp((double)ebh + (double)ebl, 2 * xeb));
    const double ia = na > 0.0 ? 1.0 / na : 0.0;
    const double ib = nb > 0.0 ? 1.0 / nb : 0.0;
    a.norms[row_a] = na;
    a.inv_norms[row_a] = split_double(ia);
    if (has_b) {
      a.norms[row_b] = nb;
      a.inv_norms[row_b] = split_double(ib);
    }
    float *scale = reinterpret_cast<float *>(red);
    scale[0] = a.prescale ? (float)ia : 1.f;
    scale[1] = a.prescale ? (float)ib : 1.f;
  }
  group_sync<G>(g);

  using PL = FftPlan<P>;
  pass_read<P, PL::R2>(buf, v, t);
  group_sync<G>(g);
  pass_compute<P, PL::R2, 16, -1>(v, t, a.twiddles);
  pass_write<P, PL::R2, 16>(buf, v, t);
  group_sync<G>(g);
  if constexpr (PL::R3 != 0) {
    pass_read<P, PL::R3>(buf, v, t);
    group_sync<G>(g);
    pass_compute<P, PL::R3, 16 * PL::R2, -1>(v, t, a.twiddles);
    pass_write<P, PL::R3, 16 * PL::R2>(buf, v, t);
    group_sync<G>(g);
  }
  if constexpr (PL::R4 != 0) {
    pass_read<P, PL::R4>(buf, v, t);
    group_sync<G>(g);
    pass_compute<P, PL::R4, 16 * PL::R2 * PL::R3, -1>(v, t, a.twiddles);
    pass_write<P, PL::R4, 16 * PL::R2 * PL::R3>(buf, v, t);
    group_sync<G>(g);
  }

  // ---- split the two rows, scale, write packed half spectra
  const float sa = reinterpret_cast<const float *>(red)[0], sb = reinterpret_cast<const float *>(red)[1];
  const long long off_a = row_a * (long long)H, off_b = row_b * (long long)H;
#pragma unroll 4
  for (int k = t; k < H; k += G) {
    const float2 zk = buf[pad16(k)];
    float2 va, vb;
    if (k == 0) {
      const float2 zh = buf[pad16(H)];
      va = make_float2(zk.x * sa, zh.x * sa);
      vb = make_float2(zk.y * sb, zh.y * sb);
    } else {
      const float2 zm = buf[pad16(P - k)];
      // A = (Z[k] + conj Z[P-k]) / 2 ; B = (Z[k] - conj Z[P-k]) / (2i)
      const float2 A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      const float2 B = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
      va = make_float2(A.x * sa, A.y * sa);
      vb = make_float2(B.x * sb, B.y * sb);
    }
    store_spectrum(a.spectra, a.stype, off_a + k, va);
    if (has_b) store_spectrum(a.spectra, a.stype, off_b + k, vb);
  }
}

template <int P> static cudaError_t launch_spectra_t(const SpectraArgs &a, cudaStream_t s) {
  constexpr int G = P / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  const long long rows = a.n_events * (long long)a.n_channels;
  const long long groups = (rows + 1) / 2;
  const long long ctas = (groups + NG - 1) / NG;
  if (ctas <= 0) return cudaSuccess;
  if (ctas > 0x7fffffffLL) return cudaErrorInvalidValue;
  const size_t smem = (size_t)NG * padded_len<P>() * sizeof(float2) + (size_t)NG * 2 * ((G + 31) / 32) * sizeof(double);
  cudaError_t e = ensure_dynamic_smem((const void *)spectra_kernel<P>, (int)smem);
  if (e != cudaSuccess) return e;
  spectra_kernel<P><<<(unsigned)ctas, NG * G, smem, s>>>(a);
  return cudaGetLastError();
}

// Batched form: each item is up to one CTA's worth of row pairs (NG of its
// size P) of one catalog; CTAs stride over the item list.
__global__ void __launch_bounds__(256)
    batched_spectra_kernel(const BatchCatalog *__restrict__ cats, const BatchItem *__restrict__ items,
                           long long n_items) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const SpectraArgs a = cats[w.cat].spec;
    const int P = cats[w.cat].P;
    const long long idx = w.begin + threadIdx.x / (P / 32);
    if (idx < w.end) {
      switch (P) {
        case 64: spectra_body<64>(a, idx, smem_raw); break;
        case 128: spectra_body<128>(a, idx, smem_raw); break;
        case 256: spectra_body<256>(a, idx, smem_raw); break;
        case 512: spectra_body<512>(a, idx, smem_raw); break;
        case 1024: spectra_body<1024>(a, idx, smem_raw); break;
        case 2048: spectra_body<2048>(a, idx, smem_raw); break;
        case 4096: spectra_body<4096>(a, idx, smem_raw); break;
        case 8192: spectra_body<8192>(a, idx, smem_raw); break;
        default: break;
      }
    }
    __syncthreads();  // the next item may lay its groups out differently
  }
}

cudaError_t launch_batched_spectra(const BatchCatalog *cats, const BatchItem *items, long long n_items, int grid,
                                   cudaStream_t s) {
  // every size uses NG * (P + P/16) float2 = 69,632 bytes plus <= 2 KB of reduction slots
  const size_t smem = (size_t)8 * (8192 + 512) + 2048;
  // the first call per device happens before any capture (batch planning)
  cudaError_t e = ensure_dynamic_smem((const void *)batched_spectra_kernel, (int)smem);
  if (e != cudaSuccess) return e;
  if (n_items <= 0) return cudaSuccess;
  batched_spectra_kernel<<<grid, 256, smem, s>>>(cats, items, n_items);
  return cudaGetLastError();
}

cudaError_t launch_spectra(int P, const SpectraArgs &a, cudaStream_t s) {
  switch (P) {
    case 64: return launch_spectra_t<64>(a, s);
    case 128: return launch_spectra_t<128>(a, s);
    case 256: return launch_spectra_t<256>(a, s);
    case 512: return launch_spectra_t<512>(a, s);
    case 1024: return launch_spectra_t<1024>(a, s);
    case 2048: return launch_spectra_t<2048>(a, s);
    case 4096: return launch_spectra_t<4096>(a, s);
    case 8192: return launch_spectra_t<8192>(a, s);
    case 16384: return launch_spectra_t<16384>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

bool supported_padded_size(int P) { return P >= kMinP && P <= kMaxP && (P & (P - 1)) == 0; }

// ------------------------------------------------------- overlap-save frames
// One group of G = Q/32 threads per (event, channel) row: the row's FP64
// norm over its L samples (the same float-pair energy as spectra_body), then
// for every block b one complex size-Q FFT whose real part is the A frame
// and imaginary part the W frame, split as in spectra_body.  Both spectra
// carry the row's 1/norm when prescale is set.
template <int Q>
__global__ void __launch_bounds__(256) block_spectra_kernel(SpectraArgs a) {
  constexpr int G = Q / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  constexpr int S = Q / 16;
  constexpr int H = Q / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *bufs = reinterpret_cast<float2 *>(smem_raw);
  double *reds = reinterpret_cast<double *>(bufs + NG * padded_len<Q>());
  const int g = threadIdx.x / G;
  const int t = threadIdx.x % G;
  float2 *buf = bufs + g * padded_len<Q>();
  double *red = reds + g * 2 * ((G + 31) / 32);
  const long long rows = a.n_events * (long long)a.n_channels;
  const long long row = (long long)blockIdx.x * NG + g;
  if (row >= rows) return;  // whole group leaves together
  const float *src = a.events + (row / a.n_channels) * a.ev_stride + (row % a.n_channels) * a.ch_stride;
  const int L = a.length;

  // ---- norm over the L samples
  float m = 0.f;
  for (int s = t; s < L; s += G) m = fmaxf(m, fabsf(__ldg(src + s)));
  const int xe = energy_exponent(group_max_float<G>(m, red, g, t));
  const EnergyScale sc(xe);
  float eh = 0.f, el = 0.f;
  for (int s = t; s < L; s += G) add_square(sc(__ldg(src + s)), eh, el);
  group_sum_pair<G>(eh, el, red, g, t);
  if (t == 0) {
    const double nrm = sqrt(ldexp((double)eh + (double)el, 2 * xe));
    const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    a.norms[row] = nrm;
    a.inv_norms[row] = split_double(inv);
    reinterpret_cast<float *>(red)[0] = a.prescale ? (float)inv : 1.f;
  }
  group_sync<G>(g);
  const float scale = reinterpret_cast<const float *>(red)[0];

  using PL = FftPlan<Q>;
  for (int b = 0; b < a.blocks; ++b) {
    const int o = b * a.block_len - a.block_shift;  // frame origin in the row
    float2 v[32];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int c = t + half * (S / 2);
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int k = c + r * S;  // frame index
        const int n = o + k;      // sample index
        const float x = (n >= 0 && n < L) ? __ldg(src + n) : 0.f;
        const bool in_a = k >= a.block_shift && k < a.block_shift + a.block_len;
        v[half * 16 + r] = make_float2(in_a ? x : 0.f, x);
      }
    }
    group_sync<G>(g);  // the previous block's split has read buf
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      dft<16, -1>(&v[half * 16]);
      const int c = t + half * (S / 2);
#pragma unroll
      for (int r = 0; r < 16; ++r) buf[pad16(c * 16 + r)] = v[half * 16 + r];
    }
    group_sync<G>(g);
    pass_read<Q, PL::R2>(buf, v, t);
    group_sync<G>(g);
    pass_compute<Q, PL::R2, 16, -1>(v, t, a.twiddles);
    pass_write<Q, PL::R2, 16>(buf, v, t);
    group_sync<G>(g);
    if constexpr (PL::R3 != 0) {
      pass_read<Q, PL::R3>(buf, v, t);
      group_sync<G>(g);
      pass_compute<Q, PL::R3, 16 * PL::R2, -1>(v, t, a.twiddles);
      pass_write<Q, PL::R3, 16 * PL::R2>(buf, v, t);
      group_sync<G>(g);
    }
    if constexpr (PL::R4 != 0) {
      pass_read<Q, PL::R4>(buf, v, t);
      group_sync<G>(g);
      pass_compute<Q, PL::R4, 16 * PL::R2 * PL::R3, -1>(v, t, a.twiddles);
      pass_write<Q, PL::R4, 16 * PL::R2 * PL::R3>(buf, v, t);
      group_sync<G>(g);
    }
    const long long off = (row * a.blocks + b) * (long long)H;
#pragma unroll 4
    for (int k = t; k < H; k += G) {
      const float2 zk = buf[pad16(k)];
      float2 va, vw;
      if (k == 0) {
        const float2 zh = buf[pad16(H)];
        va = make_float2(zk.x * scale, zh.x * scale);
        vw = make_float2(zk.y * scale, zh.y * scale);
      } else {
        const float2 zm = buf[pad16(Q - k)];
        const float2 A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        const float2 W = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        va = make_float2(A.x * scale, A.y * scale);
        vw = make_float2(W.x * scale, W.y * scale);
      }
      if (a.spectra) store_spectrum(a.spectra, a.stype, off + k, va);  // either may be left out
      if (a.spectra_w) store_spectrum(a.spectra_w, a.stype, off + k, vw);
    }
  }
}

template <int Q> static cudaError_t launch_block_spectra_t(const SpectraArgs &a, cudaStream_t s) {
  constexpr int G = Q / 32;
  constexpr int NG = (256 / G) > 0 ? (256 / G) : 1;
  const long long rows = a.n_events * (long long)a.n_channels;
  const long long ctas = (rows + NG - 1) / NG;
  if (ctas <= 0) return cudaSuccess;
  if (ctas > 0x7fffffffLL || a.blocks < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)NG * padded_len<Q>() * sizeof(float2) + (size_t)NG * 2 * ((G + 31) / 32) * sizeof(double);
  cudaError_t e = ensure_dynamic_smem((const void *)block_spectra_kernel<Q>, (int)smem);
  if (e != cudaSuccess) return e;
  block_spectra_kernel<Q><<<(unsigned)ctas, NG * G, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_block_spectra(int Q, const SpectraArgs &a, cudaStream_t s) {
  switch (Q) {
    case 512: return launch_block_spectra_t<512>(a, s);
    case 1024: return launch_block_spectra_t<1024>(a, s);
    case 2048: return launch_block_spectra_t<2048>(a, s);
    case 4096: return launch_block_spectra_t<4096>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
