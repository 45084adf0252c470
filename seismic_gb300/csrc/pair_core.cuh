// Device building blocks of the pair kernels (pairs.cu, staged_core.cuh):
// the conj-product accumulation of one couple, the assembly of its complex
// spectrum, the group inverse FFT, the lag-window scan with first-occurrence
// argmax / argmin, and the normalise / histogram / threshold / packed-write
// epilogue.
//
// A "couple" is two pairs (i, ja), (i, jb) that share event i, computed as
// ONE size-P complex inverse FFT:
//   Z = Y1 + i Y2,  Y1 = sum_c X_ic conj X_(ja)c,  Y2 = sum_c X_ic conj X_(jb)c,
// and, because both lag series are real, Re z and Im z are the two series.
// Thread t of a group of G = P/32 threads owns the Hermitian-mirror columns
// ca = t and cb = S - t (S = P/16; t = 0 owns columns 0 and S/2) of the
// radix-16 first pass, i.e. bins ca + r S and cb + r S for r = 0..7, so
// every spectral bin is read once per couple and both Z[k] and Z[P-k] are
// formed in registers.
//
// Lag semantics.  z[m] is the circular correlation sum_k x_i[k] x_j[k-d] at
// d = m (mod P).  The reference scans corr_t[L + t], t = -shift .. shift-1,
// reporting lag t+1 (Correlation_in_OMP/correlation_c.cpp:102-111);
// corr_t[L+t] equals the circular correlation at d = t+1, so lag d is read
// at m = d mod P, and the first-occurrence rule becomes "largest value, ties
// to the smallest d".
#pragma once

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

// Tile x of the upper triangle of nb x nb tiles in row-band order: bands of
// `band` tile rows (band <= 0: one band), each walked column by column from
// its own diagonal to the right edge, top to bottom within a column.  The
// rows of one band (its i spectra) stay in L2 while every column to their
// right passes over them once, and the outputs of one band are the packed
// rows of its events: a contiguous range of the packed triangle.
__host__ __device__ __forceinline__ void band_tile(long long x, long long nb, long long band, long long &bi,
                                                   long long &bj) {
  if (band <= 0 || band > nb) band = nb;
  long long r0 = 0;  // first tile row of the band
  for (;;) {
    const long long re = r0 + band < nb ? r0 + band : nb;
    const long long wb = re - r0;
    const long long tri = wb * (wb + 1) / 2;
    const long long cnt = tri + wb * (nb - re);
    if (x < cnt || re >= nb) {
      if (x < tri) {  // the band's own triangle: column c holds c + 1 tiles
        long long c = (long long)((sqrtf(8.0f * (float)x + 1.0f) - 1.0f) * 0.5f);
        if (c < 0) c = 0;
        if (c > wb - 1) c = wb - 1;
        while (c + 1 < wb && (c + 1) * (c + 2) / 2 <= x) ++c;
        while (c > 0 && c * (c + 1) / 2 > x) --c;
        bi = r0 + (x - c * (c + 1) / 2);
        bj = r0 + c;
      } else {        // full columns right of the band, wb tiles each
        const long long y = x - tri;
        // 32-bit division when it fits (a 64-bit one is a long software routine)
        const long long q = (y < 0x7fffffffLL && wb < 0x7fffffffLL) ? (long long)((unsigned)y / (unsigned)wb) : y / wb;
        bj = re + q;
        bi = r0 + (y - q * wb);
      }
      return;
    }
    x -= cnt;
    r0 = re;
  }
}


// Spectrum storage types: 0 float2 (FP32 form), 1 half2, 2 bfloat162.  For
// the half types the pointwise product a * conj(b) takes 16-bit factors and
// accumulates over channels in FP32.
template <int ST> struct SpecT;
template <> struct SpecT<0> {
  using T = float2;
  __device__ static __forceinline__ void cmac_conj(float2 &y, float2 a, float2 b) {
    y.x = fmaf(a.x, b.x, fmaf(a.y, b.y, y.x));
    y.y = fmaf(a.y, b.x, fmaf(-a.x, b.y, y.y));
  }
  __device__ static __forceinline__ float2 f2(float2 a) { return a; }
};
// Half types: y += a conj(b) by mixed-precision FMA (16-bit factors, FP32
// addend and result): each product of two 16-bit values is exact in FP32 and
// is added with one rounding, in the FP32 form's order -- four FMAs, like
// FP32, where HMUL2 products rounded every product to 16 bits and needed
// conversions and adds besides (FP16 spectra at N=4096, C=3, P=4096: 79 ->
// 102 M pairs/s).
template <> struct SpecT<1> {
  using T = __half2;
  __device__ static __forceinline__ void cmac_conj(float2 &y, __half2 a, __half2 b) {
    asm("{\n .reg .b16 ax, ay, bx, by, nax;\n mov.b32 {ax, ay}, %2;\n mov.b32 {bx, by}, %3;\n neg.f16 nax, ax;\n"
        " fma.rn.f32.f16 %0, ay, by, %0;\n fma.rn.f32.f16 %0, ax, bx, %0;\n"
        " fma.rn.f32.f16 %1, nax, by, %1;\n fma.rn.f32.f16 %1, ay, bx, %1;\n}"
        : "+f"(y.x), "+f"(y.y)
        : "r"(*reinterpret_cast<const unsigned *>(&a)), "r"(*reinterpret_cast<const unsigned *>(&b)));
  }
  __device__ static __forceinline__ float2 f2(__half2 a) { return __half22float2(a); }
};
template <> struct SpecT<2> {
  using T = __nv_bfloat162;
  __device__ static __forceinline__ void cmac_conj(float2 &y, __nv_bfloat162 a, __nv_bfloat162 b) {
    asm("{\n .reg .b16 ax, ay, bx, by, nax;\n mov.b32 {ax, ay}, %2;\n mov.b32 {bx, by}, %3;\n neg.bf16 nax, ax;\n"
        " fma.rn.f32.bf16 %0, ay, by, %0;\n fma.rn.f32.bf16 %0, ax, bx, %0;\n"
        " fma.rn.f32.bf16 %1, nax, by, %1;\n fma.rn.f32.bf16 %1, ay, bx, %1;\n}"
        : "+f"(y.x), "+f"(y.y)
        : "r"(*reinterpret_cast<const unsigned *>(&a)), "r"(*reinterpret_cast<const unsigned *>(&b)));
  }
  __device__ static __forceinline__ float2 f2(__nv_bfloat162 a) { return __bfloat1622float2(a); }
};

// 4-byte asynchronous global -> shared copy (no register holds the value),
// and the wait for this thread's copies.
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(smem_dst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Float-pair arithmetic of the final normalisation (values hi + lo).
// (a.x + a.y)(b.x + b.y) to ~2^-46 relative: the exact product of the his by
// FMA, plus the cross terms (Dekker's product with FMA).
__device__ __forceinline__ float2 product_pair(float2 a, float2 b) {
  const float h = a.x * b.x;
  float l = fmaf(a.x, b.x, -h);
  l = fmaf(a.x, b.y, fmaf(a.y, b.x, l));
  return make_float2(h, l);
}
// 1/c as hi + lo: hi rounded, lo the rounded rest (1 - hi c exact by FMA).
__device__ __forceinline__ float2 reciprocal_pair(int c) {
  const float fc = (float)c;
  const float h = 1.0f / fc;
  return make_float2(h, fmaf(-h, fc, 1.0f) / fc);
}
// x (s.x + s.y) rounded once to float (up to a rare double rounding).
__device__ __forceinline__ float compensated_scale(float x, float2 s) { return fmaf(x, s.x, x * s.y); }

__device__ __forceinline__ int hist_bin(float v, float delta, int n_hist) {
  if (v >= 1.0f) return n_hist - 1;
  int b = (int)(v / delta);
  return b > n_hist - 1 ? n_hist - 1 : (b < 0 ? 0 : b);
}

// Conj-product accumulators of one couple for one thread's 16 bins.
struct CoupleAcc {
  float2 ya1[8], ya2[8], yb1[8], yb2[8];
  float dc1, dc2, nq1, nq2;  // DC and Nyquist bins (real), packed in slot 0

  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int r = 0; r < 8; ++r) ya1[r] = ya2[r] = yb1[r] = yb2[r] = make_float2(0.f, 0.f);
    dc1 = dc2 = nq1 = nq2 = 0.f;
  }
  // Bin ca + r S (values xa, pa, qa of rows i, ja, jb) and cb + r S (xb, pb, qb).
  template <int ST, typename V>
  __device__ __forceinline__ void add(int r, V xa, V pa, V qa, V xb, V pb, V qb) {
    using SP = SpecT<ST>;
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
};

// Z = Y1 + i Y2 over the full Hermitian range for columns ca, cb:
// v[r] = Z[ca + r S], v[16 + r] = Z[cb + r S], r = 0..15.
__device__ __forceinline__ void assemble_couple(const CoupleAcc &y, int t, float2 (&v)[32]) {
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const float2 A1 = y.ya1[r], A2 = y.ya2[r], B1 = y.yb1[r], B2 = y.yb2[r];
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
        v[0] = make_float2(y.dc1, y.dc2);
        v[8] = make_float2(y.nq1, y.nq2);
      } else {
        v[r] = za;
        v[16 - r] = zac;
      }
    }
  }
}

// Unnormalised inverse FFT of size P by a group of G = P/32 threads: pass 1
// (radix 16, no twiddles) on both columns in registers, then the Stockham
// passes of FftPlan<P> through the group's padded exchange buffer.
// With `stop` (the staged form's abort), the first group barrier also ORs
// *stop over the group; if it comes out set, every thread of the group
// returns there (the caller then leaves its item loop).
template <int P>
__device__ __forceinline__ void inverse_fft_group(float2 (&v)[32], float2 *buf, int t, int g, int ca, int cb,
                                                  const float2 *__restrict__ tw, const TwiddleRoots<P, 1> &roots,
                                                  bool *stop = nullptr) {
  using PL = FftPlan<P>;
  constexpr int G = P / 32;
  dft<16, 1>(&v[0]);
  dft<16, 1>(&v[16]);
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    buf[pad16(ca * 16 + r)] = v[r];
    buf[pad16(cb * 16 + r)] = v[16 + r];
  }
  if (stop) {
    *stop = group_sync_any<G>(g, *stop);
    if (*stop) return;
  } else {
    group_sync<G>(g);
  }
  pass_read<P, PL::R2>(buf, v, t);
  group_sync<G>(g);
  pass_compute_held<P, PL::R2, 16, 1>(v, roots.template get<2>());
  if constexpr (PL::R3 != 0) {
    pass_write<P, PL::R2, 16>(buf, v, t);
    group_sync<G>(g);
    pass_read<P, PL::R3>(buf, v, t);
    group_sync<G>(g);
    pass_compute_held<P, PL::R3, 16 * PL::R2, 1>(v, roots.template get<3>());
    if constexpr (PL::R4 != 0) {
      pass_write<P, PL::R3, 16 * PL::R2>(buf, v, t);
      group_sync<G>(g);
      pass_read<P, PL::R4>(buf, v, t);
      group_sync<G>(g);
      pass_compute_held<P, PL::R4, 16 * PL::R2 * PL::R3, 1>(v, roots.template get<4>());
    }
  }
}

// inverse_fft_group through a half-size exchange buffer of padded_len<P/2>():
// each exchange runs in two rounds, round h moving the values whose index
// lies in [h P/2, (h+1) P/2).  Readers of a radix-R pass take r in
// [h R/2, (h+1) R/2) of every job: index t + q G + r P/R, with t + q G < P/R,
// lies in round h's half exactly then, at the same local index t + q G +
// r' P/R in both rounds.  Writers: after pass 1 the column set h (ca, then
// cb: ca < S/2 <= cb); after a later pass of radix R and stride NS the jobs
// q in [h J/2, (h+1) J/2), whose indices (j / NS) NS R + j % NS + r NS lie in
// half h when P / (2R) is a multiple of NS.  Round h's reads land in the
// registers round h wrote (v[16 h .. 16 h + 15]) and a compile-time renaming
// restores the v[q R + r] order.  Two more group barriers per exchange buy
// half the shared memory, which the staged form gives to its ring.  Same
// arithmetic as inverse_fft_group, bit for bit.
template <int P, int R> __device__ __forceinline__ void split_read(const float2 *buf, float2 (&v)[32], int t, int h) {
  constexpr int G = P / 32, J = 32 / R;
#pragma unroll
  for (int q = 0; q < J; ++q) {
    const float2 *row = buf + pad16(t + q * G);
#pragma unroll
    for (int r = 0; r < R / 2; ++r) v[16 * h + (R / 2) * q + r] = row[r * (P / R) * 17 / 16];
  }
}
// v[16 h + (R/2) q + r'] holds job q's value r = h R/2 + r'  ->  v[q R + r]
template <int R> __device__ __forceinline__ void split_order(float2 (&v)[32]) {
  constexpr int J = 32 / R;
  float2 w[32];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int q = 0; q < J; ++q)
#pragma unroll
      for (int r = 0; r < R / 2; ++r) w[q * R + h * (R / 2) + r] = v[16 * h + (R / 2) * q + r];
#pragma unroll
  for (int e = 0; e < 32; ++e) v[e] = w[e];
}
template <int P, int R, int NS>
__device__ __forceinline__ void split_write(float2 *buf, const float2 (&v)[32], int t, int h) {
  constexpr int G = P / 32, J = 32 / R;
  static_assert(NS % 16 == 0 && (P / (2 * R)) % NS == 0 && J % 2 == 0, "split_write: jobs not split by halves");
#pragma unroll
  for (int q = h * (J / 2); q < (h + 1) * (J / 2); ++q) {
    const int j = t + q * G;
    float2 *row = buf + pad16((j / NS) * NS * R + (j % NS) - h * (P / 2));
#pragma unroll
    for (int r = 0; r < R; ++r) row[r * NS * 17 / 16] = v[q * R + r];
  }
}
// One later exchange (writer: radix RW, stride NSW; reader: radix RR) in two
// rounds; the first barrier is a plain one (the abort vote sits at pass 1's).
template <int P, int RW, int NSW, int RR>
__device__ __forceinline__ void split_exchange(float2 *buf, float2 (&v)[32], int t, int g) {
  constexpr int G = P / 32;
  split_write<P, RW, NSW>(buf, v, t, 0);
  group_sync<G>(g);
  split_read<P, RR>(buf, v, t, 0);
  group_sync<G>(g);
  split_write<P, RW, NSW>(buf, v, t, 1);
  group_sync<G>(g);
  split_read<P, RR>(buf, v, t, 1);
  split_order<RR>(v);
  group_sync<G>(g);
}
template <int P>
__device__ __forceinline__ void inverse_fft_group_split(float2 (&v)[32], float2 *buf, int t, int g, int ca, int cb,
                                                        const TwiddleRoots<P, 1> &roots, bool *stop = nullptr) {
  using PL = FftPlan<P>;
  constexpr int G = P / 32;
  dft<16, 1>(&v[0]);
  dft<16, 1>(&v[16]);
  // first exchange: columns ca (indices < P/2), then cb (>= P/2)
#pragma unroll
  for (int r = 0; r < 16; ++r) buf[pad16(ca * 16 + r)] = v[r];
  if (stop) {
    *stop = group_sync_any<G>(g, *stop);
    if (*stop) return;
  } else {
    group_sync<G>(g);
  }
  split_read<P, PL::R2>(buf, v, t, 0);
  group_sync<G>(g);
#pragma unroll
  for (int r = 0; r < 16; ++r) buf[pad16(cb * 16 + r - P / 2)] = v[16 + r];
  group_sync<G>(g);
  split_read<P, PL::R2>(buf, v, t, 1);
  split_order<PL::R2>(v);
  group_sync<G>(g);
  pass_compute_held<P, PL::R2, 16, 1>(v, roots.template get<2>());
  if constexpr (PL::R3 != 0) {
    split_exchange<P, PL::R2, 16, PL::R3>(buf, v, t, g);
    pass_compute_held<P, PL::R3, 16 * PL::R2, 1>(v, roots.template get<3>());
    if constexpr (PL::R4 != 0) {
      split_exchange<P, PL::R3, 16 * PL::R2, PL::R4>(buf, v, t, g);
      pass_compute_held<P, PL::R4, 16 * PL::R2 * PL::R3, 1>(v, roots.template get<4>());
    }
  }
}

// Bit q * RL + r set when the thread's last-pass value v[q * RL + r] (output
// index last_pass_index) lies inside the lag window 1 - shift .. shift (every
// bit for a window as wide as P).  It depends only on t and shift, so a
// kernel computes it once and the scan tests one bit per value.
template <int P> __device__ __forceinline__ uint32_t window_mask(int t, int shift) {
  using PL = FftPlan<P>;
  constexpr int RL = PL::R4 ? PL::R4 : (PL::R3 ? PL::R3 : PL::R2);
  if (2LL * shift >= P) return 0xffffffffu;
  const int d0 = 1 - shift;
  const int span = 2 * shift - 1;  // inside iff (m - d0) mod P <= span
  uint32_t mask = 0;
#pragma unroll
  for (int q = 0; q < 32 / RL; ++q) {
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      const int m = last_pass_index<P, RL>(t, q, r);
      if (((m - d0) & (P - 1)) <= span) mask |= 1u << (q * RL + r);
    }
  }
  return mask;
}

// Lag-window scan of the two series held in v after the last FFT pass,
// first-occurrence argmax / argmin, then (thread t == 0 of the group) the
// epilogue for pairs (ia, ja) (real part) and, if out_b, (ib, jb) (imaginary
// part): normalise, histogram (before the threshold), threshold, packed
// write.  `red` is the group's
// reduction scratch (NW * 8 words), `hist` the CTA's shared histogram,
// `xbuf` the group's exchange buffer (free once the transform's last pass
// has read it).
// Prescaled liveness by the copy-and-vote path of scan_and_write (VOTE), or
// by thread 0's loads in the epilogue.  Measured, M pairs/s, vote vs loads:
// FP32 spectra N=4096 C=3 P=4096 94.7 vs 91.5; FP16 there 93.4 vs 102.4; FP32
// at N=16384 P=512 (not prescaled; the code alone) 825 vs 831.
template <int P, int ST> constexpr bool kLivenessVote = ST == 0 && P >= 1024;
// Lag-window scan that skips a thread's r rows outside the window (ROWSKIP)
// instead of zeroing the values outside it one by one.  Measured, M
// pairs/s, skip vs zeroing (the full-window shape through the code alone):
// Q=512 x 4 FP32 841 vs 830, FP16 854 vs 812; Q=1024 x 2, three channels,
// 349 vs 339 and 385 vs 378; P=4096 three channels (full window) FP32 104.5 vs
// 102.1 but FP16 85 vs 102; plain P=2048 one channel 253-261 vs 268.
template <int P, int ST> constexpr bool kScanRowSkip = P <= 1024 || (P == 4096 && ST == 0);

template <int P, bool VOTE, bool ROWSKIP>
__device__ __forceinline__ void scan_and_write(const PairArgs &a, float2 (&v)[32], long long ia, long long ja,
                                               long long ib, long long jb, bool out_b, int t, int g, unsigned *red,
                                               int *hist, bool smem_hist, uint32_t wmask, float2 *xbuf) {
  using PL = FftPlan<P>;
  constexpr int G = P / 32;
  constexpr int NW = (G + 31) / 32;
  constexpr int RL = PL::R4 ? PL::R4 : (PL::R3 ? PL::R3 : PL::R2);
  const int d0 = 1 - a.shift;
  const unsigned gmask = group_lane_mask<G>();
  // the couple's inverse norms (one-channel forms), loaded before the scan
  // so their latency overlaps it; thread 0 of the group uses them below
  float2 pre_ni = make_float2(0.f, 0.f), pre_nja = pre_ni, pre_njb = pre_ni;
  if (t == 0 && !a.prescaled) {
    const int C = a.n_channels;
    pre_ni = (a.rect ? a.inv_norms_q : a.inv_norms)[ia * C];
    pre_nja = a.inv_norms[ja * C];
    pre_njb = a.inv_norms[jb * C];
  }
  // prescaled forms: a pair is live when some channel has both norms
  // nonzero.  Lane c < VL of the group copies channel c's inverse norms of
  // i, ja, jb into the group's exchange buffer by cp.async (the buffer is
  // free after the transform's last barrier) and a vote after the scan
  // combines them (channels from VL on: thread 0 below).  No loads on the
  // epilogue's path and no registers held across the scan.
  constexpr int VL = G < 32 ? G : 32;
  float *chn = reinterpret_cast<float *>(xbuf);
  if (VOTE && a.prescaled && t < VL && t < a.n_channels) {
    const int C = a.n_channels;
    cp_async4(chn + t, &(a.rect ? a.inv_norms_q : a.inv_norms)[ia * C + t].x);
    cp_async4(chn + 32 + t, &a.inv_norms[ja * C + t].x);
    cp_async4(chn + 64 + t, &a.inv_norms[jb * C + t].x);
  }

  // ---- phase A: per-thread max / min of both series.  Values outside the
  //      lag window (wmask = window_mask<P>(t, a.shift)) count as 0: 0 never
  //      wins, only a strictly positive maximum / negative minimum counts.
  //      A thread's values of one r (v[q RL + r], q = 0 .. J-1) lie P/RL lags
  //      apart, so a short window leaves whole r rows outside it: those are
  //      skipped (at Q = 512 and +-128 lags, rows r = 1, 2 of 4).
  if (!ROWSKIP && wmask != 0xffffffffu) {
#pragma unroll
    for (int e = 0; e < 32; ++e)
      if (!((wmask >> e) & 1u)) v[e] = make_float2(0.f, 0.f);
  }
  float mx0 = 0.f, mn0 = 0.f, mx1 = 0.f, mn1 = 0.f;
  if (!ROWSKIP || wmask == 0xffffffffu) {
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      mx0 = fmaxf(mx0, v[e].x);
      mn0 = fminf(mn0, v[e].x);
      mx1 = fmaxf(mx1, v[e].y);
      mn1 = fminf(mn1, v[e].y);
    }
  } else {
    constexpr int J = 32 / RL;
    constexpr uint32_t kRowBits = [] {
      uint32_t b = 0;
      for (int q = 0; q < J; ++q) b |= 1u << (q * RL);
      return b;
    }();
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      if (((wmask >> r) & kRowBits) == 0) continue;
#pragma unroll
      for (int q = 0; q < J; ++q) {
        const int e = q * RL + r;
        if ((wmask >> e) & 1u) {
          mx0 = fmaxf(mx0, v[e].x);
          mn0 = fminf(mn0, v[e].x);
          mx1 = fmaxf(mx1, v[e].y);
          mn1 = fminf(mn1, v[e].y);
        }
      }
    }
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
        if (ROWSKIP && !((wmask >> (q * RL + r)) & 1u)) continue;  // outside the lag window
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
  // the liveness vote, before the group barrier below: no thread of the
  // group writes the exchange buffer (next transform) until it is read
  bool live_a = false, live_b = false;
  if (VOTE && a.prescaled && t < VL) {
    float ci = 0.f, cja = 0.f, cjb = 0.f;
    if (t < a.n_channels) {
      cp_async_wait_all();
      ci = chn[t];
      cja = chn[32 + t];
      cjb = chn[64 + t];
    }
    const unsigned wm = group_lane_mask<VL>();
    live_a = __any_sync(wm, ci > 0.f && cja > 0.f);
    live_b = __any_sync(wm, ci > 0.f && cjb > 0.f);
  }
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
  //      final normalisation peak / (P |x_i| |x_j|) is taken at FP64-equivalent
  //      accuracy from the per-event FP64 inverse norms (hi + lo floats): the
  //      scale ni nj / P as a compensated float pair, then one compensated
  //      product with the peak.  FP32 instructions only: on this GPU an FP64
  //      instruction issues at 1/64 of the FP32 rate, and plain FP64 here,
  //      on the one thread per group that runs the epilogue, slowed the whole
  //      pair kernel by 12 % (242 vs 274 M pairs/s, N=16384 P=2048).
  if (t == 0) {
    const long long N = a.n_events;
    const int C = a.n_channels;
    const float2 *inv_i = a.rect ? a.inv_norms_q : a.inv_norms;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      if (p == 1 && !out_b) break;
      const long long i = p == 0 ? ia : ib;
      const long long j = p == 0 ? ja : jb;
      const unsigned kp = key[2 * p], kn = key[2 * p + 1];
      float2 scale;  // hi + lo
      bool live = false;
      if (a.prescaled) {  // spectra already carry 1/norm: mean over channels
        if constexpr (VOTE) {
          live = p == 0 ? live_a : live_b;
          for (int c = VL; c < C && !live; ++c)
            live = (inv_i[i * C + c].x > 0.f) && (a.inv_norms[j * C + c].x > 0.f);
        } else {
          for (int c = 0; c < C; ++c) live |= (inv_i[i * C + c].x > 0.f) && (a.inv_norms[j * C + c].x > 0.f);
        }
        scale = reciprocal_pair(C);
      } else {
        const float2 ni = pre_ni, nj = p == 0 ? pre_nja : pre_njb;  // ia == ib: one event i per couple
        live = ni.x > 0.f && nj.x > 0.f;
        scale = product_pair(ni, nj);
      }
      // 1/P is a power of two: exact on both parts
      scale.x *= 1.0f / (float)P;
      scale.y *= 1.0f / (float)P;
      float vp = 0.f, vn = 0.f;
      int lp = 0, ln = 0;
      if (live) {
        vp = compensated_scale(__uint_as_float(kp), scale);
        vn = -compensated_scale(__uint_as_float(kn), scale);
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

}  // namespace seismic
