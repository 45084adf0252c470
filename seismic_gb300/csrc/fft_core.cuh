// Register/shared-memory FFT building blocks for the sm_103a kernels.
//
// Layout conventions used by every kernel in this library:
//  * A transform of size P is owned by a "group" of G = P/32 threads.  Each
//    thread holds 32 complex values in registers; passes are radix-16 first,
//    then the radices of FftPlan<P> (mixed-radix Stockham autosort,
//    Govindaraju et al., SC'08), with the data exchanged through a padded
//    shared-memory buffer between passes.
//  * Shared buffers hold float2 at index pad(i) = i + (i >> 4): with 64-bit
//    accesses (served per half-warp) this makes the stride-16 writes of the
//    first pass and the contiguous reads/writes of later passes bank-conflict
//    free.
//  * DIR = +1 is the unnormalised inverse transform (e^{+2 pi i nk/P}, the
//    convention of an FFTW c2r plan), DIR = -1 the forward transform.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace seismic {

__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

// Radix plan after the first radix-16 pass; 0 terminates.
template <int P> struct FftPlan;
template <> struct FftPlan<64> { static constexpr int R2 = 4, R3 = 0, R4 = 0; };
template <> struct FftPlan<128> { static constexpr int R2 = 8, R3 = 0, R4 = 0; };
template <> struct FftPlan<256> { static constexpr int R2 = 16, R3 = 0, R4 = 0; };
template <> struct FftPlan<512> { static constexpr int R2 = 8, R3 = 4, R4 = 0; };
template <> struct FftPlan<1024> { static constexpr int R2 = 16, R3 = 4, R4 = 0; };
template <> struct FftPlan<2048> { static constexpr int R2 = 16, R3 = 8, R4 = 0; };
template <> struct FftPlan<4096> { static constexpr int R2 = 16, R3 = 16, R4 = 0; };
template <> struct FftPlan<8192> { static constexpr int R2 = 16, R3 = 8, R4 = 4; };
template <> struct FftPlan<16384> { static constexpr int R2 = 16, R3 = 16, R4 = 4; };

__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
template <int P> __host__ __device__ constexpr int padded_len() { return P + P / 16; }

// ---------------------------------------------------------------- complex ops
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * (DIR * i)
template <int DIR> __device__ __forceinline__ float2 mul_i(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Multiply by exp(DIR * 2 pi i * K / N) for the compile-time constants used
// inside the radix-8/16 kernels.
template <int DIR, int K, int N> __device__ __forceinline__ float2 twc(float2 v) {
  constexpr int k = ((K % N) + N) % N;
  constexpr float h = 0.70710678118654752440f;   // cos(pi/4)
  constexpr float c1 = 0.92387953251128675613f;  // cos(pi/8)
  constexpr float s1 = 0.38268343236508977173f;  // sin(pi/8)
  if constexpr (k == 0) {
    return v;
  } else if constexpr (N == 16 && (k % 2 == 0)) {
    return twc<DIR, k / 2, 8>(v);
  } else if constexpr (N == 8 && (k % 2 == 0)) {
    return twc<DIR, k / 2, 4>(v);
  } else if constexpr (N == 4) {
    if constexpr (k == 1) return mul_i<DIR>(v);
    else if constexpr (k == 2) return make_float2(-v.x, -v.y);
    else return mul_i<-DIR>(v);
  } else if constexpr (N == 8) {
    // k odd: 1, 3, 5, 7 -> (+-h, +-h)
    constexpr float c = (k == 1 || k == 7) ? h : -h;
    constexpr float s = (k == 1 || k == 3) ? h : -h;
    return cmul(v, make_float2(c, DIR * s));
  } else {
    static_assert(N == 16, "twc: unsupported N");
    // k odd in 1..15: cos/sin of k*pi/8
    constexpr float cs[16] = {1.f, c1, h, s1, 0.f, -s1, -h, -c1, -1.f, -c1, -h, -s1, 0.f, s1, h, c1};
    constexpr float sn[16] = {0.f, s1, h, c1, 1.f, c1, h, s1, 0.f, -s1, -h, -c1, -1.f, -c1, -h, -s1};
    return cmul(v, make_float2(cs[k], DIR * sn[k]));
  }
}

// ------------------------------------------------------------ radix kernels
template <int DIR> __device__ __forceinline__ void dft2(float2 &a, float2 &b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int DIR> __device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
  const float2 s02 = cadd(v0, v2), d02 = csub(v0, v2);
  const float2 s13 = cadd(v1, v3), d13 = mul_i<DIR>(csub(v1, v3));
  v0 = cadd(s02, s13);
  v2 = csub(s02, s13);
  v1 = cadd(d02, d13);
  v3 = csub(d02, d13);
}

// DFT_R in place on v[0..R), natural order in and out.
template <int R, int DIR> __device__ __forceinline__ void dft(float2 *v) {
  if constexpr (R == 2) {
    dft2<DIR>(v[0], v[1]);
  } else if constexpr (R == 4) {
    dft4<DIR>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    // r = r1 + 2 r2 ; DFT4 over r2, twiddle w8^{r1 q2}, DFT2 over r1 ; X[q2 + 4 q1]
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    o1 = twc<DIR, 1, 8>(o1);
    o2 = twc<DIR, 2, 8>(o2);
    o3 = twc<DIR, 3, 8>(o3);
    v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
  } else {
    static_assert(R == 16, "dft: unsupported radix");
    // r = r1 + 4 r2 ; DFT4 over r2 for each r1 ; twiddle w16^{r1 q2} ; DFT4 over r1 ; X[q2 + 4 q1]
    float2 u[4][4];
#pragma unroll
    for (int r1 = 0; r1 < 4; ++r1) {
      u[r1][0] = v[r1]; u[r1][1] = v[r1 + 4]; u[r1][2] = v[r1 + 8]; u[r1][3] = v[r1 + 12];
      dft4<DIR>(u[r1][0], u[r1][1], u[r1][2], u[r1][3]);
    }
    u[1][1] = twc<DIR, 1, 16>(u[1][1]); u[1][2] = twc<DIR, 2, 16>(u[1][2]); u[1][3] = twc<DIR, 3, 16>(u[1][3]);
    u[2][1] = twc<DIR, 2, 16>(u[2][1]); u[2][2] = twc<DIR, 4, 16>(u[2][2]); u[2][3] = twc<DIR, 6, 16>(u[2][3]);
    u[3][1] = twc<DIR, 3, 16>(u[3][1]); u[3][2] = twc<DIR, 6, 16>(u[3][2]); u[3][3] = twc<DIR, 9, 16>(u[3][3]);
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) {
      float2 a = u[0][q2], b = u[1][q2], c = u[2][q2], d = u[3][q2];
      dft4<DIR>(a, b, c, d);
      v[q2] = a; v[q2 + 4] = b; v[q2 + 8] = c; v[q2 + 12] = d;
    }
  }
}

// --------------------------------------------------------------- twiddles
// tw[k] = exp(+2 pi i k / kMaxP), computed in double and rounded once
// (twiddle_table()).  A size-P transform reads entry k * (kMaxP / P).
template <int DIR> __device__ __forceinline__ float2 twiddle_lookup(const float2 *__restrict__ tw, int k_maxp) {
  const float2 w = __ldg(&tw[k_maxp & (kMaxP - 1)]);
  return DIR > 0 ? w : make_float2(w.x, -w.y);
}

// v[r] *= w^r, r = 1..R-1, w = exp(DIR 2 pi i m / (NS R)); powers from one
// table entry and a shallow product tree (at most 4 roundings per power).
template <int R> __device__ __forceinline__ void root_powers(float2 w1, float2 (&w)[R]) {
  w[1] = w1;
#pragma unroll
  for (int r = 2; r < R; ++r) w[r] = (r & 1) ? cmul(w[r - 1], w1) : cmul(w[r / 2], w[r / 2]);
}
template <int R> __device__ __forceinline__ void apply_powers(float2 *v, const float2 (&w)[R]) {
#pragma unroll
  for (int r = 1; r < R; ++r) v[r] = cmul(v[r], w[r]);
}
template <int R> __device__ __forceinline__ void apply_root_powers(float2 *v, float2 w1) {
  float2 w[R];
  root_powers<R>(w1, w);
  apply_powers<R>(v, w);
}

template <int P, int R, int NS, int DIR>
__device__ __forceinline__ void apply_twiddles(float2 *v, int m, const float2 *__restrict__ tw) {
  if constexpr (NS == 1) {
    return;
  } else {
    constexpr int step = kMaxP / (NS * R);
    apply_root_powers<R>(v, twiddle_lookup<DIR>(tw, m * step));
  }
}

// cos and sin of x for |x| <= pi, in double at compile time (Taylor series
// to the 41st power: far below double rounding there).
constexpr double ct_sin(double x) {
  double term = x, sum = x;
  for (int n = 1; n <= 20; ++n) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}
constexpr double ct_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n <= 20; ++n) {
    term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}

// v * exp(DIR 2 pi i NUM / DEN), the root rounded once from double at compile
// time: exp(i a) = -exp(i (a - pi)) with a - pi in [-pi, pi).
template <int NUM, int DEN, int DIR> __device__ __forceinline__ float2 mul_turn(float2 v) {
  constexpr int k = ((NUM % DEN) + DEN) % DEN;
  if constexpr (k == 0) {
    return v;
  } else {
    constexpr double x = 6.28318530717958647692528676655900577 * k / DEN - 3.14159265358979323846264338327950288;
    constexpr float c = (float)(-ct_cos(x));
    constexpr float s = (float)(-ct_sin(x) * DIR);
    return cmul(v, make_float2(c, s));
  }
}

// Twiddle roots of the passes after the first, held by a persistent kernel
// (they depend only on the thread index).  In every plan each later pass is
// one of two kinds, both served by ONE root r_t = exp(DIR 2 pi i t / (NS R)):
//  * uniform (G % NS == 0): every job of the thread has m = t mod NS = t;
//  * base (the thread's J jobs have m = t + q G < NS): job q's root is r_t
//    times the compile-time root exp(DIR 2 pi i q G / (NS R)) (mul_turn).
// So no pass looks a twiddle up in the pair loop.
template <int P, int DIR> struct TwiddleRoots {
  using PL = FftPlan<P>;
  static constexpr int G = P / 32;
  static constexpr int NS2 = 16, NS3 = 16 * PL::R2, NS4 = 16 * PL::R2 * (PL::R3 ? PL::R3 : 1);
  float2 w2, w3, w4;

  __device__ __forceinline__ void load(int t, const float2 *__restrict__ tw) {
    w2 = twiddle_lookup<DIR>(tw, (t % NS2) * (kMaxP / (NS2 * PL::R2)));
    if constexpr (PL::R3 != 0) w3 = twiddle_lookup<DIR>(tw, (t % NS3) * (kMaxP / (NS3 * PL::R3)));
    if constexpr (PL::R4 != 0) w4 = twiddle_lookup<DIR>(tw, (t % NS4) * (kMaxP / (NS4 * PL::R4)));
  }
  template <int PASS> __device__ __forceinline__ float2 get() const {
    if constexpr (PASS == 2) return w2;
    else if constexpr (PASS == 3) return w3;
    else return w4;
  }
};

// Job q of a pass served by a held root (TwiddleRoots): twiddles then DFT_R,
// for q = Q .. J-1.
template <int P, int R, int NS, int DIR, int Q = 0>
__device__ __forceinline__ void base_root_jobs(float2 (&v)[32], float2 root) {
  constexpr int G = P / 32;
  constexpr int J = 32 / R;
  if constexpr (Q < J) {
    apply_root_powers<R>(&v[Q * R], mul_turn<Q * G, NS * R, DIR>(root));
    dft<R, DIR>(&v[Q * R]);
    base_root_jobs<P, R, NS, DIR, Q + 1>(v, root);
  }
}

// A later pass with its held root (uniform or base kind, see TwiddleRoots).
template <int P, int R, int NS, int DIR>
__device__ __forceinline__ void pass_compute_held(float2 (&v)[32], float2 root) {
  constexpr int G = P / 32;
  constexpr int J = 32 / R;
  static_assert(NS > 1 && (G % NS == 0 || J * G <= NS), "pass_compute_held: root not of one kind");
  if constexpr (G % NS == 0) {
    float2 w[R];
    root_powers<R>(root, w);
#pragma unroll
    for (int q = 0; q < J; ++q) {
      apply_powers<R>(&v[q * R], w);
      dft<R, DIR>(&v[q * R]);
    }
  } else {
    base_root_jobs<P, R, NS, DIR>(v, root);
  }
}

// ------------------------------------------------------------- group sync
// A group is G consecutive threads of a CTA.  Groups of <= 32 threads live in
// one warp and sync with __syncwarp on their own lanes; larger groups use a
// hardware named barrier (ids 1..15, id 0 is __syncthreads).
template <int G> __device__ __forceinline__ unsigned group_lane_mask() {
  if constexpr (G >= 32) {
    return 0xffffffffu;
  } else {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned base = lane & ~(unsigned)(G - 1);
    return ((G == 32) ? 0xffffffffu : ((1u << G) - 1u)) << base;
  }
}

template <int G> __device__ __forceinline__ void group_sync(int group_in_cta) {
  if constexpr (G <= 32) {
    __syncwarp(group_lane_mask<G>());
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(group_in_cta + 1), "r"(G) : "memory");
  }
}

// group_sync that also returns, on every thread of the group, whether `v`
// is set on any of them (a warp vote, or a named-barrier OR-reduction for
// groups wider than a warp, which is a barrier like bar.sync).
template <int G> __device__ __forceinline__ bool group_sync_any(int group_in_cta, bool v) {
  if constexpr (G <= 32) {
    __syncwarp(group_lane_mask<G>());
    return __any_sync(group_lane_mask<G>(), v);
  } else {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.or.pred po, %2, %3, pi;\n"
        " selp.u32 %0, 1, 0, po;\n}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(group_in_cta + 1), "r"(G)
        : "memory");
    return r != 0;
  }
}

// Stockham pass helpers for passes after the first.  A pass of radix R has
// P/R butterflies ("jobs"); thread t of the group runs jobs t + q*G,
// q = 0..32/R-1, holding them in v[q*R + r].
template <int P, int R> __device__ __forceinline__ void pass_read(const float2 *buf, float2 (&v)[32], int t) {
  constexpr int G = P / 32;
  constexpr int J = 32 / R;
  // pad16(j + c) = pad16(j) + 17 c / 16 for c a multiple of 16: one padded
  // base per job, constant offsets for its R values
  static_assert((P / R) % 16 == 0, "pass_read: stride must be a multiple of 16");
#pragma unroll
  for (int q = 0; q < J; ++q) {
    const float2 *row = buf + pad16(t + q * G);
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = row[r * (P / R) * 17 / 16];
  }
}

template <int P, int R, int NS, int DIR>
__device__ __forceinline__ void pass_compute(float2 (&v)[32], int t, const float2 *__restrict__ tw,
                                             const float2 *roots = nullptr) {
  constexpr int G = P / 32;
  constexpr int J = 32 / R;
  if constexpr (NS > 1 && J > 1 && G % NS == 0) {
    // every job of this thread has the same m = t mod NS: one set of powers
    float2 w[R];
    root_powers<R>(roots != nullptr ? roots[0] : twiddle_lookup<DIR>(tw, (t % NS) * (kMaxP / (NS * R))), w);
#pragma unroll
    for (int q = 0; q < J; ++q) {
      apply_powers<R>(&v[q * R], w);
      dft<R, DIR>(&v[q * R]);
    }
  } else {
#pragma unroll
    for (int q = 0; q < J; ++q) {
      const int j = t + q * G;
      if (roots != nullptr)
        apply_root_powers<R>(&v[q * R], roots[q]);
      else
        apply_twiddles<P, R, NS, DIR>(&v[q * R], j % NS, tw);
      dft<R, DIR>(&v[q * R]);
    }
  }
}

template <int P, int R, int NS> __device__ __forceinline__ void pass_write(float2 *buf, const float2 (&v)[32], int t) {
  constexpr int G = P / 32;
  constexpr int J = 32 / R;
#pragma unroll
  for (int q = 0; q < J; ++q) {
    const int j = t + q * G;
    static_assert(NS % 16 == 0, "pass_write: stride must be a multiple of 16");
    float2 *row = buf + pad16((j / NS) * NS * R + (j % NS));  // constant offsets below
#pragma unroll
    for (int r = 0; r < R; ++r) row[r * NS * 17 / 16] = v[q * R + r];
  }
}

// Output index of v[q*R + r] after the LAST pass (NS * R == P): j + r * NS.
template <int P, int R> __device__ __forceinline__ int last_pass_index(int t, int q, int r) {
  constexpr int G = P / 32;
  return t + q * G + r * (P / R);
}

}  // namespace seismic
