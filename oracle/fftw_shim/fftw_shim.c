/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Implementation of the FFTW-3 look-alike
 * declared in fftw3.h.  Written from the mathematics, not from FFTW:
 *
 *  complex FFT of size m (power of two): in-place bit-reversal permutation
 *  followed by log2(m) radix-2 decimation-in-time butterfly stages
 *  (Cooley & Tukey 1965), twiddles w^k = exp(sign 2 pi i k / m) computed in
 *  double and rounded to float once per plan.
 *
 *  r2c of size n = 2m:  z[j] = x[2j] + i x[2j+1],  Z = DFT_m(z),
 *     Fe[k] = (Z[k] + conj Z[m-k]) / 2,  Fo[k] = (Z[k] - conj Z[m-k]) / (2i),
 *     X[k]  = Fe[k] + e^{-2 pi i k/n} Fo[k],   k = 0..m   (Z[m] == Z[0]).
 *
 *  c2r of size n = 2m (unnormalised):
 *     Z[k] = (X[k] + conj X[m-k]) + i e^{+2 pi i k/n} (X[k] - conj X[m-k]),
 *     z = IDFT_m(Z),  y[2j] = Re z[j],  y[2j+1] = Im z[j].
 *
 * Every execute call is re-entrant: the only state is the read-only plan.
 */
#define _POSIX_C_SOURCE 200112L /* posix_memalign under -std=c11 */
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { SHIM_R2C = 1, SHIM_C2R = 2 };

struct shim_fftwf_plan_s {
  int kind;
  int n;          /* real length */
  int m;          /* n / 2, complex FFT length */
  int log2m;
  void *in;       /* arrays bound at plan time (for fftwf_execute) */
  void *out;
  float *tw_fwd;  /* m/2 complex twiddles e^{-2 pi i k/m} */
  float *tw_inv;  /* m/2 complex twiddles e^{+2 pi i k/m} */
  float *post;    /* m+1 complex twiddles e^{-+2 pi i k/n} for the packing step */
  int *bitrev;    /* bit-reversal permutation of 0..m-1 */
};

static int ilog2_exact(int v) {
  int l = 0;
  if (v <= 0 || (v & (v - 1)) != 0) return -1;
  while ((1 << l) < v) ++l;
  return l;
}

static fftwf_plan make_plan(int kind, int n, void *in, void *out) {
  const double two_pi = 6.283185307179586476925286766559;
  fftwf_plan p;
  int k;
  if (n < 4 || ilog2_exact(n) < 0) return NULL;
  p = (fftwf_plan)calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->kind = kind;
  p->n = n;
  p->m = n / 2;
  p->log2m = ilog2_exact(p->m);
  p->in = in;
  p->out = out;
  p->tw_fwd = (float *)malloc(sizeof(float) * 2 * (size_t)(p->m / 2 + 1));
  p->tw_inv = (float *)malloc(sizeof(float) * 2 * (size_t)(p->m / 2 + 1));
  p->post = (float *)malloc(sizeof(float) * 2 * (size_t)(p->m + 1));
  p->bitrev = (int *)malloc(sizeof(int) * (size_t)p->m);
  if (!p->tw_fwd || !p->tw_inv || !p->post || !p->bitrev) {
    fftwf_destroy_plan(p);
    return NULL;
  }
  for (k = 0; k <= p->m / 2; ++k) {
    double a = two_pi * (double)k / (double)p->m;
    p->tw_fwd[2 * k] = (float)cos(a);
    p->tw_fwd[2 * k + 1] = (float)(-sin(a));
    p->tw_inv[2 * k] = (float)cos(a);
    p->tw_inv[2 * k + 1] = (float)sin(a);
  }
  for (k = 0; k <= p->m; ++k) {
    double a = two_pi * (double)k / (double)n;
    double s = (kind == SHIM_R2C) ? -1.0 : 1.0;
    p->post[2 * k] = (float)cos(a);
    p->post[2 * k + 1] = (float)(s * sin(a));
  }
  for (k = 0; k < p->m; ++k) {
    int r = 0, v = k, b;
    for (b = 0; b < p->log2m; ++b) {
      r = (r << 1) | (v & 1);
      v >>= 1;
    }
    p->bitrev[k] = r;
  }
  return p;
}

/* In-place complex FFT of length m on interleaved float data. */
static void cfft_inplace(const struct shim_fftwf_plan_s *p, float *d, int inverse) {
  const int m = p->m;
  const float *tw = inverse ? p->tw_inv : p->tw_fwd;
  int k, len;
  for (k = 0; k < m; ++k) {
    int r = p->bitrev[k];
    if (r > k) {
      float t0 = d[2 * k], t1 = d[2 * k + 1];
      d[2 * k] = d[2 * r];
      d[2 * k + 1] = d[2 * r + 1];
      d[2 * r] = t0;
      d[2 * r + 1] = t1;
    }
  }
  for (len = 2; len <= m; len <<= 1) {
    const int half = len >> 1;
    const int step = m / len;
    int base;
    for (base = 0; base < m; base += len) {
      int q;
      for (q = 0; q < half; ++q) {
        const float wr = tw[2 * (q * step)];
        const float wi = tw[2 * (q * step) + 1];
        float *a = d + 2 * (base + q);
        float *b = d + 2 * (base + q + half);
        const float br = b[0] * wr - b[1] * wi;
        const float bi = b[0] * wi + b[1] * wr;
        const float ar = a[0], ai = a[1];
        a[0] = ar + br;
        a[1] = ai + bi;
        b[0] = ar - br;
        b[1] = ai - bi;
      }
    }
  }
}

static void exec_r2c(const struct shim_fftwf_plan_s *p, const float *x, float *X) {
  const int m = p->m;
  int k;
  /* X has room for m+1 complex; pack z[j] = x[2j] + i x[2j+1] into X[0..m) */
  if ((const void *)x != (const void *)X) memmove(X, x, sizeof(float) * 2 * (size_t)m);
  cfft_inplace(p, X, 0);
  /* post-processing, pairing k with m-k so it can run in place */
  {
    const float z0r = X[0], z0i = X[1];
    X[0] = z0r + z0i;
    X[1] = 0.0f;
    X[2 * m] = z0r - z0i;
    X[2 * m + 1] = 0.0f;
  }
  for (k = 1; k <= m / 2; ++k) {
    const int q = m - k;
    const float zkr = X[2 * k], zki = X[2 * k + 1];
    const float zqr = X[2 * q], zqi = X[2 * q + 1];
    /* Fe[k] = (Z[k] + conj Z[q]) / 2 ; Fo[k] = (Z[k] - conj Z[q]) / (2i) */
    const float fekr = 0.5f * (zkr + zqr), feki = 0.5f * (zki - zqi);
    const float fokr = 0.5f * (zki + zqi), foki = -0.5f * (zkr - zqr);
    /* for index q: Fe[q] = conj Fe[k], Fo[q] = conj Fo[k] */
    const float wkr = p->post[2 * k], wki = p->post[2 * k + 1];
    const float wqr = p->post[2 * q], wqi = p->post[2 * q + 1];
    const float xkr = fekr + (wkr * fokr - wki * foki);
    const float xki = feki + (wkr * foki + wki * fokr);
    const float xqr = fekr + (wqr * fokr + wqi * foki);
    const float xqi = -feki + (wqi * fokr - wqr * foki);
    X[2 * k] = xkr;
    X[2 * k + 1] = xki;
    X[2 * q] = xqr;
    X[2 * q + 1] = xqi;
  }
}

static void exec_c2r(const struct shim_fftwf_plan_s *p, const float *X, float *y) {
  const int m = p->m;
  int k;
  float *Z = y; /* y holds n floats = m complex */
  if ((const void *)X == (const void *)y) {
    /* in-place c2r is not used by the reference; refuse silently */
    return;
  }
  for (k = 0; k < m; ++k) {
    const int q = m - k;
    const float xkr = X[2 * k], xki = X[2 * k + 1];
    const float xqr = X[2 * q], xqi = -X[2 * q + 1]; /* conj X[m-k] */
    const float er = xkr + xqr, ei = xki + xqi;     /* X[k] + conj X[m-k] */
    const float dr = xkr - xqr, di = xki - xqi;     /* X[k] - conj X[m-k] */
    const float wr = p->post[2 * k], wi = p->post[2 * k + 1];
    const float tr = wr * dr - wi * di, ti = wr * di + wi * dr;
    /* Z = e + i t */
    Z[2 * k] = er - ti;
    Z[2 * k + 1] = ei + tr;
  }
  cfft_inplace(p, Z, 1);
}

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags) {
  (void)flags;
  return make_plan(SHIM_R2C, n, in, out);
}

fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags) {
  (void)flags;
  return make_plan(SHIM_C2R, n, in, out);
}

void fftwf_execute(const fftwf_plan p) {
  if (!p) return;
  if (p->kind == SHIM_R2C)
    exec_r2c(p, (const float *)p->in, (float *)p->out);
  else
    exec_c2r(p, (const float *)p->in, (float *)p->out);
}

void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) {
  if (!p || p->kind != SHIM_R2C) return;
  exec_r2c(p, in, (float *)out);
}

void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) {
  if (!p || p->kind != SHIM_C2R) return;
  exec_c2r(p, (const float *)in, out);
}

void fftwf_destroy_plan(fftwf_plan p) {
  if (!p) return;
  free(p->tw_fwd);
  free(p->tw_inv);
  free(p->post);
  free(p->bitrev);
  free(p);
}

void *fftwf_malloc(size_t n) {
  void *ptr = NULL;
  if (posix_memalign(&ptr, 64, n ? n : 1) != 0) return NULL;
  return ptr;
}

void fftwf_free(void *p) { free(p); }

void fftwf_cleanup(void) {}
