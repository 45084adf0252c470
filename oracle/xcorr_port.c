/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this library, and only as the
 * checker / the timed CPU baseline.  The product never links it.
 *
 * A plain-C restatement of the reference's CPU (OpenMP + FFTW) path,
 * Correlation_in_OMP/correlation_c.cpp, kept in the reference's own float
 * operation order so that, built with the same FFT (fftw_shim), it gives
 * bit-identical outputs to the reference source compiled by
 * the `ref` target of oracle/Makefile.  Steps and the lines they follow:
 *
 *   norms             float sequential sum of squares, sqrt   (:195-204)
 *   forward spectra   r2c of events and of reversed events    (:32-49)
 *   pair loop         upper triangle incl. diagonal, dynamic
 *                     row schedule, packed index
 *                     i*N - i(i-1)/2 + (j-i)                   (:251-293, :269)
 *   product           X_i * XR_j, plain complex product       (:188-193)
 *   inverse + scan    c2r, scan corr_t[L+t], t in [-shift,
 *                     shift), first strict max > 0 / min < 0,
 *                     lag t+1                                 (:58-111)
 *   normalise         v / ((float)P * n_i * n_j)              (:115, :127)
 *   histograms        before the threshold, last bin for
 *                     |v| >= 1, else int(|v| / delta)         (:116-117, :128-129)
 *   threshold         v > thr / v < -thr, else 0 and lag 0    (:119-136)
 *
 * Deliberate differences from the reference, all where it is undefined:
 *  - a NaN coefficient (an all-zero event, 0/0) is counted in no histogram
 *    bin; the reference indexes its histogram with int(NaN) (:117, :129);
 *  - a histogram index is clamped to the last bin;
 *  - the packed index is computed in 64-bit (the reference's `int`
 *    overflows for N >= 46341, :269);
 *  - scan positions outside corr_t (L + shift > P) read as 0.0 instead of
 *    past the buffer (:102-103).
 * The port prints nothing (the reference prints its parameters, :215-249).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "fftw_shim/fftw3.h"

static void port_norms(const float *events, float *norms, int n_events, int event_length,
                       int padded) {
  int i, j;
  for (i = 0; i < n_events; i++) {
    float pot = 0.0f;
    for (j = 0; j < event_length; j++) {
      const float v = events[(size_t)i * padded + j];
      pot += v * v;
    }
    norms[i] = sqrtf(pot);
  }
}

/* One pair's inverse FFT, window scan, normalisation, histogram and threshold. */
static void port_pair(fftwf_complex *corr_f, float *corr_t, fftwf_plan plan, int event_length,
                      int shift, int padded, float norm1, float norm2, float threshold,
                      int *hmax, int *hmin, int n_hist, float delta_hist, float *val_pos,
                      int *lag_pos, float *val_neg, int *lag_neg) {
  float pos = 0.0f, neg = 0.0f, vp, vn;
  int l_pos = 0, l_neg = 0, t;
  fftwf_execute_dft_c2r(plan, corr_f, corr_t);
  for (t = -shift; t < shift; t++) {
    const int idx = event_length + t;
    const float v = (idx >= 0 && idx < padded) ? corr_t[idx] : 0.0f;
    if (v > pos) {
      pos = v;
      l_pos = t + 1;
    } else if (v < neg) {
      neg = v;
      l_neg = t + 1;
    }
  }
  vp = pos / ((float)padded * norm1 * norm2);
  if (vp >= 1.0) {
    hmax[n_hist - 1]++;
  } else if (vp == vp) {
    int b = (int)(vp / delta_hist);
    if (b > n_hist - 1) b = n_hist - 1;
    if (b < 0) b = 0;
    hmax[b]++;
  }
  if (vp > threshold) {
    *val_pos = vp;
    *lag_pos = l_pos;
  } else {
    *val_pos = 0.0f;
    *lag_pos = 0;
  }
  vn = neg / ((float)padded * norm1 * norm2);
  if (vn <= -1.0) {
    hmin[n_hist - 1]++;
  } else if (vn == vn) {
    int b = (int)(-(vn) / delta_hist);
    if (b > n_hist - 1) b = n_hist - 1;
    if (b < 0) b = 0;
    hmin[b]++;
  }
  if (vn < -threshold) {
    *val_neg = vn;
    *lag_neg = l_neg;
  } else {
    *val_neg = 0.0f;
    *lag_neg = 0;
  }
}

/*
 * Same argument list and meaning as the reference's exported
 * correlationCPP (Correlation_in_OMP/correlation_c.cpp:210-213).
 * Histograms are accumulated into (+=), outputs are written in place.
 */
void port_correlationCPP(float *events, float *events_reversed, int n_events, int event_length,
                         int shift, int paddedSize, int num_threads, int chunk_size,
                         float threshold, int n_classes_hist, float *xcorr_vals_pos,
                         int *xcorr_lags_pos, float *xcorr_vals_neg, int *xcorr_lags_neg,
                         int *max_hist, int *min_hist) {
  const int fftsize = paddedSize / 2 + 1;
  const float delta_hist = (float)(1.0 / n_classes_hist);
  fftwf_complex *sf, *srf;
  float *norms;
  int i;
  if (n_events <= 0 || paddedSize < 4 || n_classes_hist < 1) return;
  if (chunk_size < 1) chunk_size = 1;
  sf = (fftwf_complex *)fftwf_malloc(sizeof(fftwf_complex) * (size_t)n_events * fftsize);
  srf = (fftwf_complex *)fftwf_malloc(sizeof(fftwf_complex) * (size_t)n_events * fftsize);
  norms = (float *)malloc(sizeof(float) * (size_t)n_events);
  if (!sf || !srf || !norms) {
    fftwf_free(sf);
    fftwf_free(srf);
    free(norms);
    return;
  }
  port_norms(events, norms, n_events, event_length, paddedSize);

#ifdef _OPENMP
  if (num_threads > 0) omp_set_num_threads(num_threads);
#pragma omp parallel default(shared)
#endif
  {
    fftwf_plan plan = fftwf_plan_dft_r2c_1d(paddedSize, events_reversed, srf, FFTW_MEASURE);
    int e;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (e = 0; e < n_events; e++) {
      fftwf_execute_dft_r2c(plan, &events[(size_t)e * paddedSize], &sf[(size_t)e * fftsize]);
      fftwf_execute_dft_r2c(plan, &events_reversed[(size_t)e * paddedSize],
                            &srf[(size_t)e * fftsize]);
    }
    fftwf_destroy_plan(plan);
  }

#ifdef _OPENMP
#pragma omp parallel default(shared)
#endif
  {
    int *pmax = (int *)calloc((size_t)n_classes_hist, sizeof(int));
    int *pmin = (int *)calloc((size_t)n_classes_hist, sizeof(int));
    fftwf_complex *corr_f = (fftwf_complex *)fftwf_malloc(sizeof(fftwf_complex) * fftsize);
    float *corr_t = (float *)fftwf_malloc(sizeof(float) * paddedSize);
    fftwf_plan plan = fftwf_plan_dft_c2r_1d(paddedSize, corr_f, corr_t, FFTW_MEASURE);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, chunk_size)
#endif
    for (i = 0; i < n_events; i++) {
      int j;
      const int64_t base = (int64_t)i * n_events - (int64_t)i * (i - 1) / 2;
      const fftwf_complex *a = &sf[(size_t)i * fftsize];
      for (j = 0; j < n_events - i; j++) {
        const fftwf_complex *b = &srf[(size_t)(i + j) * fftsize];
        int k;
        for (k = 0; k < fftsize; k++) {
          corr_f[k][0] = a[k][0] * b[k][0] - a[k][1] * b[k][1];
          corr_f[k][1] = a[k][1] * b[k][0] + a[k][0] * b[k][1];
        }
        port_pair(corr_f, corr_t, plan, event_length, shift, paddedSize, norms[i], norms[i + j],
                  threshold, pmax, pmin, n_classes_hist, delta_hist, &xcorr_vals_pos[base + j],
                  &xcorr_lags_pos[base + j], &xcorr_vals_neg[base + j],
                  &xcorr_lags_neg[base + j]);
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      int h;
      for (h = 0; h < n_classes_hist; h++) {
        max_hist[h] += pmax[h];
        min_hist[h] += pmin[h];
      }
    }
    fftwf_free(corr_f);
    fftwf_free(corr_t);
    fftwf_destroy_plan(plan);
    free(pmax);
    free(pmin);
  }
  fftwf_free(sf);
  fftwf_free(srf);
  free(norms);
}

/* Number of OpenMP threads a parallel region would use by default. */
int port_threads_available(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
