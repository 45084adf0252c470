/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Nothing in the product links this.
 *
 * A minimal single-precision FFTW-3 API look-alike, written from the
 * mathematics (iterative radix-2 Cooley-Tukey plus the standard
 * real<->half-length-complex packing).  It exists because the reference's
 * CPU path (Correlation_in_OMP/correlation_c.cpp) calls FFTW 3.3 (float,
 * `-lfftw3f`, Correlation_in_OMP/Makefile:3-4) and FFTW is not available
 * here.  Only the calls that path makes are provided:
 *   fftwf_plan_dft_r2c_1d   (correlation_c.cpp:39)
 *   fftwf_plan_dft_c2r_1d   (correlation_c.cpp:264)
 *   fftwf_execute           (correlation_c.cpp:63)
 *   fftwf_execute_dft_r2c   (correlation_c.cpp:43,45)
 *   fftwf_destroy_plan, fftwf_malloc, fftwf_free, fftwf_cleanup
 * plus the types fftwf_complex / fftw_complex and the two planner flags.
 *
 * Semantics follow the published FFTW definitions: r2c computes
 * X[k] = sum_j x[j] e^{-2 pi i jk/n} for k = 0..n/2, c2r computes the
 * UNNORMALISED inverse y[j] = sum_k X[k] e^{+2 pi i jk/n} of a Hermitian
 * spectrum.  Sizes must be powers of two (the only sizes the reference's
 * wrapper produces, correlation_lib.py:54).  Arithmetic is float, twiddles
 * are computed in double and rounded once.  Unlike real FFTW with
 * FFTW_MEASURE, planning never writes to the arrays it is given.
 */
#ifndef SEISMIC_ORACLE_FFTW3_SHIM_H
#define SEISMIC_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct shim_fftwf_plan_s *fftwf_plan;

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
void fftwf_cleanup(void);

#ifdef __cplusplus
}
#endif

#endif
