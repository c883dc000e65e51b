/*
 * fftw3.h -- FFTW-API shim used ONLY by the test oracle.
 *
 * This header is test infrastructure: it lets the reference powspec sources
 * (which include <fftw3.h>, src/fftw_define.h:29) and the oracle's own C
 * restatement link against a double-precision FFT written for this project,
 * because libfftw3 is not available on either build machine.  It declares the
 * ten symbols the reference uses (src/fftw_define.h:48-61) with FFTW's
 * conventions: forward sign -1, unnormalised transforms, row-major
 * [n0][n1][n2/2+1] half-complex layout, c2r may clobber its input.
 *
 * Nothing in the GPU product includes this file.
 */
#ifndef PS_ORACLE_FFTW3_SHIM_H
#define PS_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct ps_shim_plan *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
void fftw_cleanup(void);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_destroy_plan(fftw_plan p);

/* Shim-only helper: 1-D complex transform of length n (sign -1 or +1),
 * unnormalised, in place on n interleaved (re, im) pairs.  Exposed so the
 * oracle's tests can check the engine against numpy directly. */
int ps_shim_cfft1d(int n, int sign, double *data);

#ifdef __cplusplus
}
#endif

#endif
