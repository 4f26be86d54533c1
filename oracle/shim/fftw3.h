/* Test-infrastructure shim: the single-precision FFTW calls of
 * src/fourier.c:78-232.  src/common.h includes <complex.h> first, so the
 * complex types are the native C99 ones, as with the real FFTW header. */
#ifndef SHIM_FFTW3_H
#define SHIM_FFTW3_H
#include <complex.h>
#include <stddef.h>
typedef float _Complex fftwf_complex;
typedef double _Complex fftw_complex;
typedef struct shim_fftwf_plan_s *fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *out,
                                 unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
fftwf_complex *fftwf_alloc_complex(size_t n);
void fftwf_free(void *p);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int nthreads);
void fftwf_cleanup_threads(void);
#endif
