/*
 * FFTW-3 API subset over the oracle's FP64 DFT (oracle/fft64.c).
 *
 * TEST INFRASTRUCTURE ONLY.  FFTW 3 (unpinned; linked by the reference as
 * -lfftw3 -lfftw3f, src/makefile:7) is absent from this image.  This header
 * declares exactly the FFTW calls that the reference's CPU method layer
 * src/FFTapps.c makes (plan_dft_1d, plan_dft_r2c_1d, plan_dft_c2r_1d, execute,
 * destroy_plan, malloc, free — double and single precision), with FFTW's
 * published semantics: unnormalised transforms, FFTW_FORWARD = -1,
 * FFTW_BACKWARD = +1, r2c/c2r on n/2+1 complex bins, plans bound to their
 * arrays.  It lets src/FFTapps.c compile unmodified into oracle/_ref/.  The
 * single-precision entry points transform in FP64 and round on output.
 */
#ifndef FASTPCC_FFTW_SHIM_H
#define FASTPCC_FFTW_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
typedef float _Complex fftwf_complex;
#else
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
#endif

typedef struct fftw_shim_plan_s *fftw_plan;
typedef struct fftw_shim_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif
#endif
