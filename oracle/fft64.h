/*
 * fft64 — FP64 discrete Fourier transform used by the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is part of the oracle that the parity
 * tests, the smoke check and the CPU-baseline leg of the benchmark use as a
 * checker.  Nothing in the product library links or calls it.
 *
 * The reference (FastPCC, src/FFTapps.c) obtains every transform from FFTW 3
 * (unpinned version, linked as -lfftw3 -lfftw3f in src/makefile:7).  FFTW is not
 * present here, so the oracle restates the transform FFTW computes — the plain
 * unnormalised DFT
 *     X[k] = sum_n x[n] * exp(sign * 2*pi*i*n*k / N),   sign = -1 forward, +1 backward
 * — with an autosorting (Stockham) mixed-radix algorithm for 2/3/4/5/7-smooth N
 * and Bluestein's chirp-z algorithm for every other N.  All arithmetic is FP64
 * with twiddles from cos/sin of exact rational angles.
 */
#ifndef FASTPCC_ORACLE_FFT64_H
#define FASTPCC_ORACLE_FFT64_H

#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

/* In-place complex DFT of length n (unnormalised).  sign = -1 forward, +1 backward.
 * Thread-safe: plans are cached per (n) behind a lock.  Returns 0 on success. */
int fft64_c2c(double complex *x, unsigned n, int sign);

/* Real-input forward DFT: y[0..n/2] = DFT(x)[0..n/2] (FFTW r2c layout). */
int fft64_r2c(double complex *y, const double *x, unsigned n);

/* Hermitian-input backward DFT: y[0..n-1] = real(IDFT) of the half spectrum
 * x[0..n/2] (FFTW c2r layout, unnormalised). */
int fft64_c2r(double *y, const double complex *x, unsigned n);

/* Release all cached plans. */
void fft64_cleanup(void);

#ifdef __cplusplus
}
#endif
#endif
