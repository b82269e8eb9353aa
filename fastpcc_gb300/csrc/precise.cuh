// FP64 analytic signals for windows that FP32 transforms cannot resolve.
//
// The phase methods divide the analytic signal a = x + iH{x} by its modulus.
// An FP32 transform leaves an absolute error of order 1e-7 x rms(a) on every
// sample, so where |a| is small — inside runs of zero samples (data gaps, zero
// padding) — the phase of a is lost and correlations of such windows drift by
// up to a few 1e-4 from the FP64 result.  These kernels recompute the analytic
// signal of selected rows in FP64 (radix-2/3/4/5 Stockham passes, Bluestein's
// chirp-z transform for other lengths) and round it to float2 afterwards, which
// keeps the relative precision of every sample; the rest of the pipeline is
// unchanged.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpcc {

// Zero samples per row (counts[r]).
cudaError_t launch_zero_count(const float* x, int64_t ldx, int N, int nrows, int* counts, cudaStream_t st);

// rows r < nsel: out[r][n] = (x[rows[r]][n], 0) for n < N, 0 for N <= n < M.
cudaError_t launch_gather64(const float* x, int64_t ldx, const int* rows, int nsel, int N, int M, double2* out,
                            cudaStream_t st);
// One radix-R Stockham pass (R in 2, 3, 4, 5) over nrows rows of n values;
// tw[t] = exp(-2 pi i t / n) in FP64.
cudaError_t launch_pass64(int R, int dir, const double2* in, double2* out, int n, int Ns, int nrows,
                          const double2* tw, cudaStream_t st);
// Analytic mask with the 1/n of the inverse (rows of stride n).
cudaError_t launch_mask64(double2* a, int n, int nrows, cudaStream_t st);
// Bluestein pieces for length N in M-point transforms, chirp c[n] = exp(dir i pi n^2 / N):
//   pre:    a[n] = in[n] c[n] (n < N), 0 (N <= n < M)        (in: rows of stride ldin)
//   mul:    a[n] *= B[n]
//   post:   out[k] = c[k] a[k] (k < N)                       (out: rows of stride ldo)
//   filter: b[m] = conj(c[m]) / M at m and M - m (|m| < N), else 0 (before its forward transform)
cudaError_t launch_blue_pre64(const double2* in, int64_t ldin, double2* a, int N, int M, int dir, int nrows,
                              cudaStream_t st);
cudaError_t launch_blue_mul64(double2* a, const double2* B, int M, int nrows, cudaStream_t st);
cudaError_t launch_blue_post64(const double2* a, int M, double2* out, int64_t ldo, int N, int dir, int nrows,
                               cudaStream_t st);
cudaError_t launch_blue_filter64(double2* b, int N, int M, int dir, cudaStream_t st);
// out[rows[r]][n] = float2(a[r][n]) for n < N (a: rows of stride lda).
cudaError_t launch_store64(const double2* a, int64_t lda, const int* rows, int nsel, int N, float2* out,
                           int64_t ldo, cudaStream_t st);

}  // namespace fpcc
