// FP64 building blocks: zero-sample counts (which windows need analytic
// signals in more than FP32), FP64 gathers and FP64 Stockham passes (the
// whitening filter, the kernel spectra of the wavelet stacks).
//
// The phase methods divide the analytic signal a = x + iH{x} by its modulus.
// An FP32 transform leaves an absolute error of order 1e-7 x rms(a) on every
// sample, so where |a| is small — inside runs of zero samples (data gaps, zero
// padding) — the phase of a is lost; such windows get their analytic signals in
// double-float (multi.cuh), and these counts select them.
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

}  // namespace fpcc
