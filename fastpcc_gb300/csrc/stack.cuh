// Stacks of correlation traces over windows (linear, phase-weighted,
// time-scale phase-weighted), the device side of fpcc_stack.
//
// Groups of K traces of L samples: trace j of group g starts at
// y + g * ldg + j * ldj (so groups of adjacent rows and window-major outputs of
// the pair stage both stack in place).  The CWT of src/FWTa (complex_1D_wavelet_dec: W_s[n] = sum_l
// x[(n - c_s + l) mod L] conj(w_s[l])) and its inverse (Re_complex_1D_wavelet_rec:
// x[n] = sum_s a_s Re sum_l w_s[l] W_s[(n + c_s - l) mod L]) are circular
// convolutions of length L; they run as M-point transforms (M >= 2L - 1) with
// the L-periodic kernels laid out at offsets -(L-1)..(L-1), so any L works.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpcc {

// out[g][n] = mean_j y_gj[n] (FP64 sums).
cudaError_t launch_stack_mean(const float* y, int64_t ldg, int64_t ldj, int K, int L, int G, float* out,
                              int64_t ldo, cudaStream_t st);
// out[g][n] = mean_j y_gj * |mean_j a / |a||^nu over the group's traces (a:
// analytic signals, row g K + j of stride lda; phasors of zero modulus count as zero).
cudaError_t launch_stack_pws(const float2* a, int64_t lda, const float* y, int64_t ldg, int64_t ldj, int K, int L,
                             int G, double nu, float* out, int64_t ldo, cudaStream_t st);
// X[g K + j][m] = y_gj[m] for m < L, else 0 (rows of M complex values).
cudaError_t launch_stack_load(const float* y, int64_t ldg, int64_t ldj, int K, int G, int L, float2* X, int M,
                              cudaStream_t st);
// X[G K + g][m] = mean_j X[g K + j][m]: the spectrum of the group's linear stack.
cudaError_t launch_stack_xlin(float2* X, int K, int G, int M, cudaStream_t st);
// T[r][m] = X[r][m] F[m], rows r < rows.
cudaError_t launch_stack_mul(const float2* X, int rows, int M, const float2* F, float2* T, cudaStream_t st);
// From the inverse transforms W (rows of stride ldw; rows g K + j: the traces'
// CWT at one scale; rows G K + g: the linear stack's): Y[g][n] =
// |mean_j W/|W||^nu * W_lin[n] for n < L, 0 for L <= n < M (rows of stride M).
cudaError_t launch_stack_coherence(const float2* W, int64_t ldw, int K, int G, int L, int M, double nu, float2* Y,
                                   cudaStream_t st);
// R[g][m] (+)= a * Z[g][m] F[m] (first: assign).
cudaError_t launch_stack_acc(const float2* Z, int G, int M, const float2* F, float a, int first, float2* R,
                             cudaStream_t st);
// out[g][n] = Re r[g][n], n < L.
cudaError_t launch_stack_real(const float2* r, int G, int L, int M, float* out, int64_t ldo, cudaStream_t st);

}  // namespace fpcc
