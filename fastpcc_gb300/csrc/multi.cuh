// Analytic signals of windows of different lengths in shared launches.
//
// Bluestein's method computes DFT_N as chirp * conv(chirp * x, conj chirp) with
// the convolution done by transforms of any length M >= 2N - 1.  Windows whose
// lengths fall in the same class of M therefore share every M-point pass;
// only the chirp pre- and post-multiplications, the filter spectra and the
// analytic mask depend on each window's own N, and these kernels take them per
// row.  The analytic signal IDFT_N(mask * DFT_N(x)) runs as
//   A = pre(x); A = IFFT_M(FFT_M(A) * F_fwd); A = mask(A)
//   A = IFFT_M(FFT_M(A) * F_inv); out = post(A)
// where the forward post-chirp and the inverse pre-chirp cancel (their product
// is 1), so the middle step is a masked copy.  T is float2 or double2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpcc {

struct MultiRow {
  const float* x;        // the window's samples (real)
  float2* out;           // its analytic signal, N values
  const void* ffwd;      // M-point filter spectra (T) of the window length, forward
  const void* finv;      //   and inverse direction, including the 1/M of the inverse
  int N;
  int pad;
};

// A[r][m] = x_r[m] c_{N_r}(m, -1) for m < N_r, else 0 (rows of stride M).
template <typename T>
cudaError_t launch_multi_pre(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st);
// A[r][m] *= F_r[m], F_r the forward (inv = 0) or inverse (inv = 1) filter of row r.
template <typename T>
cudaError_t launch_multi_mul(const MultiRow* rows, int nrows, T* A, int M, int inv, cudaStream_t st);
// A[r][m] = mask_{N_r}(m) A[r][m] for m < N_r, else 0 (mask with the 1/N of the inverse).
template <typename T>
cudaError_t launch_multi_mask(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st);
// out_r[k] = A[r][k] c_{N_r}(k, +1), k < N_r.
template <typename T>
cudaError_t launch_multi_post(const MultiRow* rows, int nrows, const T* A, int M, cudaStream_t st);
// Filter rows before their forward transform: b[r][m] = conj c_{N_r}(t, dir) / M at
// t = m (m < N_r) and t = M - m (m > M - N_r), else 0.
template <typename T>
cudaError_t launch_multi_filter(const int* Ns, int nrows, T* B, int M, int dir, cudaStream_t st);
// Per row: max |a|^2 and sum |a|^2 over the row's N values.
cudaError_t launch_multi_rowstats(const MultiRow* rows, int nrows, float* rmax, float* rsum, cudaStream_t st);

}  // namespace fpcc
