// Analytic signals of windows of different lengths in shared launches.
//
// The analytic signal of an N-sample window, IDFT_N(mask * DFT_N(x)) with the
// mask of src/FFTapps.c:104-124 (1/N at bin 0 and, for even N, at N/2; 2/N on
// the bins in between; 0 above), is the circular convolution of x with
// h = IDFT_N(mask): Re h = delta, and Im h has a closed form (the discrete
// Hilbert kernel; see hk_value in multi.cu).  A circular convolution of length
// N equals a circular convolution of any length M >= 2N - 1 with the kernel
// laid out at offsets -(N-1)..(N-1), so windows whose lengths fall in the same
// class of M (2^a, 3 2^a or 5 2^a) share every M-point pass; only the kernel
// spectrum H_N = FFT_M(kernel) / M (real: the kernel is i times an odd real
// sequence, plus the delta) depends on each window's own N.  Two real
// windows share one forward transform (as the real and imaginary parts of one
// complex row); their spectra are separated by Hermitian symmetry and each
// multiplied by its own H_N before one inverse transform per window:
//   A = x_2j + i x_2j+1;  A = FFT_M(A);  B_r = X_r * H_{N_r};  B = IFFT_M(B);  out = B[0, N)
// 1.5 M-point transforms per window, and half a transform per new window length
// (two kernel spectra share one transform, launch_hk_rows).  Each window enters its row scaled by
// 2^-e, e the binary exponent of its largest |sample|, and its analytic signal
// leaves scaled by 2^e: exact in floating point, so results are unchanged, but
// the two windows of a row have the same magnitude, and the split's rounding
// (about 1e-7 of the row in FP32) stays at that level relative to each of them
// instead of relative to the stronger one; an all-zero window gives zeros.
// T is float2 (FP32 rows); the double-float rows have their own kernels (_df).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.cuh"

namespace fpcc {

struct MultiRow {
  const float* x;        // the window's samples (real)
  float2* out;           // its analytic signal, N values
  const void* filt;      // H_N: M-point kernel spectrum of the window length, including 1/M; real
                         // (float, or double-float as float2 hi, lo, for the double-float rows)
  int N;
  int e;                 // binary exponent of max |x| (set on the device by launch_multi_exp), kNoSignal if zero
};

constexpr int kNoSignal = -100000;

// rows[r].e = exponent of max |x_r| over N_r samples (kNoSignal for an all-zero window).
cudaError_t launch_multi_exp(MultiRow* rows, int nrows, cudaStream_t st);

// A[j][m] = x_{2j}[m] + i x_{2j+1}[m] (zero beyond each window's N and for a
// missing odd row), (nrows + 1) / 2 rows of stride M.
template <typename T>
cudaError_t launch_multi_load2(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st);
// From the transformed pairs in Z ((nrows + 1) / 2 rows): B[r][m] = X_r[m] H_r[m]
// for every row r (nrows rows of stride M).
template <typename T>
cudaError_t launch_multi_split(const MultiRow* rows, int nrows, const T* Z, T* B, int M, cudaStream_t st);
// out_r[k] = A[r][k], k < N_r (rounded to float2).
template <typename T>
cudaError_t launch_multi_store(const MultiRow* rows, int nrows, const T* A, int M, cudaStream_t st);
// Kernel spectra, two window lengths per M-point row.  launch_hk_rows writes
// (nk + 1) / 2 double-float rows B[j] = g_A + i g_B for the lengths Ns[2j],
// Ns[2j + 1] (g_N[m] = Im h(m) / M for 0 < m < N, g_N[M - m] = -g_N[m], else 0;
// T: nk FP64 tables of hk_table_len(M) entries); after their forward transform Z,
// launch_hk_extract writes the real spectra H_k = 1/M -+ (Im, Re) Z, kernel k at
// out + k M (double-float float2 when df_out, else float).
int hk_table_len(int M);
cudaError_t launch_hk_rows(const int* Ns, int nk, double2* T, float4* B, int M, cudaStream_t st);
cudaError_t launch_hk_extract(const float4* Z, int nk, int M, bool df_out, void* out, cudaStream_t st);
// dst[i] = src[i] rounded to T (n values).
template <typename T>
cudaError_t launch_multi_convert(const double2* src, T* dst, int64_t n, cudaStream_t st);
// Double-float (float4 = re.hi, im.hi, re.lo, im.lo) variants for the windows
// that need more than FP32 (dfloat.cuh): load, split and store as above, one
// radix-R (2, 3, 4, 5, 16) Stockham pass, and double -> double-float conversion.
struct DfConsts {
  df s3, c1, c2, s1, s2;   // sin(2 pi/3), cos(2 pi/5), cos(4 pi/5), sin(2 pi/5), sin(4 pi/5)
  df c8, s8, r2;           // cos(pi/8), sin(pi/8), sqrt(1/2) (radix 16)
};
cudaError_t launch_multi_load2_df(const MultiRow* rows, int nrows, float4* A, int M, cudaStream_t st);
cudaError_t launch_multi_split_df(const MultiRow* rows, int nrows, const float4* Z, float4* B, int M,
                                  cudaStream_t st);
cudaError_t launch_multi_store_df(const MultiRow* rows, int nrows, const float4* A, int M, cudaStream_t st);
cudaError_t launch_pass_df(int R, int dir, const float4* in, float4* out, int n, int Ns, int nrows, const float4* tw,
                           const DfConsts& kc, cudaStream_t st);
cudaError_t launch_df_from_double(const double2* src, float4* dst, int n, cudaStream_t st);
// Per row: max |a|^2 and sum |a|^2 over the row's N values.
cudaError_t launch_multi_rowstats(const MultiRow* rows, int nrows, float* rmax, float* rsum, cudaStream_t st);

}  // namespace fpcc
