// Four-step transforms for lengths above the in-block menu.
//
// For n = n1 * n2 (input index j = j1*n2 + j2, output k = k1 + n1*k2):
//   column kernel: for each j2, T[k1*n2 + j2] = W_n^(dir*j2*k1) * DFT_n1(x[j1*n2 + j2])[k1]
//   row kernel:    for each k1, X[k1 + n1*k2] = DFT_n2(T[k1*n2 + .])[k2]
// Each kernel keeps C vectors in shared memory and moves C-element segments, so
// global accesses stay coalesced; load and store stages carry the fused
// per-method pre/post-processing.
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "kernels.cuh"

namespace fpcc {

__device__ __forceinline__ bool isnormal_pos(float v) { return v >= FLT_MIN && v <= FLT_MAX; }

// Amplitude normalisation of a row from its statistic `ref` (max |x|^2): the
// rule's epsilon, then the factor of a sample of |x|^2 = m2.
__device__ __forceinline__ float eps_of(int rule, float ref) {
  if (rule == AMP_F_REG) return (float)(1e-6 * sqrt((double)ref));
  if (rule == AMP_PURE) return 0.0f;
  return 1e-6f * ref;
}

__device__ __forceinline__ float factor_of(int rule, float m2, float eps) {
  if (rule == AMP_F_REG) {
    const float f = 1.0f / (sqrtf(m2) + eps);
    return isnormal_pos(f) ? f : 0.0f;
  }
  if (rule == AMP_D_REG) {
    const float f = rsqrtf(m2 + eps);
    return isnormal_pos(f) ? f : 0.0f;
  }
  return (m2 > eps) ? rsqrtf(m2) : 0.0f;
}

// Column-kernel input modes.
enum ColMode : int {
  COL_REAL = 0,     // float rows, zero beyond N
  COL_SIGN = 1,     // 1-bit signs of float rows, zero beyond N
  COL_PHASE = 2,    // analytic-signal rows (float2), amplitude-normalised, zero beyond N
  COL_COMPLEX = 3,  // float2 rows (all n values)
  COL_PAIR = 4,     // packed Hermitian cross-spectrum of a station pair (pair stage)
  COL_PRODUCT = 5,  // float2 rows times a per-row-group filter spectrum (wavelet bands)
  COL_NORMALISE = 6 // float2 rows amplitude-normalised with a row statistic (all n values)
};

// Row-kernel output modes.
enum RowMode : int {
  ROW_SPEC = 0,     // spectrum row (full or bins 0..n/2), F32/F16
  ROW_COMPLEX = 1,  // complex row (float2), optional per-row max |x|^2 (atomic)
  ROW_LAGS = 2      // pair stage: real lags from the half-length inverse transform
};

struct LargeArgs {
  int n, n1, n2;      // n = n1 * n2
  int dir;            // -1 forward, +1 inverse
  int nrows;          // rows (transforms) in this launch
  // column input
  int cmode;
  const void* in;
  int64_t ldin;
  int N;              // valid input samples per row (zero padding beyond)
  int in_off;         // COL_REAL / COL_SIGN: sample 0 of the row sits at index in_off
  int rule;           // COL_PHASE / COL_NORMALISE amplitude rule
  const float* rowstat;
  int sign_ge;
  // COL_PAIR
  const void* spec;
  int64_t ldspec;
  int fmt;
  int herm;
  const int2* pairs;
  int Nz;             // correlation length (n = Nz / 2 for COL_PAIR)
  // COL_PRODUCT: row r uses filter filt[(r / rows_per_filter) ... ] — see large.cu
  const float2* filt;
  int64_t ldfilt;
  int filt_of_row_div; // row r reads input row r / div and filter row r % div
  int filt_conj;       // multiply by conj(filter) instead
  float in_scale;
  // intermediate
  float2* T;          // nrows x n
  // row output
  int rmode;
  void* out;
  int64_t ldo;
  int out_fmt;
  int out_half;       // ROW_SPEC: store bins 0..n/2 only
  float* rowmax;      // ROW_COMPLEX: per-row max |x|^2 (atomicMax on the bit pattern), may be null
  // ROW_LAGS
  int lag0, L;
  float scale;
  int norm;
  const double* energy;
  int64_t ldE;
  float* y;
  int64_t ldy;
  // packed pair stage: per-row product rows, N, lags, energies and output (COL_PAIR / ROW_LAGS)
  const PairDesc* desc;
};

// True when n has a supported four-step decomposition; writes n1, n2.
bool large_supported(int n, int* n1, int* n2);
cudaError_t launch_large(const LargeArgs& a, cudaStream_t st);

}  // namespace fpcc
