// Direct (non-FFT) kernels: energies, PCC_v lag sums, 1-bit popcounts.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fastpcc_gb300.h"

namespace fpcc {

struct PccvArgs {
  const void* phase;   // phase signals, N complex per row (float2 or half2)
  int64_t ldp;
  int half;            // storage: 0 float2, 1 half2, 2 int16 of scale 1/32767
  const int2* pairs;   // (row of station 1, row of station 2)
  int npairs;
  int N;
  int Lag1;            // lag of output 0 (Lag1 <= Lag2)
  int L;               // number of outputs
  float v;             // power
  int norm_gpu;        // 1: divide by 2(N-|lag|); 0: by 2^(v/2)(N-|lag|)
  float* y;
  int64_t ldy;
  const fpcc_pair_desc* desc;   // packed mode: per-pair rows, N, lags, output (N, Lag1, L above: maxima)
};

struct Cc1bArgs {
  const uint32_t* bits;  // packed sign bits, ldb words per row
  int64_t ldb;
  const int2* pairs;
  int npairs;
  int N;
  int lag0;
  int L;
  float* y;              // optional normalised output (num / overlap)
  long long* num;        // optional exact numerators
  int64_t ldy;
  const fpcc_pair_desc* desc;   // packed mode (L above: the maximum); desc.y is int64 when desc_num
  int desc_num;
};

// FP64 prefix sums E[n] = sum_{m<n} x[m]^2 (N + 1 per row); `part` holds
// nrows * energy_chunks(N) doubles of chunk totals.  With tables set (rows of
// ldE >= 2 (N + 1)), each row also receives the GNCC normalisation tables of
// GnccNorm (kernels.cuh) after its sums, and E[0] = -0.0 flags them.
int energy_chunks(int N);
cudaError_t launch_energy_prefix(const float* x, int64_t ldx, int nrows, int N, double* E, int64_t ldE,
                                 double* part, bool tables, cudaStream_t st);
cudaError_t launch_pccv(const PccvArgs& a, cudaStream_t st);
cudaError_t launch_sign_bits(const float* x, int64_t ldx, int nrows, int N, uint32_t* bits, int64_t ldb,
                             int pos_ge, const int8_t* sel, cudaStream_t st);
cudaError_t launch_cc1b_popcount(const Cc1bArgs& a, cudaStream_t st);

}  // namespace fpcc
