// Wavelet PCC device pipeline (see wpcc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wavelet.h"

namespace fpcc {

struct WpccPlanDev {
  int N = 0;
  int Nz = 0;
  int S = 0;
  int Ls0 = 0;
  int lag0 = 0, L = 0;
  int rule = 1;          // AMP_D_REG (CPU path) or AMP_THRESH (GPU path)
  int filt_conj = 0;     // 1: bands use conj(W_s) as the GPU path does (src/ccs_cuda.cu:881-882)
  float C = 0.f;         // output scale
  const float2* d_W = nullptr;   // S x Nz wavelet spectra
  const float* d_a = nullptr;    // S weights 1/(scale_s Nz)
};

int wpcc_choose_nz(const WpccSetup& su, unsigned N, int nz_mode);
cudaError_t wpcc_filters(const WaveletFamily& wf, int Nz, float2* d_W, float2* d_tmp_T, float2* d_stage,
                         cudaStream_t st);
cudaError_t wpcc_station(const WpccPlanDev& pl, const float* d_x, int64_t ldx, int nrows, void* d_P, int fmt,
                         float2* d_X, float2* d_T, float2* d_band, float* d_rowmax, int chunk_sw, cudaStream_t st);
cudaError_t wpcc_pairs(const WpccPlanDev& pl, const void* d_P, int fmt, const int2* d_pairs, int npairs,
                       float* d_y, int64_t ldy, float2* d_Y, float2* d_T, int chunk_p, cudaStream_t st);

}  // namespace fpcc
