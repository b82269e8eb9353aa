// Run-time specialisation of the fused station kernel (NVRTC).
#pragma once

#include <cuda_runtime.h>

namespace fpcc {

// Launch k_station_fused for (N, Nz) on `st`, compiling it on first use (cached
// in memory and on disk).  Returns cudaSuccess, or an error when run-time
// compilation is unavailable or the lengths do not fit one block; callers then
// use the generic path.
cudaError_t launch_station_fused(const float* x, long long ldx, int nrows, int N, int Nz, int rule, int fmt,
                                 void* out, long long ldo, cudaStream_t st);
bool fused_fits(int N, int Nz);

}  // namespace fpcc
