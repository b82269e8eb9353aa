// Fused station kernel: the whole phase-spectrum stage of one station window
// in one block — analytic signal at the window length N (DFT_N, one-sided mask
// with 1/N, IDFT_N; reference src/FFTapps.c:104-124), amplitude normalisation
// (:178-205 and the GPU rules of src/ccs_cuda.cu), zero padding and DFT_Nz —
// with compile-time radix schedules for both lengths.  The window length varies
// per workload, so the host instantiates this template at run time (NVRTC) for
// each (N, Nz) it meets; it is written to compile both that way and with nvcc.
#pragma once

#include "fft_core.cuh"

namespace fpcc {

struct FusedArgs {
  const float* x;      // rows of N samples
  long long ldx;
  int nrows;
  int rule;            // amplitude rule (0 F_REG, 1 D_REG, 2 PURE, 3 THRESH, 4 SUMTHR)
  int fmt;             // 0 float2, 1 half2, 2 block-scaled int16 spectra (header + short2)
  void* out;           // rows of Nz bins
  long long ldo;
};

template <int... Rs>
__host__ __device__ constexpr int fused_len(Radices<Rs...>) {
  return prod_radices<Rs...>();
}

__host__ __device__ constexpr int fused_padded(int n) { return n + (n >> 5) + 1; }
__host__ __device__ constexpr int fused_max(int a, int b) { return a > b ? a : b; }

__device__ __forceinline__ float fused_factor(int rule, float m2, float eps) {
  if (rule == 0) {
    const float f = 1.0f / (sqrtf(m2) + eps);
    return (f >= 1.17549435e-38f && f <= 3.40282347e+38f) ? f : 0.0f;
  }
  if (rule == 1) {
    const float f = rsqrtf(m2 + eps);
    return (f >= 1.17549435e-38f && f <= 3.40282347e+38f) ? f : 0.0f;
  }
  return (m2 > eps) ? rsqrtf(m2) : 0.0f;
}

template <int T, typename RADN, typename RADZ>
__global__ void __launch_bounds__(T, 1) k_station_fused(FusedArgs a) {
  constexpr int N = fused_len(RADN{});
  constexpr int NZ = fused_len(RADZ{});
  constexpr int NMAX = fused_max(N, NZ);
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* nlo = s + fused_padded(NMAX);
  float2* nhi = nlo + 128;
  float2* zlo = nhi + (N + 127) / 128;
  float2* zhi = zlo + 128;
  float* red = reinterpret_cast<float*>(zhi + (NZ + 127) / 128);
  build_twiddles(nlo, nhi, N);
  build_twiddles(zlo, zhi, NZ);
  const int row = blockIdx.x;
  const float* x = a.x + (long long)row * a.ldx;
  for (int n = threadIdx.x; n < N; n += T) s[PADI(n)] = make_float2(__ldg(x + n), 0.0f);
  __syncthreads();
  ct_fft<-1, T, 1>(s, 1, 0, TwTab{nlo, nhi}, RADN{});
  {
    const float d = 1.0f / (float)N;
    constexpr int half = (N + 1) >> 1;
    for (int k = threadIdx.x; k < N; k += T) {
      float f;
      if (k == 0) f = d;
      else if (k < half) f = 2.0f * d;
      else if (!(N & 1) && k == (N >> 1)) f = d;
      else f = 0.0f;
      s[PADI(k)] = cscale(s[PADI(k)], f);
    }
  }
  __syncthreads();
  ct_fft<+1, T, 1>(s, 1, 0, TwTab{nlo, nhi}, RADN{});
  // row statistic: max |a|^2, or sum |a|^2 for rule 4
  float st = 0.0f;
  for (int n = threadIdx.x; n < N; n += T) {
    const float2 v = s[PADI(n)];
    const float m2 = v.x * v.x + v.y * v.y;
    st = (a.rule == 4) ? st + m2 : fmaxf(st, m2);
  }
  st = (a.rule == 4) ? warp_sum(st) : warp_max(st);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = st;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = (threadIdx.x < T / 32) ? red[threadIdx.x] : 0.0f;
    v = (a.rule == 4) ? warp_sum(v) : warp_max(v);
    if (threadIdx.x == 0) red[32] = v;
  }
  __syncthreads();
  const float ref = red[32];
  float eps;
  if (a.rule == 0) eps = (float)(1e-6 * sqrt((double)ref));
  else if (a.rule == 2) eps = 0.0f;
  else eps = 1e-6f * ref;
  for (int n = threadIdx.x; n < N; n += T) {
    const float2 v = s[PADI(n)];
    s[PADI(n)] = cscale(v, fused_factor(a.rule, v.x * v.x + v.y * v.y, eps));
  }
  for (int n = N + threadIdx.x; n < NZ; n += T) s[PADI(n)] = make_float2(0.0f, 0.0f);
  __syncthreads();
  ct_fft<-1, T, 1>(s, 1, 0, TwTab{zlo, zhi}, RADZ{});
  if (a.fmt == 2) {
    store_i16_row<T>(s, NZ, reinterpret_cast<char*>(a.out) + (long long)row * a.ldo * 4, red);
  } else if (a.fmt == 1) {
    __half2* o = reinterpret_cast<__half2*>(a.out) + (long long)row * a.ldo;
    for (int k = threadIdx.x; k < NZ; k += T) o[k] = __float22half2_rn(s[PADI(k)]);
  } else {
    float2* o = reinterpret_cast<float2*>(a.out) + (long long)row * a.ldo;
    for (int k = threadIdx.x; k < NZ; k += T) o[k] = s[PADI(k)];
  }
}

// Shared memory of k_station_fused in bytes.
__host__ __device__ constexpr long long fused_smem_bytes(int N, int NZ) {
  return ((long long)fused_padded(fused_max(N, NZ)) + 128 + (N + 127) / 128 + 128 + (NZ + 127) / 128) * 8 +
         34 * 4;
}

}  // namespace fpcc
