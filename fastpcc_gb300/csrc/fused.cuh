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

// From the analytic spectrum in s[0..N) (mask and 1/N applied): IDFT_N, the
// amplitude normalisation, zero padding, DFT_Nz and the store.
template <int T, typename RADN, typename RADZ>
__device__ __forceinline__ void fused_tail(const FusedArgs& a, float2* s, const TwTab& twN, const TwTab& twZ,
                                           float* red, int row) {
  constexpr int N = fused_len(RADN{});
  constexpr int NZ = fused_len(RADZ{});
  ct_fft<+1, T, 1>(s, 1, 0, twN, RADN{});
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
  ct_fft<-1, T, 1>(s, 1, 0, twZ, RADZ{});
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
  fused_tail<T, RADN, RADZ>(a, s, TwTab{nlo, nhi}, TwTab{zlo, zhi}, red, row);
}

// Even N: the DFT_N of the real window as an N/2-point complex transform of
// z[m] = x[2m] + i x[2m+1] (radices RADH), then, for the non-negative
// frequencies the analytic mask keeps,
//   X[k] = (Z[k] + conj(Z[N/2-k])) / 2 - i w^k (Z[k] - conj(Z[N/2-k])) / 2,  w = exp(-2 pi i / N),
// with X[0] = Re Z[0] + Im Z[0] and X[N/2] = Re Z[0] - Im Z[0]; the mask (1/N
// at 0 and N/2, 2/N between, 0 above) is applied in the same pass.  Thread k
// forms the pair (k, N/2 - k), so the pass is in place without a barrier.
template <int T, typename RADH, typename RADN, typename RADZ>
__global__ void __launch_bounds__(T, 1) k_station_fused_real(FusedArgs a) {
  constexpr int NH = fused_len(RADH{});
  constexpr int N = fused_len(RADN{});
  static_assert(N == 2 * NH, "half-length schedule");
  constexpr int NZ = fused_len(RADZ{});
  constexpr int NMAX = fused_max(N, NZ);
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* nlo = s + fused_padded(NMAX);
  float2* nhi = nlo + 128;
  float2* zlo = nhi + (N + 127) / 128;
  float2* zhi = zlo + 128;
  float2* hlo = zhi + (NZ + 127) / 128;
  float2* hhi = hlo + 128;
  float* red = reinterpret_cast<float*>(hhi + (NH + 127) / 128);
  build_twiddles(nlo, nhi, N);
  build_twiddles(zlo, zhi, NZ);
  build_twiddles(hlo, hhi, NH);
  const int row = blockIdx.x;
  const float* x = a.x + (long long)row * a.ldx;
  for (int m = threadIdx.x; m < NH; m += T) s[PADI(m)] = make_float2(__ldg(x + 2 * m), __ldg(x + 2 * m + 1));
  __syncthreads();
  ct_fft<-1, T, 1>(s, 1, 0, TwTab{hlo, hhi}, RADH{});
  {
    const TwTab twN{nlo, nhi};
    const float d = 1.0f / (float)N;
    for (int k = threadIdx.x; k <= NH / 2; k += T) {
      if (k == 0) {
        const float2 z0 = s[PADI(0)];
        s[PADI(0)] = make_float2((z0.x + z0.y) * d, 0.0f);
        s[PADI(NH)] = make_float2((z0.x - z0.y) * d, 0.0f);
        continue;
      }
      const int k2 = NH - k;
      const float2 A = s[PADI(k)], B = s[PADI(k2)];
      // X[k] with w^k; X[NH-k] with w^(NH-k) = -conj(w^k)
      const float2 w = twiddle(twN, k);
      const float2 e = make_float2(A.x + B.x, A.y - B.y);          // Z[k] + conj(Z[NH-k])
      const float2 f = make_float2(A.x - B.x, A.y + B.y);          // Z[k] - conj(Z[NH-k])
      const float2 wf = cmul(w, f);
      const float2 Xk = make_float2(0.5f * (e.x + wf.y), 0.5f * (e.y - wf.x));   // (e - i w f) / 2
      // for NH-k: e' = conj(e), f' = -conj(f), w' = -conj(w): w' f' = conj(w f)
      const float2 Xk2 = make_float2(0.5f * (e.x - wf.y), 0.5f * (-e.y - wf.x));
      s[PADI(k)] = cscale(Xk, 2.0f * d);
      if (k2 != k) s[PADI(k2)] = cscale(Xk2, 2.0f * d);
    }
    for (int k = NH + 1 + threadIdx.x; k < N; k += T) s[PADI(k)] = make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  fused_tail<T, RADN, RADZ>(a, s, TwTab{nlo, nhi}, TwTab{zlo, zhi}, red, row);
}

// Shared memory of k_station_fused in bytes (half > 0: k_station_fused_real,
// with the twiddle tables of the half length as well).
__host__ __device__ constexpr long long fused_smem_bytes(int N, int NZ, int half = 0) {
  return ((long long)fused_padded(fused_max(N, NZ)) + 128 + (N + 127) / 128 + 128 + (NZ + 127) / 128 +
          (half ? 128 + (half + 127) / 128 : 0)) * 8 +
         34 * 4;
}

}  // namespace fpcc
