// Analytic signals of windows of different lengths in shared launches (see multi.cuh).
#include "multi.cuh"

#include <algorithm>

namespace fpcc {
namespace {

__device__ __forceinline__ float2 mk(float a, float b, float2*) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b, double2*) { return make_double2(a, b); }

template <typename T>
__device__ __forceinline__ T zero() {
  return mk(0, 0, (T*)nullptr);
}

template <typename T>
__device__ __forceinline__ T mul(T a, T b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x, (T*)nullptr);
}

template <typename T>
__device__ __forceinline__ T cvt(double2 v) {
  return mk(v.x, v.y, (T*)nullptr);
}

// Im h(n), 0 < n < N, of h = IDFT_N(mask): for even N, (2/N) cot(pi n / N) at
// odd n and 0 at even n; for odd N, (1/N) (cos(pi n/N) - (-1)^n) / sin(pi n/N),
// written with half angles as cot(pi n / 2N) / N at odd n and -tan(pi n / 2N) / N
// at even n (no cancellation; the angles lie in (0, pi/2)).
__device__ __forceinline__ double hilbert_im(int n, int N) {
  double s, c;
  if (N & 1) {
    sincospi((double)n / (2.0 * (double)N), &s, &c);
    return (n & 1) ? c / (s * (double)N) : -s / (c * (double)N);
  }
  if (!(n & 1)) return 0.0;
  sincospi((double)n / (double)N, &s, &c);
  return 2.0 * c / (s * (double)N);
}

__global__ void __launch_bounds__(256) k_multi_exp(MultiRow* rows) {
  __shared__ float sm[8];
  const MultiRow r = rows[blockIdx.x];
  float mx = 0.0f;
  for (int n = threadIdx.x; n < r.N; n += 256) mx = fmaxf(mx, fabsf(__ldg(r.x + n)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.0f;
    for (int w = 0; w < 8; w++) a = fmaxf(a, sm[w]);
    rows[blockIdx.x].e = (a > 0.0f) ? ilogbf(a) : kNoSignal;
  }
}

// x * 2^-e exactly (0 for a window without signal)
__device__ __forceinline__ float scaled(float x, int e) { return e == kNoSignal ? 0.0f : scalbnf(x, -e); }

template <typename T>
__global__ void k_multi_load2(const MultiRow* __restrict__ rows, int nrows, T* A, int M) {
  const int j = blockIdx.y;
  const MultiRow r0 = rows[2 * j];
  const bool two = 2 * j + 1 < nrows;
  const float* x1 = two ? rows[2 * j + 1].x : nullptr;
  const int N1 = two ? rows[2 * j + 1].N : 0;
  const int e1 = two ? rows[2 * j + 1].e : kNoSignal;
  T* a = A + (int64_t)j * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float u = (m < r0.N) ? scaled(__ldg(r0.x + m), r0.e) : 0.0f;
    const float v = (m < N1) ? scaled(__ldg(x1 + m), e1) : 0.0f;
    a[m] = mk(u, v, (T*)nullptr);
  }
}

template <typename T>
__global__ void k_multi_split(const MultiRow* __restrict__ rows, int nrows, const T* __restrict__ Z, T* B, int M) {
  using S = decltype(T::x);
  const int j = blockIdx.y;
  const bool two = 2 * j + 1 < nrows;
  const T* z = Z + (int64_t)j * M;
  const T* H0 = reinterpret_cast<const T*>(rows[2 * j].filt);
  const T* H1 = two ? reinterpret_cast<const T*>(rows[2 * j + 1].filt) : nullptr;
  T* b0 = B + (int64_t)(2 * j) * M;
  T* b1 = B + (int64_t)(2 * j + 1) * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const T p = z[m];
    const T q = z[m == 0 ? 0 : M - m];
    // X0 = (Z[m] + conj Z[-m]) / 2,  X1 = (Z[m] - conj Z[-m]) / 2i
    const T x0 = mk((p.x + q.x) * (S)0.5, (p.y - q.y) * (S)0.5, (T*)nullptr);
    b0[m] = mul(x0, H0[m]);
    if (two) {
      const T x1 = mk((p.y + q.y) * (S)0.5, (q.x - p.x) * (S)0.5, (T*)nullptr);
      b1[m] = mul(x1, H1[m]);
    }
  }
}

template <typename T>
__global__ void k_multi_store(const MultiRow* __restrict__ rows, const T* A, int M) {
  const MultiRow r = rows[blockIdx.y];
  const T* a = A + (int64_t)blockIdx.y * M;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < r.N; k += gridDim.x * blockDim.x) {
    const T v = a[k];
    r.out[k] = (r.e == kNoSignal) ? make_float2(0.0f, 0.0f)
                                  : make_float2(scalbnf((float)v.x, r.e), scalbnf((float)v.y, r.e));
  }
}

__global__ void k_multi_hkernel(const int* __restrict__ Ns, double2* B, int M) {
  const int N = Ns[blockIdx.y];
  double2* b = B + (int64_t)blockIdx.y * M;
  const double inv = 1.0 / (double)M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    if (m == 0) re = inv;
    else if (m < N) im = hilbert_im(m, N) * inv;
    else if (m > M - N) im = hilbert_im(N - M + m, N) * inv;
    b[m] = make_double2(re, im);
  }
}

template <typename T>
__global__ void k_multi_convert(const double2* __restrict__ src, T* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = cvt<T>(src[i]);
}

__global__ void __launch_bounds__(256) k_multi_rowstats(const MultiRow* __restrict__ rows, float* rmax,
                                                        float* rsum) {
  __shared__ float sm[8], ss[8];
  const MultiRow r = rows[blockIdx.x];
  float mx = 0.0f, sum = 0.0f;
  for (int k = threadIdx.x; k < r.N; k += 256) {
    const float2 v = r.out[k];
    const float m2 = v.x * v.x + v.y * v.y;
    mx = fmaxf(mx, m2);
    sum += m2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
  }
  if ((threadIdx.x & 31) == 0) { sm[threadIdx.x >> 5] = mx; ss[threadIdx.x >> 5] = sum; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.0f, b = 0.0f;
    for (int w = 0; w < 8; w++) { a = fmaxf(a, sm[w]); b += ss[w]; }
    rmax[blockIdx.x] = a;
    rsum[blockIdx.x] = b;
  }
}

dim3 grid2(int len, int nrows) {
  int gx = (len + 255) / 256;
  gx = gx < 1 ? 1 : (gx > 64 ? 64 : gx);
  return dim3(gx, nrows);
}

}  // namespace

cudaError_t launch_multi_exp(MultiRow* rows, int nrows, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_multi_exp<<<nrows, 256, 0, st>>>(rows);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_multi_load2(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const int np = (nrows + 1) / 2;
  if (np > 65535) return cudaErrorInvalidValue;
  k_multi_load2<T><<<grid2(M, np), 256, 0, st>>>(rows, nrows, A, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_split(const MultiRow* rows, int nrows, const T* Z, T* B, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const int np = (nrows + 1) / 2;
  if (np > 65535) return cudaErrorInvalidValue;
  k_multi_split<T><<<grid2(M, np), 256, 0, st>>>(rows, nrows, Z, B, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_store(const MultiRow* rows, int nrows, const T* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_store<T><<<grid2(M / 2, nrows), 256, 0, st>>>(rows, A, M);
  return cudaGetLastError();
}
cudaError_t launch_multi_hkernel(const int* Ns, int nrows, double2* B, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_hkernel<<<grid2(M, nrows), 256, 0, st>>>(Ns, B, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_convert(const double2* src, T* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int g = (int)std::min<int64_t>(4096, (n + 255) / 256);
  k_multi_convert<T><<<g, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}
cudaError_t launch_multi_rowstats(const MultiRow* rows, int nrows, float* rmax, float* rsum, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_multi_rowstats<<<nrows, 256, 0, st>>>(rows, rmax, rsum);
  return cudaGetLastError();
}

template cudaError_t launch_multi_load2<float2>(const MultiRow*, int, float2*, int, cudaStream_t);
template cudaError_t launch_multi_load2<double2>(const MultiRow*, int, double2*, int, cudaStream_t);
template cudaError_t launch_multi_split<float2>(const MultiRow*, int, const float2*, float2*, int, cudaStream_t);
template cudaError_t launch_multi_split<double2>(const MultiRow*, int, const double2*, double2*, int, cudaStream_t);
template cudaError_t launch_multi_store<float2>(const MultiRow*, int, const float2*, int, cudaStream_t);
template cudaError_t launch_multi_store<double2>(const MultiRow*, int, const double2*, int, cudaStream_t);
template cudaError_t launch_multi_convert<float2>(const double2*, float2*, int64_t, cudaStream_t);
template cudaError_t launch_multi_convert<double2>(const double2*, double2*, int64_t, cudaStream_t);

}  // namespace fpcc
