// Analytic signals of windows of different lengths in shared launches (see multi.cuh).
#include "multi.cuh"

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

// exp(dir i pi n^2 / N), n^2 reduced mod 2N exactly
__device__ __forceinline__ float2 chirp_of(long long n, int N, int dir, float2*) {
  const long long q = (n * n) % (2LL * N);
  float s, c;
  sincospif((float)q / (float)N, &s, &c);
  return make_float2(c, dir * s);
}
__device__ __forceinline__ double2 chirp_of(long long n, int N, int dir, double2*) {
  const long long q = (n * n) % (2LL * N);
  double s, c;
  sincospi((double)q / (double)N, &s, &c);
  return make_double2(c, dir * s);
}

template <typename T>
__global__ void k_multi_pre(const MultiRow* __restrict__ rows, T* A, int M) {
  const MultiRow r = rows[blockIdx.y];
  T* a = A + (int64_t)blockIdx.y * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    T v = zero<T>();
    if (m < r.N) {
      const T c = chirp_of(m, r.N, -1, (T*)nullptr);
      const float x = __ldg(r.x + m);
      v = mk(x * c.x, x * c.y, (T*)nullptr);
    }
    a[m] = v;
  }
}

template <typename T>
__global__ void k_multi_mul(const MultiRow* __restrict__ rows, T* A, int M, int inv) {
  const MultiRow r = rows[blockIdx.y];
  const T* F = reinterpret_cast<const T*>(inv ? r.finv : r.ffwd);
  T* a = A + (int64_t)blockIdx.y * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) a[m] = mul(a[m], F[m]);
}

template <typename T>
__global__ void k_multi_mask(const MultiRow* __restrict__ rows, T* A, int M) {
  using S = decltype(T::x);
  const int N = rows[blockIdx.y].N;
  T* a = A + (int64_t)blockIdx.y * M;
  const int half = (N + 1) >> 1;
  const S d = (S)1 / (S)N;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    S f;
    if (m == 0) f = d;
    else if (m < half) f = 2 * d;
    else if (!(N & 1) && m == (N >> 1)) f = d;
    else f = 0;
    const T v = a[m];
    a[m] = (m < N) ? mk(v.x * f, v.y * f, (T*)nullptr) : zero<T>();
  }
}

template <typename T>
__global__ void k_multi_post(const MultiRow* __restrict__ rows, const T* A, int M) {
  const MultiRow r = rows[blockIdx.y];
  const T* a = A + (int64_t)blockIdx.y * M;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < r.N; k += gridDim.x * blockDim.x) {
    const T v = mul(a[k], chirp_of(k, r.N, +1, (T*)nullptr));
    r.out[k] = make_float2((float)v.x, (float)v.y);
  }
}

template <typename T>
__global__ void k_multi_filter(const int* __restrict__ Ns, T* B, int M, int dir) {
  const int N = Ns[blockIdx.y];
  T* b = B + (int64_t)blockIdx.y * M;
  const double inv = 1.0 / (double)M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    int t = -1;
    if (m < N) t = m;
    else if (m > M - N) t = M - m;
    T v = zero<T>();
    if (t >= 0) {
      const T c = chirp_of(t, N, dir, (T*)nullptr);
      v = mk(c.x * inv, -c.y * inv, (T*)nullptr);
    }
    b[m] = v;
  }
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

template <typename T>
cudaError_t launch_multi_pre(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_pre<T><<<grid2(M, nrows), 256, 0, st>>>(rows, A, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_mul(const MultiRow* rows, int nrows, T* A, int M, int inv, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_mul<T><<<grid2(M, nrows), 256, 0, st>>>(rows, A, M, inv);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_mask(const MultiRow* rows, int nrows, T* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_mask<T><<<grid2(M, nrows), 256, 0, st>>>(rows, A, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_post(const MultiRow* rows, int nrows, const T* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_post<T><<<grid2(M / 2, nrows), 256, 0, st>>>(rows, A, M);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multi_filter(const int* Ns, int nrows, T* B, int M, int dir, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_filter<T><<<grid2(M, nrows), 256, 0, st>>>(Ns, B, M, dir);
  return cudaGetLastError();
}
cudaError_t launch_multi_rowstats(const MultiRow* rows, int nrows, float* rmax, float* rsum, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_multi_rowstats<<<nrows, 256, 0, st>>>(rows, rmax, rsum);
  return cudaGetLastError();
}

template cudaError_t launch_multi_pre<float2>(const MultiRow*, int, float2*, int, cudaStream_t);
template cudaError_t launch_multi_pre<double2>(const MultiRow*, int, double2*, int, cudaStream_t);
template cudaError_t launch_multi_mul<float2>(const MultiRow*, int, float2*, int, int, cudaStream_t);
template cudaError_t launch_multi_mul<double2>(const MultiRow*, int, double2*, int, int, cudaStream_t);
template cudaError_t launch_multi_mask<float2>(const MultiRow*, int, float2*, int, cudaStream_t);
template cudaError_t launch_multi_mask<double2>(const MultiRow*, int, double2*, int, cudaStream_t);
template cudaError_t launch_multi_post<float2>(const MultiRow*, int, const float2*, int, cudaStream_t);
template cudaError_t launch_multi_post<double2>(const MultiRow*, int, const double2*, int, cudaStream_t);
template cudaError_t launch_multi_filter<float2>(const int*, int, float2*, int, int, cudaStream_t);
template cudaError_t launch_multi_filter<double2>(const int*, int, double2*, int, int, cudaStream_t);

}  // namespace fpcc
