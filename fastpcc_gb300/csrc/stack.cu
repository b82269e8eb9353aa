// Stacks of correlation traces (see stack.cuh).
#include "stack.cuh"

#include <algorithm>

namespace fpcc {
namespace {

dim3 grid_cols(int n, int G) {
  int gx = (n + 255) / 256;
  gx = gx < 1 ? 1 : (gx > 4096 ? 4096 : gx);
  return dim3(gx, G);
}

__device__ __forceinline__ double2 unit_d(float2 z) {
  const double x = z.x, y = z.y;
  const double a = sqrt(x * x + y * y);
  return a > 0.0 ? make_double2(x / a, y / a) : make_double2(0.0, 0.0);
}

__global__ void k_stack_mean(const float* __restrict__ y, int64_t ldy, int K, int L, float* out, int64_t ldo) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < K; j++) s += (double)__ldg(y + ((int64_t)g * K + j) * ldy + n);
    out[(int64_t)g * ldo + n] = (float)(s / K);
  }
}

__global__ void k_stack_pws(const float2* __restrict__ a, int64_t lda, const float* __restrict__ y, int64_t ldy,
                            int K, int L, double nu, float* out, int64_t ldo) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x) {
    double s = 0.0, ux = 0.0, uy = 0.0;
    for (int j = 0; j < K; j++) {
      const int64_t r = (int64_t)g * K + j;
      s += (double)__ldg(y + r * ldy + n);
      const double2 u = unit_d(a[r * lda + n]);
      ux += u.x;
      uy += u.y;
    }
    const double c = sqrt(ux * ux + uy * uy) / K;
    out[(int64_t)g * ldo + n] = (float)((s / K) * pow(c, nu));
  }
}

__global__ void k_stack_load(const float* __restrict__ y, int64_t ldy, int L, float2* X, int M) {
  const int64_t r = blockIdx.y;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x)
    X[r * M + m] = make_float2(m < L ? __ldg(y + r * ldy + m) : 0.0f, 0.0f);
}

__global__ void k_stack_xlin(float2* X, int K, int G, int M) {
  const int g = blockIdx.y;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    double sx = 0.0, sy = 0.0;
    for (int j = 0; j < K; j++) {
      const float2 v = X[((int64_t)g * K + j) * M + m];
      sx += v.x;
      sy += v.y;
    }
    X[((int64_t)G * K + g) * M + m] = make_float2((float)(sx / K), (float)(sy / K));
  }
}

__global__ void k_stack_mul(const float2* __restrict__ X, int M, const float2* __restrict__ F, float2* T) {
  const int64_t r = blockIdx.y;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float2 a = X[r * M + m], b = __ldg(F + m);
    T[r * M + m] = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
}

__global__ void k_stack_coherence(const float2* __restrict__ W, int K, int G, int L, int M, double nu,
                                  float2* Y) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < M; n += gridDim.x * blockDim.x) {
    float2 out = make_float2(0.0f, 0.0f);
    if (n < L) {
      double ux = 0.0, uy = 0.0;
      for (int j = 0; j < K; j++) {
        const double2 u = unit_d(W[((int64_t)g * K + j) * M + n]);
        ux += u.x;
        uy += u.y;
      }
      const double c = pow(sqrt(ux * ux + uy * uy) / K, nu);
      const float2 w = W[((int64_t)G * K + g) * M + n];
      out = make_float2((float)(c * w.x), (float)(c * w.y));
    }
    Y[(int64_t)g * M + n] = out;
  }
}

__global__ void k_stack_acc(const float2* __restrict__ Z, int M, const float2* __restrict__ F, float a, int first,
                            float2* R) {
  const int64_t g = blockIdx.y;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float2 z = Z[g * M + m], f = __ldg(F + m);
    const float2 p = make_float2(a * (z.x * f.x - z.y * f.y), a * (z.x * f.y + z.y * f.x));
    const float2 o = first ? make_float2(0.0f, 0.0f) : R[g * M + m];
    R[g * M + m] = make_float2(o.x + p.x, o.y + p.y);
  }
}

__global__ void k_stack_real(const float2* __restrict__ r, int L, int M, float* out, int64_t ldo) {
  const int64_t g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x)
    out[g * ldo + n] = r[g * M + n].x;
}

bool rows_ok(int rows) { return rows > 0 && rows <= 65535; }

}  // namespace

cudaError_t launch_stack_mean(const float* y, int64_t ldy, int K, int L, int G, float* out, int64_t ldo,
                              cudaStream_t st) {
  if (!rows_ok(G) || K <= 0 || L <= 0) return cudaErrorInvalidValue;
  k_stack_mean<<<grid_cols(L, G), 256, 0, st>>>(y, ldy, K, L, out, ldo);
  return cudaGetLastError();
}

cudaError_t launch_stack_pws(const float2* a, int64_t lda, const float* y, int64_t ldy, int K, int L, int G,
                             double nu, float* out, int64_t ldo, cudaStream_t st) {
  if (!rows_ok(G) || K <= 0 || L <= 0) return cudaErrorInvalidValue;
  k_stack_pws<<<grid_cols(L, G), 256, 0, st>>>(a, lda, y, ldy, K, L, nu, out, ldo);
  return cudaGetLastError();
}

cudaError_t launch_stack_load(const float* y, int64_t ldy, int rows, int L, float2* X, int M, cudaStream_t st) {
  if (!rows_ok(rows)) return cudaErrorInvalidValue;
  k_stack_load<<<grid_cols(M, rows), 256, 0, st>>>(y, ldy, L, X, M);
  return cudaGetLastError();
}

cudaError_t launch_stack_xlin(float2* X, int K, int G, int M, cudaStream_t st) {
  if (!rows_ok(G)) return cudaErrorInvalidValue;
  k_stack_xlin<<<grid_cols(M, G), 256, 0, st>>>(X, K, G, M);
  return cudaGetLastError();
}

cudaError_t launch_stack_mul(const float2* X, int rows, int M, const float2* F, float2* T, cudaStream_t st) {
  if (!rows_ok(rows)) return cudaErrorInvalidValue;
  k_stack_mul<<<grid_cols(M, rows), 256, 0, st>>>(X, M, F, T);
  return cudaGetLastError();
}

cudaError_t launch_stack_coherence(const float2* W, int K, int G, int L, int M, double nu, float2* Y,
                                   cudaStream_t st) {
  if (!rows_ok(G)) return cudaErrorInvalidValue;
  k_stack_coherence<<<grid_cols(M, G), 256, 0, st>>>(W, K, G, L, M, nu, Y);
  return cudaGetLastError();
}

cudaError_t launch_stack_acc(const float2* Z, int G, int M, const float2* F, float a, int first, float2* R,
                             cudaStream_t st) {
  if (!rows_ok(G)) return cudaErrorInvalidValue;
  k_stack_acc<<<grid_cols(M, G), 256, 0, st>>>(Z, M, F, a, first, R);
  return cudaGetLastError();
}

cudaError_t launch_stack_real(const float2* r, int G, int L, int M, float* out, int64_t ldo, cudaStream_t st) {
  if (!rows_ok(G)) return cudaErrorInvalidValue;
  k_stack_real<<<grid_cols(L, G), 256, 0, st>>>(r, L, M, out, ldo);
  return cudaGetLastError();
}

}  // namespace fpcc
