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

// Unit phasor z / |z| in FP32 (0 for z = 0; FP32 keeps 1e-7 relative, the sums
// over traces run in FP64).
__device__ __forceinline__ float2 unit_f(float2 z) {
  const float m2 = z.x * z.x + z.y * z.y;
  if (!(m2 > 0.0f)) return make_float2(0.0f, 0.0f);
  const float r = rsqrtf(m2);
  return make_float2(z.x * r, z.y * r);
}

// Coherence (|U| / K)^nu from U's squared modulus: nu = 2 and nu = 1 without
// the general power.
__device__ __forceinline__ double coherence(double ux, double uy, int K, double nu) {
  const double m2 = (ux * ux + uy * uy) / ((double)K * (double)K);
  if (nu == 2.0) return m2;
  if (nu == 1.0) return (double)sqrtf((float)m2);
  if (nu == 0.0) return 1.0;
  return (double)powf((float)m2, (float)(0.5 * nu));
}

__global__ void k_stack_mean(const float* __restrict__ y, int64_t ldg, int64_t ldj, int K, int L, float* out,
                             int64_t ldo) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x) {
    // four independent sums keep several loads in flight per thread
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    const float* p = y + (int64_t)g * ldg + n;
    int j = 0;
    for (; j + 4 <= K; j += 4) {
      s0 += (double)__ldg(p + (int64_t)j * ldj);
      s1 += (double)__ldg(p + (int64_t)(j + 1) * ldj);
      s2 += (double)__ldg(p + (int64_t)(j + 2) * ldj);
      s3 += (double)__ldg(p + (int64_t)(j + 3) * ldj);
    }
    for (; j < K; j++) s0 += (double)__ldg(p + (int64_t)j * ldj);
    out[(int64_t)g * ldo + n] = (float)(((s0 + s1) + (s2 + s3)) / K);
  }
}

__global__ void k_stack_pws(const float2* __restrict__ a, int64_t lda, const float* __restrict__ y, int64_t ldg,
                            int64_t ldj, int K, int L, double nu, float* out, int64_t ldo) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x) {
    double s = 0.0, ux = 0.0, uy = 0.0;
    for (int j = 0; j < K; j++) {
      const int64_t r = (int64_t)g * K + j;
      s += (double)__ldg(y + (int64_t)g * ldg + (int64_t)j * ldj + n);
      const float2 u = unit_f(a[r * lda + n]);
      ux += u.x;
      uy += u.y;
    }
    out[(int64_t)g * ldo + n] = (float)((s / K) * coherence(ux, uy, K, nu));
  }
}

__global__ void k_stack_load(const float* __restrict__ y, int64_t ldg, int64_t ldj, int K, int L, float2* X,
                             int M) {
  const int64_t r = blockIdx.y;
  const float* row = y + (r / K) * ldg + (r % K) * ldj;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x)
    X[r * M + m] = make_float2(m < L ? __ldg(row + m) : 0.0f, 0.0f);
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

__global__ void k_stack_coherence(const float2* __restrict__ W, int64_t ldw, int K, int G, int L, int M,
                                  double nu, float2* Y) {
  const int g = blockIdx.y;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < M; n += gridDim.x * blockDim.x) {
    float2 out = make_float2(0.0f, 0.0f);
    if (n < L) {
      // FP32 partial sums over runs of 32 traces, accumulated in FP64
      double ux = 0.0, uy = 0.0;
      for (int j0 = 0; j0 < K; j0 += 32) {
        float px = 0.0f, py = 0.0f;
        const int j1 = min(K, j0 + 32);
        for (int j = j0; j < j1; j++) {
          const float2 u = unit_f(W[((int64_t)g * K + j) * ldw + n]);
          px += u.x;
          py += u.y;
        }
        ux += px;
        uy += py;
      }
      const double c = coherence(ux, uy, K, nu);
      const float2 w = W[((int64_t)G * K + g) * ldw + n];
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

cudaError_t launch_stack_mean(const float* y, int64_t ldg, int64_t ldj, int K, int L, int G, float* out,
                              int64_t ldo, cudaStream_t st) {
  if (!rows_ok(G) || K <= 0 || L <= 0) return cudaErrorInvalidValue;
  k_stack_mean<<<grid_cols(L, G), 256, 0, st>>>(y, ldg, ldj, K, L, out, ldo);
  return cudaGetLastError();
}

cudaError_t launch_stack_pws(const float2* a, int64_t lda, const float* y, int64_t ldg, int64_t ldj, int K, int L,
                             int G, double nu, float* out, int64_t ldo, cudaStream_t st) {
  if (!rows_ok(G) || K <= 0 || L <= 0) return cudaErrorInvalidValue;
  k_stack_pws<<<grid_cols(L, G), 256, 0, st>>>(a, lda, y, ldg, ldj, K, L, nu, out, ldo);
  return cudaGetLastError();
}

cudaError_t launch_stack_load(const float* y, int64_t ldg, int64_t ldj, int K, int G, int L, float2* X, int M,
                              cudaStream_t st) {
  const int rows = K * G;
  if (!rows_ok(rows)) return cudaErrorInvalidValue;
  k_stack_load<<<grid_cols(M, rows), 256, 0, st>>>(y, ldg, ldj, K, L, X, M);
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

cudaError_t launch_stack_coherence(const float2* W, int64_t ldw, int K, int G, int L, int M, double nu, float2* Y,
                                   cudaStream_t st) {
  if (!rows_ok(G)) return cudaErrorInvalidValue;
  k_stack_coherence<<<grid_cols(M, G), 256, 0, st>>>(W, ldw, K, G, L, M, nu, Y);
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
