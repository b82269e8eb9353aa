// FP64 analytic signals of selected rows (see precise.cuh).
#include <cmath>

#include "precise.cuh"

namespace fpcc {
namespace {

struct Dft64Consts {
  double s3;           // sin(2 pi / 3)
  double c1, c2;       // cos(2 pi / 5), cos(4 pi / 5)
  double s1, s2;       // sin(2 pi / 5), sin(4 pi / 5)
};

__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 dscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// i * a
__device__ __forceinline__ double2 dmuli(double2 a) { return make_double2(-a.y, a.x); }

// v <- DFT_R(v) with kernel exp(DIR 2 pi i jk / R), natural output order.
template <int R, int DIR>
__device__ __forceinline__ void dft64(double2* v, const Dft64Consts& k) {
  if constexpr (R == 2) {
    const double2 a = v[0], b = v[1];
    v[0] = dadd(a, b);
    v[1] = dsub(a, b);
  } else if constexpr (R == 3) {
    const double2 t1 = dadd(v[1], v[2]);
    const double2 t2 = dsub(v[0], dscale(t1, 0.5));
    const double2 t3 = dmuli(dscale(dsub(v[1], v[2]), DIR * k.s3));
    v[0] = dadd(v[0], t1);
    v[1] = dadd(t2, t3);
    v[2] = dsub(t2, t3);
  } else if constexpr (R == 4) {
    const double2 a = dadd(v[0], v[2]), b = dsub(v[0], v[2]);
    const double2 c = dadd(v[1], v[3]);
    const double2 d = dmuli(dscale(dsub(v[1], v[3]), (double)DIR));
    v[0] = dadd(a, c);
    v[2] = dsub(a, c);
    v[1] = dadd(b, d);
    v[3] = dsub(b, d);
  } else {   // R == 5
    const double2 a1 = dadd(v[1], v[4]), a2 = dadd(v[2], v[3]);
    const double2 b1 = dsub(v[1], v[4]), b2 = dsub(v[2], v[3]);
    const double2 x0 = v[0];
    const double2 p1 = dadd(x0, dadd(dscale(a1, k.c1), dscale(a2, k.c2)));
    const double2 p2 = dadd(x0, dadd(dscale(a1, k.c2), dscale(a2, k.c1)));
    const double2 q1 = dmuli(dscale(dadd(dscale(b1, k.s1), dscale(b2, k.s2)), (double)DIR));
    const double2 q2 = dmuli(dscale(dsub(dscale(b1, k.s2), dscale(b2, k.s1)), (double)DIR));
    v[0] = dadd(x0, dadd(a1, a2));
    v[1] = dadd(p1, q1);
    v[4] = dsub(p1, q1);
    v[2] = dadd(p2, q2);
    v[3] = dsub(p2, q2);
  }
}

int grid_of(int64_t work) {
  int64_t b = (work + 255) / 256;
  const int64_t cap = 152 * 16;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

template <int R, int DIR>
__global__ void __launch_bounds__(256) k_pass64(const double2* __restrict__ in, double2* __restrict__ out, int n,
                                                int Ns, int nrows, const double2* __restrict__ tw, Dft64Consts kc) {
  const int m = n / R;
  const int64_t total = (int64_t)m * nrows;
  const int tstride = n / (Ns * R);
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(g / m);
    const int j = (int)(g - (int64_t)row * m);
    const double2* x = in + (int64_t)row * n;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = x[j + r * m];
    const int k = j % Ns;
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        double2 w = tw[k * r * tstride];   // k r tstride < Ns R tstride = n
        if (DIR > 0) w.y = -w.y;
        v[r] = dmul(v[r], w);
      }
    }
    dft64<R, DIR>(v, kc);
    double2* o = out + (int64_t)row * n + (int64_t)(j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) o[r * Ns] = v[r];
  }
}

__global__ void __launch_bounds__(256) k_zero_count(const float* __restrict__ x, int64_t ldx, int N,
                                                    int* __restrict__ counts) {
  __shared__ int part[8];
  const float* r = x + (int64_t)blockIdx.x * ldx;
  int c = 0;
  for (int n = threadIdx.x; n < N; n += 256) c += (__ldg(r + n) == 0.0f) ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int i = 0; i < 8; i++) s += part[i];
    counts[blockIdx.x] = s;
  }
}

__global__ void k_gather64(const float* __restrict__ x, int64_t ldx, const int* __restrict__ rows, int N, int M,
                           double2* __restrict__ out) {
  const int r = blockIdx.y;
  const float* src = x + (int64_t)rows[r] * ldx;
  double2* dst = out + (int64_t)r * M;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < M; n += gridDim.x * blockDim.x)
    dst[n] = make_double2(n < N ? (double)__ldg(src + n) : 0.0, 0.0);
}

dim3 rows_grid(int len, int nrows) {
  int gx = (len + 255) / 256;
  if (gx > 64) gx = 64;
  if (gx < 1) gx = 1;
  return dim3(gx, nrows);
}

Dft64Consts consts() {
  const double pi = 3.14159265358979323846;
  Dft64Consts k;
  k.s3 = std::sqrt(3.0) / 2.0;
  k.c1 = std::cos(2.0 * pi / 5.0);
  k.c2 = std::cos(4.0 * pi / 5.0);
  k.s1 = std::sin(2.0 * pi / 5.0);
  k.s2 = std::sin(4.0 * pi / 5.0);
  return k;
}

}  // namespace

cudaError_t launch_zero_count(const float* x, int64_t ldx, int N, int nrows, int* counts, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_zero_count<<<nrows, 256, 0, st>>>(x, ldx, N, counts);
  return cudaGetLastError();
}

cudaError_t launch_gather64(const float* x, int64_t ldx, const int* rows, int nsel, int N, int M, double2* out,
                            cudaStream_t st) {
  if (nsel <= 0) return cudaSuccess;
  if (nsel > 65535) return cudaErrorInvalidValue;
  k_gather64<<<rows_grid(M, nsel), 256, 0, st>>>(x, ldx, rows, N, M, out);
  return cudaGetLastError();
}

cudaError_t launch_pass64(int R, int dir, const double2* in, double2* out, int n, int Ns, int nrows,
                          const double2* tw, cudaStream_t st) {
  const int grid = grid_of((int64_t)(n / R) * nrows);
  const Dft64Consts kc = consts();
#define FPCC_P64(RR)                                                                               \
  if (R == RR) {                                                                                   \
    if (dir < 0) k_pass64<RR, -1><<<grid, 256, 0, st>>>(in, out, n, Ns, nrows, tw, kc);           \
    else k_pass64<RR, 1><<<grid, 256, 0, st>>>(in, out, n, Ns, nrows, tw, kc);                    \
    return cudaGetLastError();                                                                     \
  }
  FPCC_P64(2)
  FPCC_P64(3)
  FPCC_P64(4)
  FPCC_P64(5)
#undef FPCC_P64
  return cudaErrorInvalidValue;
}

}  // namespace fpcc
