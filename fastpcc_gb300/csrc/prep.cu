// Preprocessing of station windows on the device, as the reference CLI applies
// it before correlating (src/PCC_fullpair_1b.c):
//   * clipping at 4 * median(|x|) / 0.6745 (clipping :881-891, qabsmedian
//     :1179-1214): one block per window finds the exact median of |x| by a
//     radix select over the float bit patterns (non-negative floats order like
//     their bits), then clips;
//   * smooth spectral whitening (AveWhite :1065-1177): FP64 transforms of length
//     2^ceil(log2 N), the amplitude spectrum averaged over the windows of a
//     station, the reference's band-limited inverse filter with its 1000x gain
//     cap and 11-tap smoothing (computed on the host from the average), applied
//     to every window and transformed back.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/fastpcc_gb300.h"
#include "precise.cuh"

namespace fpcc {
namespace {

constexpr int kSelThreads = 512;

// k-th smallest (0-based) of |x[0..n)| by four 8-bit radix passes over the bits.
__device__ float select_abs(const float* __restrict__ x, int n, int k, unsigned* hist, unsigned* sh) {
  unsigned prefix = 0, mask = 0;
  int kk = k;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned b = __float_as_uint(fabsf(x[i]));
      if ((b & mask) == prefix) atomicAdd(&hist[(b >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned acc = 0, d = 0;
      for (; d < 256; d++) {
        if (acc + hist[d] > (unsigned)kk) break;
        acc += hist[d];
      }
      sh[0] = d;
      sh[1] = (unsigned)kk - acc;
    }
    __syncthreads();
    prefix |= sh[0] << shift;
    mask |= 255u << shift;
    kk = (int)sh[1];
    __syncthreads();
  }
  return __uint_as_float(prefix);
}

__global__ void __launch_bounds__(kSelThreads) k_clip_mad(float* __restrict__ x, int64_t ldx, int N) {
  __shared__ unsigned hist[256];
  __shared__ unsigned sh[2];
  float* r = x + (int64_t)blockIdx.x * ldx;
  const int k = N / 2;
  float med = select_abs(r, N, k, hist, sh);
  if ((N & 1) == 0) med = (med + select_abs(r, N, k - 1, hist, sh)) / 2;   // mean of the two middle values
  const float thr = (float)((double)(4 * med) / 0.6745);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float v = r[i];
    if (fabsf(v) > thr) r[i] = (v > thr) ? thr : -thr;
  }
}

// sum over rows of |X[row][b]| for bins b < nh (rows of stride n)
__global__ void k_abs_sum(const double2* __restrict__ X, int n, int nh, int nrows, double* __restrict__ H) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nh; b += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < nrows; r++) {
      const double2 v = X[(int64_t)r * n + b];
      s += hypot(v.x, v.y);
    }
    H[b] = s;
  }
}

// X[k] *= W[min(k, n-k)] (a real even filter applied to a Hermitian spectrum)
__global__ void k_apply_even(double2* X, int n, const double* __restrict__ W) {
  double2* r = X + (int64_t)blockIdx.y * n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double w = W[k <= n / 2 ? k : n - k];
    r[k].x *= w;
    r[k].y *= w;
  }
}

// out[row][i] = (float) Re a[row][i], i < N
__global__ void k_store_real(const double2* __restrict__ a, int n, float* __restrict__ out, int64_t ldo, int N) {
  const double2* r = a + (int64_t)blockIdx.y * n;
  float* o = out + (int64_t)blockIdx.y * ldo;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) o[i] = (float)r[i].x;
}

dim3 grid_rows(int len, int nrows) {
  int gx = (len + 255) / 256;
  gx = gx < 1 ? 1 : (gx > 64 ? 64 : gx);
  return dim3(gx, nrows);
}

thread_local char g_prep_err[256] = "";

int prep_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
  snprintf(g_prep_err, sizeof g_prep_err, "%s%s%s", msg, e != cudaSuccess ? ": " : "",
           e != cudaSuccess ? cudaGetErrorString(e) : "");
  return code;
}

#define PCK(call)                                          \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return prep_fail(FPCC_ECUDA, #call, e_); \
  } while (0)

// Radix-4/2 passes of a power-of-two length over rows in A (ping-pong with B).
int passes_pow2(double2* A, double2* B, int n, int nrows, int dir, const double2* tw, cudaStream_t st,
                double2** res) {
  double2* bufs[2] = {A, B};
  int cur = 0, Ns = 1, m = n;
  while (m > 1) {
    const int R = (m % 4 == 0) ? 4 : 2;
    PCK(launch_pass64(R, dir, bufs[cur], bufs[cur ^ 1], n, Ns, nrows, tw, st));
    cur ^= 1;
    Ns *= R;
    m /= R;
  }
  *res = bufs[cur];
  return 0;
}

// The reference's whitening filter from the average amplitude spectrum H (Nh
// bins of an Nz-point transform of N-sample windows): HS, the smoothed filter
// with the scales 1/(min gain) and 1/Nz^2 of the two unnormalised transforms.
void whitening_filter(std::vector<double>& H, int N, int Nz, double f1, double f2, double dt,
                      std::vector<double>& HS) {
  const int Nh = Nz / 2 + 1;
  const unsigned n1 = (unsigned)(f1 * dt * (double)Nz), n2 = (unsigned)(f2 * dt * (double)Nz);
  double g = 1.0 / H[n1];
  unsigned n = 0;
  for (; n < n1; n++) H[n] = g;
  for (; n < n2; n++) H[n] = 1.0 / H[n];
  g = 1.0 / H[n2];
  for (; n < (unsigned)Nh; n++) H[n] = g;
  double mn = H[n1], mx = H[n1];
  for (n = n1 + 1; n < n2; n++) {
    if (H[n] > mx) mx = H[n];
    else if (H[n] < mn) mn = H[n];
  }
  if (mx > 1000 * mn) mx = 1000 * mn;
  for (n = 0; n < (unsigned)Nh; n++)
    if (H[n] > mx) H[n] = mx;
  g = 1.0 / (mn * (double)Nz);
  for (n = 0; n < (unsigned)Nh; n++) H[n] *= g;
  // 11 taps 0.42 - 0.5 cos(a) + 0.08 cos(2a), a = 2 pi m / (N - 1), normalised to unit sum
  const double pi = 3.14159265358979323846;
  double win[11], s = 0;
  for (int m = 0; m < 11; m++) {
    const double a = 2 * pi * m / (double)(N - 1);
    win[m] = 0.42 - 0.5 * cos(a) + 0.08 * cos(2 * a);
    s += win[m];
  }
  for (int m = 0; m < 11; m++) win[m] /= s;
  // convolution HS[n-5] = sum_m win[m] H[n-m], mirrored at DC and at Nyquist.
  // The reference's loops skip n = 10, leaving HS[5] as its fresh allocation
  // holds it (zeros for the large buffers of long windows); it is zero here.
  HS.assign(Nh, 0.0);
  for (int k = 5; k < 10; k++) {
    double a = 0;
    int m = 0;
    for (; m <= k; m++) a += win[m] * H[k - m];
    for (; m < 11; m++) a += win[m] * H[m - k];
    HS[k - 5] = a;
  }
  for (int k = 11; k < Nh; k++) {
    double a = 0;
    for (int m = 0; m < 11; m++) a += win[m] * H[k - m];
    HS[k - 5] = a;
  }
  for (int k = Nh; k < Nh + 5; k++) {
    double a = 0;
    const int M = k - (Nh - 1);
    int m = 0;
    for (; m < M; m++) a += win[m] * H[Nh - 1 + m - M];
    for (; m < 11; m++) a += win[m] * H[k - m];
    HS[k - 5] = a;
  }
  // the filtered spectrum is scaled once more by 1/Nz before the inverse
  for (int k = 0; k < Nh; k++) HS[k] /= (double)Nz;
}

}  // namespace
}  // namespace fpcc

using namespace fpcc;

extern "C" const char* fpcc_prep_last_error(void) { return g_prep_err; }

extern "C" int fpcc_clip_rows(fpcc_ctx* ctx, float* d_x, int64_t ldx, int nrows, int N) {
  if (!ctx || !d_x || N <= 0 || ldx < N) return prep_fail(FPCC_EARG, "fpcc_clip_rows: bad arguments");
  if (nrows <= 0) return 0;
  k_clip_mad<<<nrows, kSelThreads, 0, (cudaStream_t)fpcc_get_stream(ctx)>>>(d_x, ldx, N);
  PCK(cudaGetLastError());
  return 0;
}

extern "C" int fpcc_whiten_rows(fpcc_ctx* ctx, float* d_x, int64_t ldx, int nrows, int N, double f1, double f2,
                                double dt) {
  if (!ctx || !d_x || N < 2 || ldx < N || !(f1 > 0) || !(f2 > f1) || !(dt > 0))
    return prep_fail(FPCC_EARG, "fpcc_whiten_rows: bad arguments");
  if (nrows <= 0) return 0;
  int Nz = 1;
  while (Nz < N) Nz <<= 1;
  const int Nh = Nz / 2 + 1;
  if ((unsigned)(f2 * dt * Nz) >= (unsigned)Nh)
    return prep_fail(FPCC_EARG, "fpcc_whiten_rows: the band reaches the Nyquist frequency");
  cudaStream_t st = (cudaStream_t)fpcc_get_stream(ctx);
  // FP64 scratch: rows of Nz complex in chunks of at most 256 MB per buffer
  int chunk = (int)std::max<int64_t>(1, ((int64_t)256 << 20) / ((int64_t)Nz * 16));
  if (chunk > nrows) chunk = nrows;
  if (chunk > 65535) chunk = 65535;
  double2 *A = nullptr, *B = nullptr, *tw = nullptr;
  double *dH = nullptr, *dW = nullptr;
  int *rows = nullptr;
  int rc = 0;
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    cudaFree(A); cudaFree(B); cudaFree(tw); cudaFree(dH); cudaFree(dW); cudaFree(rows);
  };
  if (cudaMalloc(&A, (size_t)chunk * Nz * 16) != cudaSuccess || cudaMalloc(&B, (size_t)chunk * Nz * 16) != cudaSuccess ||
      cudaMalloc(&tw, (size_t)Nz * 16) != cudaSuccess || cudaMalloc(&dH, (size_t)Nh * 8) != cudaSuccess ||
      cudaMalloc(&dW, (size_t)Nh * 8) != cudaSuccess || cudaMalloc(&rows, (size_t)chunk * sizeof(int)) != cudaSuccess) {
    cleanup();
    return prep_fail(FPCC_ENOMEM, "fpcc_whiten_rows: device memory");
  }
  {
    std::vector<double2> h(Nz);
    for (int t = 0; t < Nz; t++) {
      const double a = -2.0 * 3.14159265358979323846 * (double)t / (double)Nz;
      h[t] = make_double2(cos(a), sin(a));
    }
    std::vector<int> idx(chunk);
    for (int i = 0; i < chunk; i++) idx[i] = i;
    if (cudaMemcpy(tw, h.data(), (size_t)Nz * 16, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(rows, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
      cleanup();
      return prep_fail(FPCC_ECUDA, "fpcc_whiten_rows: upload");
    }
  }
  // pass 1: average amplitude spectrum
  std::vector<double> H(Nh, 0.0), part(Nh);
  for (int r0 = 0; r0 < nrows && !rc; r0 += chunk) {
    const int n = std::min(chunk, nrows - r0);
    double2* X = nullptr;
    if (launch_gather64(d_x + (int64_t)r0 * ldx, ldx, rows, n, N, Nz, A, st) != cudaSuccess ||
        (rc = passes_pow2(A, B, Nz, n, -1, tw, st, &X)))
      break;
    k_abs_sum<<<(Nh + 255) / 256, 256, 0, st>>>(X, Nz, Nh, n, dH);
    if (cudaMemcpyAsync(part.data(), dH, (size_t)Nh * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      rc = prep_fail(FPCC_ECUDA, "fpcc_whiten_rows: spectrum average");
      break;
    }
    for (int b = 0; b < Nh; b++) H[b] += part[b];
  }
  if (!rc) {
    for (int b = 0; b < Nh; b++) H[b] /= (double)nrows;
    std::vector<double> HS;
    whitening_filter(H, N, Nz, f1, f2, dt, HS);
    if (cudaMemcpy(dW, HS.data(), (size_t)Nh * 8, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = prep_fail(FPCC_ECUDA, "fpcc_whiten_rows: filter upload");
  }
  // pass 2: filter every window and transform back
  for (int r0 = 0; r0 < nrows && !rc; r0 += chunk) {
    const int n = std::min(chunk, nrows - r0);
    double2 *X = nullptr, *Y = nullptr;
    if (launch_gather64(d_x + (int64_t)r0 * ldx, ldx, rows, n, N, Nz, A, st) != cudaSuccess ||
        (rc = passes_pow2(A, B, Nz, n, -1, tw, st, &X)))
      break;
    k_apply_even<<<grid_rows(Nz, n), 256, 0, st>>>(X, Nz, dW);
    if ((rc = passes_pow2(X, X == A ? B : A, Nz, n, +1, tw, st, &Y))) break;
    k_store_real<<<grid_rows(N, n), 256, 0, st>>>(Y, Nz, d_x + (int64_t)r0 * ldx, ldx, N);
    if (cudaGetLastError() != cudaSuccess) rc = prep_fail(FPCC_ECUDA, "fpcc_whiten_rows: launch");
  }
  cleanup();
  return rc;
}
