// Analytic signals of windows of different lengths in shared launches (see multi.cuh).
#include "multi.cuh"
#include "dfloat.cuh"

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

// Im h(n), 0 < n < N, of h = IDFT_N(mask) has closed forms: for even N,
// (2/N) cot(pi n / N) at odd n and 0 at even n; for odd N, cot(pi n / 2N) / N at
// odd n and -tan(pi n / 2N) / N at even n.  Each is +-f cot(pi m / D) with m odd
// and m <= D / 2 (D = N for even N, 2N for odd N): m = n or N - n, using
// cot(pi - a) = -cot(a) and tan(a) = cot(pi/2 - a).  The angle pi m / D, in the
// first quadrant, is the sum of pi 256 a / D and pi b / D (m = 256 a + b), whose
// sines and cosines come from FP64 tables (k_hk_tables); then
// sin = sa cb + ca sb has no cancellation, so small sines keep their relative
// precision, and cot = cos / sin.
__global__ void k_hk_tables(const int* __restrict__ Ns, int nk, double2* T, int ldt) {
  const int k = blockIdx.y;
  if (k >= nk) return;
  const int N = Ns[k];
  const int D = (N & 1) ? 2 * N : N;
  const int nt = 256 + D / 512 + 1;
  double2* t = T + (int64_t)k * ldt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    const double num = i < 256 ? (double)i : 256.0 * (double)(i - 256);
    double sn, cs;
    sincospi(num / (double)D, &sn, &cs);
    t[i] = make_double2(cs, sn);
  }
}

// +-f cot(pi m / D) for 0 < n < N (t: the length's tables); with f = c / M, c the
// closed form's factor (2/N for even N, 1/N for odd N), this is Im h(n) / M.
__device__ __forceinline__ double hk_value(int n, int N, const double2* __restrict__ t, double f) {
  int m;
  bool neg;
  if (N & 1) {
    neg = !(n & 1);
    m = neg ? N - n : n;
  } else {
    if (!(n & 1)) return 0.0;
    neg = 2 * n > N;
    m = neg ? N - n : n;
  }
  const double2 cb = __ldg(t + (m & 255)), ca = __ldg(t + 256 + (m >> 8));
  const double sn = fma(ca.y, cb.x, ca.x * cb.y);
  const double cs = fma(ca.x, cb.x, -(ca.y * cb.y));
  const double v = f * (cs / sn);
  return neg ? -v : v;
}

// Rows of two kernels each (lengths Ns[2j] and Ns[2j+1]; none for the second
// when nk is odd), double-float: B[j][m] = g_A[m] + i g_B[m] with
// g_N[m] = Im h(m) / M (0 < m < N), g_N[M - m] = -g_N[m], 0 elsewhere.
__global__ void k_hk_rows(const int* __restrict__ Ns, int nk, const double2* __restrict__ T, int ldt, float4* B,
                          int M) {
  const int j = blockIdx.y;
  const int NA = Ns[2 * j], NB = (2 * j + 1 < nk) ? Ns[2 * j + 1] : 0;
  const double2* tA = T + (int64_t)(2 * j) * ldt;
  const double2* tB = tA + ldt;
  const double fA = ((NA & 1) ? 1.0 : 2.0) / ((double)NA * (double)M);
  const double fB = NB ? ((NB & 1) ? 1.0 : 2.0) / ((double)NB * (double)M) : 0.0;
  float4* row = B + (int64_t)j * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m <= M / 2; m += gridDim.x * blockDim.x) {
    const double a = (m > 0 && m < NA) ? hk_value(m, NA, tA, fA) : 0.0;
    const double b = (m > 0 && m < NB) ? hk_value(m, NB, tB, fB) : 0.0;
    row[m] = dfc(df_from_double(a), df_from_double(b));
    if (m > 0 && M - m != m) row[M - m] = dfc(df_from_double(-a), df_from_double(-b));
  }
}

// g_N is real and odd, so FFT_M(g_N) = -i S_N with S_N real, and the kernel
// spectrum is H_N = 1/M + S_N (real; the 1/M is the transform of the delta at
// 0).  A transformed row Z = FFT(g_A + i g_B) = S_B - i S_A gives
// H_A = 1/M - Im Z and H_B = 1/M + Re Z: double-float reals (float2 hi, lo)
// or rounded to float.
template <bool DF>
__global__ void k_hk_extract(const float4* __restrict__ Z, int nk, int M, void* out) {
  const int j = blockIdx.y;
  const bool two = 2 * j + 1 < nk;
  const df c = df_from_double(1.0 / (double)M);
  const float4* z = Z + (int64_t)j * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float4 v = z[m];
    const df ha = df_sub(c, df_im(v));
    const df hb = df_add(c, df_re(v));
    if constexpr (DF) {
      float2* o = reinterpret_cast<float2*>(out);
      o[(int64_t)(2 * j) * M + m] = make_float2(ha.hi, ha.lo);
      if (two) o[(int64_t)(2 * j + 1) * M + m] = make_float2(hb.hi, hb.lo);
    } else {
      float* o = reinterpret_cast<float*>(out);
      o[(int64_t)(2 * j) * M + m] = df_to_float(ha);
      if (two) o[(int64_t)(2 * j + 1) * M + m] = df_to_float(hb);
    }
  }
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
  const S* H0 = reinterpret_cast<const S*>(rows[2 * j].filt);
  const S* H1 = two ? reinterpret_cast<const S*>(rows[2 * j + 1].filt) : nullptr;
  T* b0 = B + (int64_t)(2 * j) * M;
  T* b1 = B + (int64_t)(2 * j + 1) * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const T p = z[m];
    const T q = z[m == 0 ? 0 : M - m];
    // X0 = (Z[m] + conj Z[-m]) / 2,  X1 = (Z[m] - conj Z[-m]) / 2i
    const T x0 = mk((p.x + q.x) * (S)0.5, (p.y - q.y) * (S)0.5, (T*)nullptr);
    const S h0 = H0[m];
    b0[m] = mk(x0.x * h0, x0.y * h0, (T*)nullptr);
    if (two) {
      const T x1 = mk((p.y + q.y) * (S)0.5, (q.x - p.x) * (S)0.5, (T*)nullptr);
      const S h1 = H1[m];
      b1[m] = mk(x1.x * h1, x1.y * h1, (T*)nullptr);
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

template <typename T>
__global__ void k_multi_convert(const double2* __restrict__ src, T* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = cvt<T>(src[i]);
}

// ---- double-float (float4) variants of the row kernels and the radix passes
__global__ void k_multi_load2_df(const MultiRow* __restrict__ rows, int nrows, float4* A, int M) {
  const int j = blockIdx.y;
  const MultiRow r0 = rows[2 * j];
  const bool two = 2 * j + 1 < nrows;
  const float* x1 = two ? rows[2 * j + 1].x : nullptr;
  const int N1 = two ? rows[2 * j + 1].N : 0;
  const int e1 = two ? rows[2 * j + 1].e : kNoSignal;
  float4* a = A + (int64_t)j * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float u = (m < r0.N) ? scaled(__ldg(r0.x + m), r0.e) : 0.0f;
    const float v = (m < N1) ? scaled(__ldg(x1 + m), e1) : 0.0f;
    a[m] = make_float4(u, v, 0.0f, 0.0f);
  }
}

__global__ void k_multi_split_df(const MultiRow* __restrict__ rows, int nrows, const float4* __restrict__ Z,
                                 float4* B, int M) {
  const int j = blockIdx.y;
  const bool two = 2 * j + 1 < nrows;
  const float4* z = Z + (int64_t)j * M;
  const float2* H0 = reinterpret_cast<const float2*>(rows[2 * j].filt);
  const float2* H1 = two ? reinterpret_cast<const float2*>(rows[2 * j + 1].filt) : nullptr;
  float4* b0 = B + (int64_t)(2 * j) * M;
  float4* b1 = B + (int64_t)(2 * j + 1) * M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const float4 p = z[m];
    const float4 q = z[m == 0 ? 0 : M - m];
    // X0 = (Z[m] + conj Z[-m]) / 2,  X1 = (Z[m] - conj Z[-m]) / 2i
    const df pr = df_re(p), pi = df_im(p), qr = df_re(q), qi = df_im(q);
    const float4 x0 = dfc(df_scale2(df_add(pr, qr), 0.5f), df_scale2(df_sub(pi, qi), 0.5f));
    const float2 h0 = H0[m];
    b0[m] = dfc_mul_r(x0, df{h0.x, h0.y});
    if (two) {
      const float4 x1 = dfc(df_scale2(df_add(pi, qi), 0.5f), df_scale2(df_sub(qr, pr), 0.5f));
      const float2 h1 = H1[m];
      b1[m] = dfc_mul_r(x1, df{h1.x, h1.y});
    }
  }
}

__global__ void k_multi_store_df(const MultiRow* __restrict__ rows, const float4* A, int M) {
  const MultiRow r = rows[blockIdx.y];
  const float4* a = A + (int64_t)blockIdx.y * M;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < r.N; k += gridDim.x * blockDim.x) {
    const float4 v = a[k];
    r.out[k] = (r.e == kNoSignal) ? make_float2(0.0f, 0.0f)
                                  : make_float2(scalbnf(df_to_float(df_re(v)), r.e), scalbnf(df_to_float(df_im(v)), r.e));
  }
}

// v <- DFT_R(v) with kernel exp(DIR 2 pi i jk / R), natural output order (double-float)
template <int R, int DIR>
__device__ __forceinline__ void dft_df(float4* v, const DfConsts& k) {
  if constexpr (R == 2) {
    const float4 a = v[0], b = v[1];
    v[0] = dfc_add(a, b);
    v[1] = dfc_sub(a, b);
  } else if constexpr (R == 3) {
    const float4 t1 = dfc_add(v[1], v[2]);
    const float4 t2 = dfc_sub(v[0], dfc_scale2(t1, 0.5f));
    float4 t3 = dfc_muli(dfc_mul_r(dfc_sub(v[1], v[2]), k.s3));
    if (DIR < 0) t3 = dfc_scale2(t3, -1.0f);
    v[0] = dfc_add(v[0], t1);
    v[1] = dfc_add(t2, t3);
    v[2] = dfc_sub(t2, t3);
  } else if constexpr (R == 4) {
    const float4 a = dfc_add(v[0], v[2]), b = dfc_sub(v[0], v[2]);
    const float4 c = dfc_add(v[1], v[3]);
    float4 d = dfc_muli(dfc_sub(v[1], v[3]));
    if (DIR < 0) d = dfc_scale2(d, -1.0f);
    v[0] = dfc_add(a, c);
    v[2] = dfc_sub(a, c);
    v[1] = dfc_add(b, d);
    v[3] = dfc_sub(b, d);
  } else {   // R == 5
    const float4 a1 = dfc_add(v[1], v[4]), a2 = dfc_add(v[2], v[3]);
    const float4 b1 = dfc_sub(v[1], v[4]), b2 = dfc_sub(v[2], v[3]);
    const float4 x0 = v[0];
    const float4 p1 = dfc_add(x0, dfc_add(dfc_mul_r(a1, k.c1), dfc_mul_r(a2, k.c2)));
    const float4 p2 = dfc_add(x0, dfc_add(dfc_mul_r(a1, k.c2), dfc_mul_r(a2, k.c1)));
    float4 q1 = dfc_muli(dfc_add(dfc_mul_r(b1, k.s1), dfc_mul_r(b2, k.s2)));
    float4 q2 = dfc_muli(dfc_sub(dfc_mul_r(b1, k.s2), dfc_mul_r(b2, k.s1)));
    if (DIR < 0) {
      q1 = dfc_scale2(q1, -1.0f);
      q2 = dfc_scale2(q2, -1.0f);
    }
    v[0] = dfc_add(x0, dfc_add(a1, a2));
    v[1] = dfc_add(p1, q1);
    v[4] = dfc_sub(p1, q1);
    v[2] = dfc_add(p2, q2);
    v[3] = dfc_sub(p2, q2);
  }
}

// DFT_16 (natural order) as 4 x 4: DFT_4 over n2 of x[4 n2 + n1], twiddles
// w16^(n1 k1), DFT_4 over n1; w16 = exp(DIR 2 pi i / 16).
template <int DIR>
__device__ __forceinline__ void dft16_df(float4* v, const DfConsts& k) {
  float4 y[4][4];
#pragma unroll
  for (int n1 = 0; n1 < 4; n1++) {
    float4 t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
    dft_df<4, DIR>(t, k);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) y[n1][k1] = t[k1];
  }
  // w16^e for e = n1 k1 in {1, 2, 3, 4, 6, 9}
  const float s = (float)DIR;
  const float4 w1 = dfc(k.c8, df{s * k.s8.hi, s * k.s8.lo});
  const float4 w2 = dfc(k.r2, df{s * k.r2.hi, s * k.r2.lo});
  const float4 w3 = dfc(k.s8, df{s * k.c8.hi, s * k.c8.lo});
  y[1][1] = dfc_mul(y[1][1], w1);
  y[1][2] = dfc_mul(y[1][2], w2);
  y[1][3] = dfc_mul(y[1][3], w3);
  y[2][1] = dfc_mul(y[2][1], w2);
  y[2][2] = (DIR < 0) ? dfc_scale2(dfc_muli(y[2][2]), -1.0f) : dfc_muli(y[2][2]);                        // w^4
  y[2][3] = dfc_mul(y[2][3], dfc(df{-k.r2.hi, -k.r2.lo}, df{s * k.r2.hi, s * k.r2.lo}));                // w^6
  y[3][1] = dfc_mul(y[3][1], w3);
  y[3][2] = dfc_mul(y[3][2], dfc(df{-k.r2.hi, -k.r2.lo}, df{s * k.r2.hi, s * k.r2.lo}));                // w^6
  y[3][3] = dfc_mul(y[3][3], dfc(df{-k.c8.hi, -k.c8.lo}, df{-s * k.s8.hi, -s * k.s8.lo}));              // w^9
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float4 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft_df<4, DIR>(t, k);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = t[k2];
  }
}

// One radix-R Stockham pass over nrows rows of n points (as the FP64 pass):
// 32-bit indices (callers keep n * nrows below 2^31).
template <int R, int DIR>
__global__ void __launch_bounds__(256) k_pass_df(const float4* __restrict__ in, float4* __restrict__ out, int n,
                                                 int Ns, int nrows, const float4* __restrict__ tw, DfConsts kc) {
  const int m = n / R;
  const int total = m * nrows;
  const int tstride = n / (Ns * R);
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int row = g / m;
    const int j = g - row * m;
    const float4* x = in + (int64_t)row * n;
    float4 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = x[j + r * m];
    const int k = j % Ns;
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = dfc_mul_c(v[r], __ldg(tw + k * r * tstride), DIR > 0);
    }
    if constexpr (R == 16) dft16_df<DIR>(v, kc);
    else dft_df<R, DIR>(v, kc);
    float4* o = out + (int64_t)row * n + (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) o[r * Ns] = v[r];
  }
}


__global__ void k_df_from_double(const double2* __restrict__ src, float4* dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[i] = dfc(df_from_double(v.x), df_from_double(v.y));
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

cudaError_t launch_multi_load2_df(const MultiRow* rows, int nrows, float4* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const int np = (nrows + 1) / 2;
  if (np > 65535) return cudaErrorInvalidValue;
  k_multi_load2_df<<<grid2(M, np), 256, 0, st>>>(rows, nrows, A, M);
  return cudaGetLastError();
}
cudaError_t launch_multi_split_df(const MultiRow* rows, int nrows, const float4* Z, float4* B, int M,
                                  cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const int np = (nrows + 1) / 2;
  if (np > 65535) return cudaErrorInvalidValue;
  k_multi_split_df<<<grid2(M, np), 256, 0, st>>>(rows, nrows, Z, B, M);
  return cudaGetLastError();
}
cudaError_t launch_multi_store_df(const MultiRow* rows, int nrows, const float4* A, int M, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_multi_store_df<<<grid2(M / 2, nrows), 256, 0, st>>>(rows, A, M);
  return cudaGetLastError();
}
cudaError_t launch_pass_df(int R, int dir, const float4* in, float4* out, int n, int Ns, int nrows, const float4* tw,
                           const DfConsts& kc, cudaStream_t st) {
  if ((int64_t)n * nrows >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  const int64_t work = (int64_t)(n / R) * nrows;
  int64_t b = (work + 255) / 256;
  const int grid = (int)(b < 1 ? 1 : (b < 152 * 16 ? b : 152 * 16));
#define FPCC_PASS_DF(RR)                                                                      \
  if (R == RR) {                                                                              \
    if (dir < 0) k_pass_df<RR, -1><<<grid, 256, 0, st>>>(in, out, n, Ns, nrows, tw, kc);      \
    else k_pass_df<RR, 1><<<grid, 256, 0, st>>>(in, out, n, Ns, nrows, tw, kc);               \
    return cudaGetLastError();                                                                \
  }
  FPCC_PASS_DF(2)
  FPCC_PASS_DF(3)
  FPCC_PASS_DF(4)
  FPCC_PASS_DF(5)
  FPCC_PASS_DF(16)
#undef FPCC_PASS_DF
  return cudaErrorInvalidValue;
}

cudaError_t launch_df_from_double(const double2* src, float4* dst, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int g = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_df_from_double<<<g, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

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
int hk_table_len(int M) { return 256 + (M + 1) / 512 + 2; }

cudaError_t launch_hk_rows(const int* Ns, int nk, double2* T, float4* B, int M, cudaStream_t st) {
  if (nk <= 0) return cudaSuccess;
  if (nk > 65535) return cudaErrorInvalidValue;
  const int ldt = hk_table_len(M);
  k_hk_tables<<<dim3((ldt + 255) / 256, nk), 256, 0, st>>>(Ns, nk, T, ldt);
  k_hk_rows<<<grid2(M / 2 + 1, (nk + 1) / 2), 256, 0, st>>>(Ns, nk, T, ldt, B, M);
  return cudaGetLastError();
}
cudaError_t launch_hk_extract(const float4* Z, int nk, int M, bool df_out, void* out, cudaStream_t st) {
  if (nk <= 0) return cudaSuccess;
  const int rows = (nk + 1) / 2;
  if (rows > 65535) return cudaErrorInvalidValue;
  if (df_out) k_hk_extract<true><<<grid2(M, rows), 256, 0, st>>>(Z, nk, M, out);
  else k_hk_extract<false><<<grid2(M, rows), 256, 0, st>>>(Z, nk, M, out);
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
template cudaError_t launch_multi_split<float2>(const MultiRow*, int, const float2*, float2*, int, cudaStream_t);
template cudaError_t launch_multi_store<float2>(const MultiRow*, int, const float2*, int, cudaStream_t);
template cudaError_t launch_multi_convert<float2>(const double2*, float2*, int64_t, cudaStream_t);

}  // namespace fpcc
