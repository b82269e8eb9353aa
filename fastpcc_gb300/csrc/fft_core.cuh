// CTA-level FFT building blocks for the correlation kernels (sm_103a).
//
// One thread block transforms one or more vectors held in shared memory with an
// autosorting (Stockham) mixed-radix schedule: one pass per radix factor R, each
// pass reading R points at stride n/R, applying the twiddles w^(r*k) with
// w = exp(dir*2*pi*i/(Ns*R)), k = j mod Ns, transforming them with a radix-R DFT
// in registers, and writing them back at (j/Ns)*Ns*R + k + r*Ns.  A pass stages
// every butterfly of the thread in registers before the block-wide barrier, so
// the transform runs in place in a single buffer.  Shared-memory rows are
// padded by one element per 32 (PADI) so that strided writes spread over banks.
//
// Twiddles come from two 128-entry-granular tables per length, built once per
// block with sincospif: exp(-2*pi*i*t/n) = hi[t >> 7] * lo[t & 127].  Powers
// w^r are formed by repeated complex multiplication (error about R ulps).
#pragma once

#ifdef __CUDACC_RTC__
// run-time compilation (NVRTC): builtin vector types; fixed-width integers by hand
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned int uint32_t;
#include <cuda_fp16.h>
#else
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#endif

namespace fpcc {

constexpr int kMaxPass = 10;

struct FftPlan {
  int n;                  // transform length
  int npass;              // number of radix passes
  int rad[kMaxPass];      // radix of each pass, in execution order
  uint64_t code;          // the same radices, 5 bits each (read without indexing rad)
};

__host__ __device__ __forceinline__ int plan_radix(const FftPlan& p, int i) {
  return (int)((p.code >> (5 * i)) & 31u);
}

__host__ __device__ __forceinline__ int PADI(int i) { return i + (i >> 5); }
__host__ __device__ __forceinline__ int padded_len(int n) { return n + (n >> 5) + 1; }
__host__ __device__ __forceinline__ int tw_hi_len(int n) { return (n + 127) / 128; }

// ---------------------------------------------------------------- complex ops
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
// conj(a) * b
__device__ __forceinline__ float2 cconjmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by dir*i  (dir = -1 forward: -i, dir = +1 inverse: +i)
template <int DIR>
__device__ __forceinline__ float2 cmul_i(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------- small DFTs
// All compute X[q] = sum_r v[r] * exp(DIR*2*pi*i*q*r/R) in place.
template <int DIR>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int DIR>
__device__ __forceinline__ void dft3(float2* v) {
  const float c = -0.5f;
  const float s = 0.86602540378443864676f;  // sin(2*pi/3)
  float2 t = cadd(v[1], v[2]);
  float2 d = csub(v[1], v[2]);
  float2 m = make_float2(fmaf(c, t.x, v[0].x), fmaf(c, t.y, v[0].y));
  float2 id = cmul_i<DIR>(cscale(d, s));
  v[0] = cadd(v[0], t);
  v[1] = cadd(m, id);
  v[2] = csub(m, id);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2* v) {
  float2 t0 = cadd(v[0], v[2]);
  float2 t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]);
  float2 t3 = cmul_i<DIR>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <int DIR>
__device__ __forceinline__ void dft5(float2* v) {
  const float c1 = 0.30901699437494742410f;   // cos(2*pi/5)
  const float c2 = -0.80901699437494742410f;  // cos(4*pi/5)
  const float s1 = 0.95105651629515357212f;   // sin(2*pi/5)
  const float s2 = 0.58778525229247312917f;   // sin(4*pi/5)
  float2 t1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]);
  float2 t2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
  float2 a1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  float2 a2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  float2 b1 = cmul_i<DIR>(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
  float2 b2 = cmul_i<DIR>(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(a1, b1);
  v[4] = csub(a1, b1);
  v[2] = cadd(a2, b2);
  v[3] = csub(a2, b2);
}

// Radix 8 and 16 work in place and leave X[r] at v[dft_perm<R>(r)].
template <int DIR>
__device__ __forceinline__ void dft8(float2* v) {
  // even/odd halves: e[k] = v[2k], o[k] = v[2k+1]
  {
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    dft4<DIR>(e);
    v[0] = e[0]; v[2] = e[1]; v[4] = e[2]; v[6] = e[3];
  }
  {
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4<DIR>(o);
    v[1] = o[0]; v[3] = o[1]; v[5] = o[2]; v[7] = o[3];
  }
  const float r = 0.70710678118654752440f;
  // o[k] *= exp(DIR*2*pi*i*k/8)
  float2 t = v[3];
  v[3] = make_float2(r * (t.x - DIR * t.y), r * (t.y + DIR * t.x));
  v[5] = cmul_i<DIR>(v[5]);
  t = v[7];
  v[7] = make_float2(-r * (t.x + DIR * t.y), r * (DIR * t.x - t.y));
  // X[k] = e[k] + o[k] -> v[2k],  X[k+4] = e[k] - o[k] -> v[2k+1]
#pragma unroll
  for (int k = 0; k < 4; k++) dft2<DIR>(v[2 * k], v[2 * k + 1]);
}

// 16 = 4 x 4 with n = 4 n1 + n2, k = k1 + 4 k2: DFT4 over n1 for each column
// n2 (results k1 at v[4 k1 + n2]) and the twiddles exp(DIR*2*pi*i*n2*k1/16);
// dft16 then takes a DFT4 over n2 for each k1 (k2 at v[4 k1 + k2]).
template <int DIR>
__device__ __forceinline__ void dft16_head(float2* v) {
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) {
    float2 c[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
    dft4<DIR>(c);
    v[n2] = c[0]; v[4 + n2] = c[1]; v[8 + n2] = c[2]; v[12 + n2] = c[3];
  }
  const float c1 = 0.92387953251128675613f;  // cos(pi/8)
  const float s1 = 0.38268343236508977173f;  // sin(pi/8)
  const float r = 0.70710678118654752440f;
  const float2 w1 = make_float2(c1, DIR * s1);
  const float2 w2 = make_float2(r, DIR * r);
  const float2 w3 = make_float2(s1, DIR * c1);
  const float2 w6 = make_float2(-r, DIR * r);
  const float2 w9 = make_float2(-c1, -DIR * s1);
  // v[4 k1 + n2] *= w^(n2 k1)
  v[5] = cmul(v[5], w1);
  v[9] = cmul(v[9], w2);
  v[13] = cmul(v[13], w3);
  v[6] = cmul(v[6], w2);
  v[10] = cmul_i<DIR>(v[10]);
  v[14] = cmul(v[14], w6);
  v[7] = cmul(v[7], w3);
  v[11] = cmul(v[11], w6);
  v[15] = cmul(v[15], w9);
}

template <int DIR>
__device__ __forceinline__ void dft16(float2* v) {
  dft16_head<DIR>(v);
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) dft4<DIR>(v + 4 * k1);
}

// Composite radices R = A x B done as two stages of small DFTs in registers
// (dft_comp below): A for each.
__host__ __device__ constexpr int comp_a(int R) {
  return R == 6 ? 2 : R == 9 ? 3 : R == 10 ? 2 : R == 12 ? 4 : R == 15 ? 3 : R == 20 ? 4 : R == 24 ? 8 : 0;
}

// Position of output X[r] after dft<R> (radix 8/16 and the composite radices
// leave a transposed order).
template <int R>
__host__ __device__ constexpr int dft_perm(int r) {
  if constexpr (comp_a(R) > 0) {
    return r / (R / comp_a(R)) + comp_a(R) * (r % (R / comp_a(R)));
  } else {
    return R == 16 ? 4 * (r & 3) + (r >> 2) : (R == 8 ? 2 * (r & 3) + (r >> 2) : r);
  }
}

// ---- compile-time twiddles
constexpr double kPiD = 3.14159265358979323846264338327950288;
// Taylor series of sin and cos, for arguments reduced to [-pi, pi]
constexpr double cx_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int n = 1; n < 20; n++) {
    term *= -x2 / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}
constexpr double cx_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int n = 1; n < 20; n++) {
    term *= -x2 / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}
// v * exp(DIR 2 pi i T / N): exact quarter turns as swaps, otherwise a
// constant computed at compile time (angle reduced to [-pi, pi]).
template <int T, int N, int DIR>
__device__ __forceinline__ float2 cmul_ct(float2 v) {
  constexpr int t = ((T % N) + N) % N;
  constexpr int q4 = ((4 * t) % N == 0) ? (4 * t) / N : -1;
  if constexpr (q4 == 0) {
    return v;
  } else if constexpr (q4 == 1) {
    return cmul_i<DIR>(v);
  } else if constexpr (q4 == 2) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (q4 == 3) {
    return cmul_i<-DIR>(v);
  } else {
    constexpr double ang = 2.0 * kPiD * (double)(2 * t > N ? t - N : t) / (double)N;
    constexpr float c = (float)cx_cos(ang);
    constexpr float s = (float)((double)DIR * cx_sin(ang));
    return cmul(v, make_float2(c, s));
  }
}

template <int V>
struct IntC {
  static constexpr int value = V;
};
// fn(IntC<B>{}), ..., fn(IntC<E - 1>{}): a loop whose index is a constant
template <int B, int E, typename Fn>
__device__ __forceinline__ void sfor(Fn&& fn) {
  if constexpr (B < E) {
    fn(IntC<B>{});
    sfor<B + 1, E>(static_cast<Fn&&>(fn));
  }
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2* v);

// In-place DFT of R = A x B points: with n = r1 + A r2 and k = s2 + B s1,
//   X[k] = sum_r1 w_A^(r1 s1) w_R^(r1 s2) sum_r2 v[r1 + A r2] w_B^(r2 s2);
// the B-point DFTs (one per r1) and their twiddles first, then the A-point
// DFTs (one per s2); X[k] is left at v[s1 + A s2] (dft_perm<R>).
template <int A, int B, int DIR>
__device__ __forceinline__ void dft_comp(float2* v) {
  constexpr int R = A * B;
  sfor<0, A>([&](auto i1) {
    constexpr int r1 = decltype(i1)::value;
    float2 t[B];
#pragma unroll
    for (int r2 = 0; r2 < B; r2++) t[r2] = v[r1 + A * r2];
    dft<B, DIR>(t);
    sfor<0, B>([&](auto i2) {
      constexpr int s2 = decltype(i2)::value;
      v[r1 + A * s2] = cmul_ct<r1 * s2, R, DIR>(t[dft_perm<B>(s2)]);
    });
  });
#pragma unroll
  for (int s2 = 0; s2 < B; s2++) {
    float2 t[A];
#pragma unroll
    for (int r1 = 0; r1 < A; r1++) t[r1] = v[r1 + A * s2];
    dft<A, DIR>(t);
#pragma unroll
    for (int s1 = 0; s1 < A; s1++) v[s1 + A * s2] = t[dft_perm<A>(s1)];
  }
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2* v) {
  if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
  else if constexpr (R == 3) dft3<DIR>(v);
  else if constexpr (R == 4) dft4<DIR>(v);
  else if constexpr (R == 5) dft5<DIR>(v);
  else if constexpr (R == 8) dft8<DIR>(v);
  else if constexpr (R == 16) dft16<DIR>(v);
  else if constexpr (comp_a(R) > 0) dft_comp<comp_a(R), R / comp_a(R), DIR>(v);
}

// ---------------------------------------------------------------- twiddles
struct TwTab {
  const float2* lo;  // exp(-2*pi*i*j/n), j in [0,128)
  const float2* hi;  // exp(-2*pi*i*128*i/n), i in [0, ceil(n/128))
};

// Fill a table pair (all threads of the block cooperate; caller syncs).
__device__ __forceinline__ void build_twiddles(float2* lo, float2* hi, int n) {
  const float inv = 2.0f / (float)n;
  for (int j = threadIdx.x; j < 128; j += blockDim.x) {
    float s, c;
    // exact reduction of the angle: t/n in [0,1)
    sincospif(-(float)j * inv, &s, &c);
    lo[j] = make_float2(c, s);
  }
  const int nh = tw_hi_len(n);
  for (int i = threadIdx.x; i < nh; i += blockDim.x) {
    int t = (128 * i) % n;
    float a = -(float)t * inv;
    if (a < -1.0f) a += 2.0f;  // keep |a| <= 1 (angle in units of pi)
    float s, c;
    sincospif(a, &s, &c);
    hi[i] = make_float2(c, s);
  }
}

__device__ __forceinline__ float2 twiddle(const TwTab& tw, int t) {
  return cmul(tw.hi[t >> 7], tw.lo[t & 127]);
}

// ---------------------------------------------------------------- passes
// One Stockham pass of radix R over nvec vectors of compile-time length N stored
// at s + vec*vstride (each vector padded with PADI), with Ns the product of the
// radices already applied.  Each of the T threads stages B = ceil(nvec*N/R / T)
// butterflies in registers (B is bounded by BMAX, a compile-time value that the
// caller derives from its nvec bound).
// Powers w^1..w^(R-1) of a twiddle, formed as a shallow product tree
// (w^(2a) = (w^a)^2, w^(2a+1) = w^(2a) w) so the multiplications overlap.
template <int R>
__device__ __forceinline__ void twiddle_powers(float2 w1, float2* w) {
  w[1] = w1;
#pragma unroll
  for (int r = 2; r < R; r++) w[r] = (r & 1) ? cmul(w[r - 1], w1) : cmul(w[r >> 1], w[r >> 1]);
}

template <int R, int DIR, int N, int Ns, int T, int BMAX>
__device__ __forceinline__ void ct_pass(float2* s, int nvec, int vstride, const TwTab& tw) {
  constexpr int m = N / R;
  constexpr int tstride = N / (Ns * R);
  const int total = m * nvec;
  float2 v[BMAX][R];
#pragma unroll
  for (int b = 0; b < BMAX; b++) {
    const int g = threadIdx.x + b * T;
    if (g < total) {
      const int vec = g / m;
      const int j = g - vec * m;
      const float2* sv = s + vec * vstride;
      if constexpr (m % 32 == 0) {
        // PADI(j + r m) = PADI(j) + r m + r m / 32: constant offsets
        const float2* sj = sv + PADI(j);
#pragma unroll
        for (int r = 0; r < R; r++) v[b][r] = sj[r * m + ((r * m) >> 5)];
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) v[b][r] = sv[PADI(j + r * m)];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < BMAX; b++) {
    const int g = threadIdx.x + b * T;
    if (g < total) {
      const int vec = g / m;
      const int j = g - vec * m;
      const int k = (Ns == 1) ? 0 : j % Ns;
      if (Ns > 1 && k != 0) {
        float2 w1 = twiddle(tw, k * tstride);
        if (DIR > 0) w1.y = -w1.y;
        float2 w[R];
        twiddle_powers<R>(w1, w);
#pragma unroll
        for (int r = 1; r < R; r++) v[b][r] = cmul(v[b][r], w[r]);
      }
      dft<R, DIR>(v[b]);
      const int base = (j - k) * R + k;
      float2* sv = s + vec * vstride;
      if constexpr (Ns % 32 == 0) {
        float2* sb = sv + PADI(base);
#pragma unroll
        for (int r = 0; r < R; r++) sb[r * Ns + ((r * Ns) >> 5)] = v[b][dft_perm<R>(r)];
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) sv[PADI(base + r * Ns)] = v[b][dft_perm<R>(r)];
      }
    }
  }
  __syncthreads();
}

template <int R, int... Rest>
constexpr int prod_radices() {
  if constexpr (sizeof...(Rest) == 0) return R;
  else return R * prod_radices<Rest...>();
}

// Out-of-place Stockham pass (ping-pong): butterflies go from src to dst one
// at a time, so a thread holds only R values and each pass needs one barrier.
template <int R, int DIR, int N, int Ns, int T>
__device__ __forceinline__ void pp_pass(const float2* __restrict__ src, float2* __restrict__ dst, const TwTab& tw) {
  constexpr int m = N / R;
  constexpr int tstride = N / (Ns * R);
#pragma unroll 1
  for (int j = threadIdx.x; j < m; j += T) {
    float2 v[R];
    if constexpr (m % 32 == 0) {
      const float2* sj = src + PADI(j);
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = sj[r * m + ((r * m) >> 5)];
    } else {
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = src[PADI(j + r * m)];
    }
    const int k = (Ns == 1) ? 0 : j % Ns;
    if (Ns > 1 && k != 0) {
      float2 w1 = twiddle(tw, k * tstride);
      if (DIR > 0) w1.y = -w1.y;
      float2 w[R];
      twiddle_powers<R>(w1, w);
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], w[r]);
    }
    dft<R, DIR>(v);
    const int base = (j - k) * R + k;
    if constexpr (Ns % 32 == 0) {
      float2* sb = dst + PADI(base);
#pragma unroll
      for (int r = 0; r < R; r++) sb[r * Ns + ((r * Ns) >> 5)] = v[dft_perm<R>(r)];
    } else {
#pragma unroll
      for (int r = 0; r < R; r++) dst[PADI(base + r * Ns)] = v[dft_perm<R>(r)];
    }
  }
  __syncthreads();
}

template <int DIR, int N, int Ns, int T, int R, int... Rest>
__device__ __forceinline__ void pp_passes(float2* a, float2* b, const TwTab& tw) {
  pp_pass<R, DIR, N, Ns, T>(a, b, tw);
  if constexpr (sizeof...(Rest) > 0) pp_passes<DIR, N, Ns * R, T, Rest...>(b, a, tw);
}

template <int... Rs>
struct Radices;

// Transform of one vector held in a (padded); the result ends in a when the
// number of passes is even, else in b.  The caller synchronises before the call.
template <int DIR, int T, int... Rs>
__device__ __forceinline__ float2* pp_fft(float2* a, float2* b, const TwTab& tw, Radices<Rs...>) {
  constexpr int N = prod_radices<Rs...>();
  pp_passes<DIR, N, 1, T, Rs...>(a, b, tw);
  return (sizeof...(Rs) % 2 == 0) ? a : b;
}

template <int... Rs>
struct Radices {};


// Staging bound of a pass: ceil(NV*N/R / T) butterflies per thread.
template <int N, int R, int T, int NV>
constexpr int bmax_of() {
  return ((N / R) * NV + T - 1) / T;
}

template <int DIR, int N, int Ns, int T, int NV, int R, int... Rest>
__device__ __forceinline__ void ct_passes(float2* s, int nvec, int vstride, const TwTab& tw) {
  ct_pass<R, DIR, N, Ns, T, bmax_of<N, R, T, NV>()>(s, nvec, vstride, tw);
  if constexpr (sizeof...(Rest) > 0) ct_passes<DIR, N, Ns * R, T, NV, Rest...>(s, nvec, vstride, tw);
}

// Full transform (unnormalised) of nvec <= NV vectors of length prod(Rs) held
// in shared memory, by a block of exactly T threads.
template <int DIR, int T, int NV, int... Rs>
__device__ __forceinline__ void ct_fft(float2* s, int nvec, int vstride, const TwTab& tw, Radices<Rs...>) {
  constexpr int N = prod_radices<Rs...>();
  ct_passes<DIR, N, 1, T, NV, Rs...>(s, nvec, vstride, tw);
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide max; scratch holds >= 32 floats.  All threads get the result.
__device__ __forceinline__ float block_max(float v, float* scratch) {
  v = warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (l < nw) ? scratch[l] : 0.0f;
  v = warp_max(v);
  return v;
}

// Block-scaled int16 storage: a row starts with a 16-byte header holding the
// row's float scale, then short2 values; value = q * scale, with the scale set
// so that the largest component maps to 32767.  Relative to FP16 (11-bit
// significands) it keeps about 15 bits for components near the row maximum and
// more absolute precision for the typical component of a flat spectrum.
constexpr int kI16Header = 16;
constexpr float kI16Max = 32767.0f;

__device__ __forceinline__ float i16_row_scale(const void* row) { return *reinterpret_cast<const float*>(row); }
__device__ __forceinline__ const short2* i16_row_bins(const void* row) {
  return reinterpret_cast<const short2*>(reinterpret_cast<const char*>(row) + kI16Header);
}
__device__ __forceinline__ short i16_quant(float v, float inv) {
  const float q = fminf(fmaxf(rintf(v * inv), -kI16Max), kI16Max);
  return (short)q;
}

// Quantise the n values s[PADI(0..n)] of a block into the int16 row `row`
// (header + bins); every thread of the block calls it.  scratch: >= 32 floats.
template <int T>
__device__ __forceinline__ void store_i16_row(const float2* s, int n, void* row, float* scratch) {
  float m = 0.0f;
  for (int k = threadIdx.x; k < n; k += T) {
    const float2 v = s[PADI(k)];
    m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  m = block_max(m, scratch);
  const float inv = (m > 0.0f) ? kI16Max / m : 0.0f;
  if (threadIdx.x < 4) reinterpret_cast<float*>(row)[threadIdx.x] = (threadIdx.x == 0) ? m / kI16Max : 0.0f;
  short2* o = reinterpret_cast<short2*>(reinterpret_cast<char*>(row) + kI16Header);
  for (int k = threadIdx.x; k < n; k += T) {
    const float2 v = s[PADI(k)];
    o[k] = make_short2(i16_quant(v.x, inv), i16_quant(v.y, inv));
  }
}

}  // namespace fpcc
