// Direct (non-FFT) kernels:
//   - FP64 prefix sums of x^2 per station window (GNCC overlap energies,
//     reference gn_lowlevel src/FFTapps.c:372-399 updates the same sums
//     incrementally),
//   - PCC at power v by direct lag sums over phase signals
//     (src/FFTapps.c:223-336, src/ccs_cuda.cu:260-321,388-453),
//   - 1-bit GNCC numerators as exact popcounts of packed sign bits.
#include "direct.cuh"
#include "kernels.cuh"

namespace fpcc {

namespace {

// ---------------------------------------------------------------- energies
// FP64 prefix sums of x^2 over chunks of kEChunk samples, in two launches:
// per-chunk totals, then each chunk's scan from the total of the chunks before
// it.  Every x^2 is exact in FP64 (24-bit by 24-bit product), so only the
// additions round.
constexpr int kEChunk = 4096;
constexpr int kEPer = kEChunk / 256;   // samples per thread

__global__ void __launch_bounds__(256) k_energy_chunks(const float* __restrict__ x, int64_t ldx, int N, int nch,
                                                       double* __restrict__ part) {
  __shared__ double ws[8];
  const int c = blockIdx.x;
  const float* xr = x + (int64_t)blockIdx.y * ldx + (int64_t)c * kEChunk;
  const int len = min(kEChunk, N - c * kEChunk);
  double s = 0.0;
  for (int i = threadIdx.x; i < len; i += 256) {
    const double f = (double)__ldg(xr + i);
    s += f * f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += ws[w];
    part[(int64_t)blockIdx.y * nch + c] = t;
  }
}

__global__ void __launch_bounds__(256) k_energy_scan(const float* __restrict__ x, int64_t ldx, int N, int nch,
                                                     const double* __restrict__ part, double* __restrict__ E,
                                                     int64_t ldE) {
  __shared__ double ws[8];
  __shared__ double base_s;
  const int c = blockIdx.x, row = blockIdx.y;
  const float* xr = x + (int64_t)row * ldx + (int64_t)c * kEChunk;
  double* Er = E + (int64_t)row * ldE + (int64_t)c * kEChunk;
  const int len = min(kEChunk, N - c * kEChunk);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int j = 0; j < c; j++) b += part[(int64_t)row * nch + j];
    base_s = b;
    if (c == 0) Er[0] = 0.0;
  }
  // each thread: kEPer consecutive samples, prefix in registers
  double v[kEPer];
  double t = 0.0;
  const int i0 = threadIdx.x * kEPer;
#pragma unroll
  for (int j = 0; j < kEPer; j++) {
    double f = 0.0;
    if (i0 + j < len) f = (double)__ldg(xr + i0 + j);
    t += f * f;
    v[j] = t;
  }
  // exclusive scan of the thread totals
  double incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  double off = base_s;
  for (int k = 0; k < w; k++) off += ws[k];
  off += incl - t;
#pragma unroll
  for (int j = 0; j < kEPer; j++)
    if (i0 + j < len) Er[i0 + j + 1] = off + v[j];
}

// Normalisation tables of each row (layout and rule: GnccNorm in
// kernels.cuh): one thread per n = 0..N writes the prefix and suffix entries;
// the thread of n = 0 sets the flag E[0] = -0.0 after reading E[0].
__global__ void __launch_bounds__(256) k_energy_tables(double* __restrict__ E, int64_t ldE, int N) {
  const int n = blockIdx.x * 256 + threadIdx.x;
  if (n > N) return;
  double* Er = E + (int64_t)blockIdx.y * ldE;
  float* T = reinterpret_cast<float*>(Er + N + 1);
  const double e = Er[n];
  T[n] = energy_table_entry(e);
  T[N + 1 + n] = energy_table_entry(Er[N] - e);
  if (n == 0) Er[0] = -0.0;
}

// ---------------------------------------------------------------- PCC_v direct
// One thread per lag, 256 lags per block; phase signals staged in shared memory
// in tiles of TILE samples (zeros outside [0,N), which contribute nothing since
// |0+b| - |0-b| = 0).  Each tile's terms are summed in FP32 and the tile sums
// are accumulated in FP64.
constexpr int kLagBlock = 256;
constexpr int kTile = 512;

// Square root by the hardware approximation (relative error about 1 ulp); the
// terms are summed in FP32 tiles and FP64 across tiles, far below the 1e-4 bound.
__device__ __forceinline__ float sqrt_fast(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Phase sample n of a row in storage format FMT (0 float2, 1 half2, 2 int16 of scale 1/32767).
template <int FMT>
__device__ __forceinline__ float2 phase_at(const void* row, int n) {
  if constexpr (FMT == 1) {
    return __half22float2(reinterpret_cast<const __half2*>(row)[n]);
  } else if constexpr (FMT == 2) {
    const short2 q = reinterpret_cast<const short2*>(row)[n];
    return make_float2((float)q.x * (1.0f / 32767.0f), (float)q.y * (1.0f / 32767.0f));
  } else {
    return reinterpret_cast<const float2*>(row)[n];
  }
}

// S threads per lag (S = 1: one lag per thread, 256 lags per block; S = 4: 64
// lags per block, each lag's tile sum split over 4 threads and their FP64
// partial sums added in a fixed order), so a block's duration is N / S tiles of
// work: long windows no longer make a few very long blocks.
template <int MODE, int FMT, int S>   // MODE 1: v = 1, 2: v = 2, 0: general power
__global__ void __launch_bounds__(kLagBlock) k_pccv(PccvArgs a) {
  constexpr int LB = kLagBlock / S;               // lags per block
  __shared__ float2 s1[kTile];
  __shared__ float2 s2[kTile + LB];
  __shared__ double red[S > 1 ? kLagBlock : 1];
  // grid (lag blocks, pairs): blocks are issued pair by pair, so descriptors
  // ordered by decreasing window length start the longest blocks first
  const int p = blockIdx.y;
  const int sub = threadIdx.x / LB, li = threadIdx.x - sub * LB;
  const int lblk = blockIdx.x * LB;               // first lag index of the block
  const int l = lblk + li;
  int N, Lag1, L;
  const void* R1;
  const void* R2;
  float* y;
  if (a.desc) {
    const fpcc_pair_desc& d = a.desc[p];
    N = d.N;
    Lag1 = d.lag0;
    L = d.L;
    R1 = d.a;
    R2 = d.b;
    y = reinterpret_cast<float*>(d.y);
    if (lblk >= L) return;                       // whole block beyond this pair's lags
  } else {
    const int2 pr = a.pairs[p];
    N = a.N;
    Lag1 = a.Lag1;
    L = a.L;
    const int64_t esz = FMT ? 4 : 8;
    R1 = reinterpret_cast<const char*>(a.phase) + (int64_t)pr.x * a.ldp * esz;
    R2 = reinterpret_cast<const char*>(a.phase) + (int64_t)pr.y * a.ldp * esz;
    y = a.y + (int64_t)p * a.ldy;
  }
  const int lagb = Lag1 + lblk;                   // lag of thread 0
  const float V = 0.5f * a.v;
  double acc = 0.0;
  // samples n of station 1 that overlap any lag of the block
  int nlo = -(lagb + LB - 1);
  if (nlo < 0) nlo = 0;
  int nhi = N - lagb;
  if (nhi > N) nhi = N;
  for (int n0 = nlo; n0 < nhi; n0 += kTile) {
    for (int i = threadIdx.x; i < kTile; i += kLagBlock) {
      const int n = n0 + i;
      float2 v = make_float2(0.f, 0.f);
      if (n < N) v = phase_at<FMT>(R1, n);
      s1[i] = v;
    }
    for (int i = threadIdx.x; i < kTile + LB; i += kLagBlock) {
      const int n = n0 + lagb + i;
      float2 v = make_float2(0.f, 0.f);
      if (n >= 0 && n < N) v = phase_at<FMT>(R2, n);
      s2[i] = v;
    }
    __syncthreads();
    float part = 0.0f;
    const float2* b = s2 + li;
    constexpr int span = kTile / S;
#pragma unroll 8
    for (int i = sub * span; i < (sub + 1) * span; i++) {
      const float2 u = s1[i];
      const float2 w = b[i];
      const float sx = u.x + w.x, sy = u.y + w.y;
      const float dx = u.x - w.x, dy = u.y - w.y;
      const float s2v = sx * sx + sy * sy;
      const float d2v = dx * dx + dy * dy;
      if (MODE == 1) part += sqrt_fast(s2v) - sqrt_fast(d2v);
      else if (MODE == 2) part += s2v - d2v;
      else part += powf(s2v, V) - powf(d2v, V);
    }
    acc += (double)part;
    __syncthreads();
  }
  if constexpr (S > 1) {
    red[threadIdx.x] = acc;
    __syncthreads();
    if (sub != 0) return;
    acc = red[li];
#pragma unroll
    for (int s = 1; s < S; s++) acc += red[s * LB + li];
  }
  if (l < L) {
    const int lag = Lag1 + l;
    if (lag < -N || lag > N) { y[l] = 0.0f; return; }
    const double cnt = (double)(N - abs(lag));
    const double D = a.norm_gpu ? 2.0 * cnt : exp2((double)V) * cnt;
    y[l] = (float)(acc / D);
  }
}

// ---------------------------------------------------------------- PCC1 direct
// PCC at power 1 (the reference's pcc1f_lowlevel, src/FFTapps.c:251-278, and
// the GPU kernel of src/ccs_cuda.cu:260-321): as k_pccv with v = 1, but each
// thread takes two adjacent lags, and the station-2 tile is staged as its even
// and odd samples, so that per pair of samples of station 1 (one broadcast
// 16-byte load) a thread loads two station-2 values and reuses a third from the
// previous step for four terms: five shared-memory wavefronts per 128 terms of
// a warp instead of twelve.
//
// Terms: |a + b| - |a - b|.  For |a| = |b| = 1 this equals 2c / sqrt(1 + |s|)
// with c + i s = a conj(b) (|a +- b|^2 = 2 +- 2c and c^2 + s^2 = 1), one
// reciprocal square root instead of two square roots; with a or b = 0 both
// forms give 0.  A tile whose staged samples of both stations all have
// | |x|^2 - 1 | <= 2^-20 or x = 0 (phase signals of the pure-phase rules,
// src/ccs_cuda.cu:201-208,223-230) uses it; any other tile (the regularised
// rules of src/FFTapps.c:147-205, where moduli fall below 1 by 1e-6 max|x|/|x|
// and much more inside gaps) keeps the two square roots.  The choice depends
// only on the pair's own samples, so a result does not depend on the launch.
__device__ __forceinline__ float rsqrt_fast(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ bool unit_or_zero(float2 v) {
  const float m2 = v.x * v.x + v.y * v.y;
  return m2 == 0.0f || fabsf(m2 - 1.0f) <= 0x1p-20f;
}

// |w + u| - |w - u| / 2 for unit-modulus (or zero) w, u
__device__ __forceinline__ float pcc1_term_unit(float2 w, float ux, float uy) {
  const float c = fmaf(w.x, ux, w.y * uy);
  const float sn = fmaf(w.y, ux, -w.x * uy);
  return c * rsqrt_fast(1.0f + fabsf(sn));
}

__device__ __forceinline__ float pcc1_term(float2 w, float ux, float uy) {
  const float sx = w.x + ux, sy = w.y + uy, dx = w.x - ux, dy = w.y - uy;
  return sqrt_fast(fmaf(sx, sx, sy * sy)) - sqrt_fast(fmaf(dx, dx, dy * dy));
}

template <int FMT, int S>
__global__ void __launch_bounds__(kLagBlock) k_pcc1(PccvArgs a) {
  constexpr int TS = kLagBlock / S;          // threads of one sub-range = lag pairs per block
  constexpr int LB = 2 * TS;                 // lags per block
  constexpr int NE = (kTile + LB) / 2 + 1;   // even / odd station-2 samples of a tile
  __shared__ float4 s1p[kTile / 2];          // station-1 samples 2k, 2k + 1
  __shared__ float2 s2e[NE], s2o[NE];
  __shared__ double red[S > 1 ? 2 * kLagBlock : 1];
  const int p = blockIdx.y;
  const int sub = threadIdx.x / TS, li = threadIdx.x - sub * TS;
  const int lblk = blockIdx.x * LB;          // first lag index of the block
  const int l = lblk + 2 * li;               // this thread's lag indices l, l + 1
  int N, Lag1, L;
  const void* R1;
  const void* R2;
  float* y;
  if (a.desc) {
    const fpcc_pair_desc& d = a.desc[p];
    N = d.N;
    Lag1 = d.lag0;
    L = d.L;
    R1 = d.a;
    R2 = d.b;
    y = reinterpret_cast<float*>(d.y);
    if (lblk >= L) return;                   // whole block beyond this pair's lags
  } else {
    const int2 pr = a.pairs[p];
    N = a.N;
    Lag1 = a.Lag1;
    L = a.L;
    const int64_t esz = FMT ? 4 : 8;
    R1 = reinterpret_cast<const char*>(a.phase) + (int64_t)pr.x * a.ldp * esz;
    R2 = reinterpret_cast<const char*>(a.phase) + (int64_t)pr.y * a.ldp * esz;
    y = a.y + (int64_t)p * a.ldy;
  }
  const int lagb = Lag1 + lblk;              // lag of index lblk
  double acc0 = 0.0, acc1 = 0.0;
  int nlo = -(lagb + LB - 1);
  if (nlo < 0) nlo = 0;
  int nhi = N - lagb;
  if (nhi > N) nhi = N;
  for (int n0 = nlo; n0 < nhi; n0 += kTile) {
    bool unit = true;
    for (int i = threadIdx.x; i < kTile / 2; i += kLagBlock) {
      const int n = n0 + 2 * i;
      float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
      if (n < N) v0 = phase_at<FMT>(R1, n);
      if (n + 1 < N) v1 = phase_at<FMT>(R1, n + 1);
      unit = unit && unit_or_zero(v0) && unit_or_zero(v1);
      s1p[i] = make_float4(v0.x, v0.y, v1.x, v1.y);
    }
    for (int i = threadIdx.x; i < 2 * NE; i += kLagBlock) {
      const int n = n0 + lagb + i;           // station-2 sample of tile position i
      float2 v = make_float2(0.f, 0.f);
      if (n >= 0 && n < N) v = phase_at<FMT>(R2, n);
      unit = unit && unit_or_zero(v);
      if (i & 1) s2o[i >> 1] = v;
      else s2e[i >> 1] = v;
    }
    const bool fast = __syncthreads_and(unit) != 0;
    // lag l at sample pair k: station-2 positions 2 li + 2k (even) and 2 li + 2k + 1 (odd);
    // lag l + 1: 2 li + 2k + 1 (odd) and 2 li + 2k + 2 (the next even one)
    constexpr int span = kTile / 2 / S;
    const int k0 = sub * span;
    float part0 = 0.0f, part1 = 0.0f;
    float2 e0 = s2e[li + k0];
    if (fast) {
#pragma unroll 4
      for (int k = k0; k < k0 + span; k++) {
        const float4 u = s1p[k];
        const float2 o0 = s2o[li + k];
        const float2 e1 = s2e[li + k + 1];
        part0 += pcc1_term_unit(e0, u.x, u.y) + pcc1_term_unit(o0, u.z, u.w);
        part1 += pcc1_term_unit(o0, u.x, u.y) + pcc1_term_unit(e1, u.z, u.w);
        e0 = e1;
      }
      part0 *= 2.0f;
      part1 *= 2.0f;
    } else {
#pragma unroll 4
      for (int k = k0; k < k0 + span; k++) {
        const float4 u = s1p[k];
        const float2 o0 = s2o[li + k];
        const float2 e1 = s2e[li + k + 1];
        part0 += pcc1_term(e0, u.x, u.y) + pcc1_term(o0, u.z, u.w);
        part1 += pcc1_term(o0, u.x, u.y) + pcc1_term(e1, u.z, u.w);
        e0 = e1;
      }
    }
    acc0 += (double)part0;
    acc1 += (double)part1;
    __syncthreads();
  }
  if constexpr (S > 1) {
    red[threadIdx.x] = acc0;
    red[kLagBlock + threadIdx.x] = acc1;
    __syncthreads();
    if (sub != 0) return;
    acc0 = red[li];
    acc1 = red[kLagBlock + li];
#pragma unroll
    for (int k = 1; k < S; k++) {
      acc0 += red[k * TS + li];
      acc1 += red[kLagBlock + k * TS + li];
    }
  }
  const double V = 0.5;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int lh = l + h;
    if (lh >= L) break;
    const int lag = Lag1 + lh;
    if (lag < -N || lag > N) {
      y[lh] = 0.0f;
      continue;
    }
    const double cnt = (double)(N - abs(lag));
    const double D = a.norm_gpu ? 2.0 * cnt : exp2(V) * cnt;
    y[lh] = (float)((h ? acc1 : acc0) / D);
  }
}

// ---------------------------------------------------------------- 1-bit bits
// bit i of word w is 1 when sample 32w+i maps to -1: x < 0 for the station-1
// rule (x >= 0 -> +1), x <= 0 for the station-2 rule (x > 0 -> +1).
__global__ void k_sign_bits(const float* __restrict__ x, int64_t ldx, int N, uint32_t* __restrict__ bits,
                            int64_t ldb, int pos_ge, const int8_t* __restrict__ sel) {
  // one warp per 32-sample word (blockDim is a multiple of 32)
  const int row = blockIdx.x;
  const int n = blockIdx.y * blockDim.x + threadIdx.x;
  const int nw = (N + 31) >> 5;
  const int ge = sel ? sel[row] : pos_ge;
  const float* xr = x + (int64_t)row * ldx;
  bool neg = false;
  if (n < N) {
    const float v = __ldg(xr + n);
    neg = ge ? !(v >= 0.0f) : !(v > 0.0f);
  }
  const uint32_t m = __ballot_sync(0xffffffffu, neg);
  if ((threadIdx.x & 31) == 0 && (n >> 5) < nw) bits[(int64_t)row * ldb + (n >> 5)] = m;
}

// 32 bits of a packed stream starting at bit position b (b >= 0); words beyond
// the row read as zero.
__device__ __forceinline__ uint32_t bits_at(const uint32_t* r, int nw, int b) {
  const int w = b >> 5, s = b & 31;
  const uint32_t lo = (w < nw) ? __ldg(r + w) : 0u;
  const uint32_t hi = (w + 1 < nw) ? __ldg(r + w + 1) : 0u;
  return __funnelshift_r(lo, hi, s);
}

// numerator(lag) = overlap - 2 * popcount(b1[n] xor b2[n+lag]) over the overlap.
// A block takes 256 consecutive lags of one pair.  The whole words of station 1
// that lie inside a lag's overlap are counted from shared-memory tiles: the
// station-1 word is the same for every lag of the block (broadcast) and the
// station-2 bits of a lag are a funnel shift of two staged words, the upper
// one carried to the next word, so each word costs two shared loads, a shift,
// an xor and a popcount.  The partial words at the two ends of the overlap are
// counted with masks straight from global memory.
constexpr int kPopTile = 1024;   // station-1 words per tile

__global__ void __launch_bounds__(256) k_cc1b_popcount(Cc1bArgs a) {
  __shared__ uint32_t s1[kPopTile];
  __shared__ uint32_t s2[kPopTile + 9];
  const int p = blockIdx.y;   // grid (lag blocks, pairs), as k_pccv
  const int l0 = blockIdx.x * blockDim.x;
  const int l = l0 + threadIdx.x;
  int N, lag0, L;
  const uint32_t* B1;
  const uint32_t* B2;
  if (a.desc) {
    const fpcc_pair_desc& d = a.desc[p];
    L = d.L;
    if (l0 >= L) return;                          // whole block beyond this pair's lags
    N = d.N;
    lag0 = d.lag0;
    B1 = reinterpret_cast<const uint32_t*>(d.a);
    B2 = reinterpret_cast<const uint32_t*>(d.b);
  } else {
    L = a.L;
    const int2 pr = a.pairs[p];
    N = a.N;
    lag0 = a.lag0;
    B1 = a.bits + (int64_t)pr.x * a.ldb;
    B2 = a.bits + (int64_t)pr.y * a.ldb;
  }
  const int nw = (N + 31) >> 5;
  const bool active = l < L;
  const int lag = lag0 + l;
  const int n1 = lag < 0 ? -lag : 0;              // overlap [n1, n2) in station-1 samples
  const int n2 = lag < 0 ? N : N - lag;
  const int cnt = n2 - n1;
  const bool some = active && n2 > n1;
  const int wa = (n1 + 31) >> 5, wb = n2 >> 5;    // whole words [wa, wb)
  int mism = 0;
  if (some) {
    // partial words: [n1, n2) inside one word, or [n1, 32 wa) and [32 wb, n2)
    const int s0 = n1, e0 = (wa > wb) ? n2 : 32 * wa;
    const int s9 = (wa > wb) ? n2 : 32 * wb, e9 = n2;
    if (e0 > s0) mism += __popc((bits_at(B1, nw, s0) ^ bits_at(B2, nw, s0 + lag)) & ((1u << (e0 - s0)) - 1u));
    if (e9 > s9) mism += __popc((bits_at(B1, nw, s9) ^ bits_at(B2, nw, s9 + lag)) & ((1u << (e9 - s9)) - 1u));
  }
  // whole words of any lag of the block: from the largest lag's first to the smallest lag's last
  const int lagb = lag0 + l0;
  const int lag_max = lag0 + min(L - 1, l0 + (int)blockDim.x - 1);
  const int w_lo = (max(0, -lag_max) + 31) >> 5;
  const int w_hi = max(0, min(N, N - lagb)) >> 5;
  const int sh = (lagb & 31) + (int)threadIdx.x;   // = lag - 32 floor(lagb / 32)
  const int q = sh >> 5, r = sh & 31;
  for (int w0 = w_lo; w0 < w_hi; w0 += kPopTile) {
    const int ct = min(kPopTile, w_hi - w0);
    const int base2 = w0 + (lagb >> 5);           // floor(lagb / 32)
    for (int i = threadIdx.x; i < ct; i += blockDim.x) s1[i] = __ldg(B1 + w0 + i);
    for (int j = threadIdx.x; j < ct + 9; j += blockDim.x) {
      const int k = base2 + j;
      s2[j] = (k >= 0 && k < nw) ? __ldg(B2 + k) : 0u;
    }
    __syncthreads();
    if (some) {
      const int i0 = max(wa, w0) - w0, i1 = min(wb, w0 + ct) - w0;
      if (i0 < i1) {
        uint32_t lo = s2[i0 + q];
#pragma unroll 4
        for (int i = i0; i < i1; i++) {
          const uint32_t hi = s2[i + q + 1];
          mism += __popc(s1[i] ^ __funnelshift_r(lo, hi, r));
          lo = hi;
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  const long long num = (long long)cnt - 2LL * mism;
  if (a.desc) {
    if (a.desc_num) reinterpret_cast<long long*>(a.desc[p].y)[l] = num;
    else reinterpret_cast<float*>(a.desc[p].y)[l] = (float)((double)num / (double)cnt);
    return;
  }
  if (a.num) a.num[(int64_t)p * a.ldy + l] = num;
  if (a.y) a.y[(int64_t)p * a.ldy + l] = (float)((double)num / (double)cnt);
}

}  // namespace

int energy_chunks(int N) { return (N + kEChunk - 1) / kEChunk; }

cudaError_t launch_energy_prefix(const float* x, int64_t ldx, int nrows, int N, double* E, int64_t ldE,
                                 double* part, bool tables, cudaStream_t st) {
  if (nrows <= 0 || N <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  if (tables && ldE < 2 * ((int64_t)N + 1)) return cudaErrorInvalidValue;
  const int nch = energy_chunks(N);
  k_energy_chunks<<<dim3(nch, nrows), 256, 0, st>>>(x, ldx, N, nch, part);
  k_energy_scan<<<dim3(nch, nrows), 256, 0, st>>>(x, ldx, N, nch, part, E, ldE);
  if (tables) k_energy_tables<<<dim3(N / 256 + 1, nrows), 256, 0, st>>>(E, ldE, N);
  return cudaGetLastError();
}

cudaError_t launch_pccv(const PccvArgs& a, cudaStream_t st) {
  if (a.npairs <= 0 || a.L <= 0) return cudaSuccess;
  if (a.half < 0 || a.half > 2) return cudaErrorInvalidValue;
  const int mode = (a.v == 1.0f) ? 1 : (a.v == 2.0f ? 2 : 0);
  // packed launches (windows of any lengths) split each lag over 4 threads; the
  // choice depends on the launch form only, so a request's result does not
  // depend on the other windows in its launch
  // k_pcc1 (v = 1) always splits each lag over 4 threads (128 lags per block),
  // so that launches of few pairs still fill the GPU
  const bool split = a.desc != nullptr || mode == 1;
  // lags per block: k_pccv one per thread (or sub-range), k_pcc1 two
  const int per = (split ? kLagBlock / 4 : kLagBlock) * (mode == 1 ? 2 : 1);
  const int lb = (a.L + per - 1) / per;
  for (int p0 = 0; p0 < a.npairs; p0 += 65535) {   // grid.y holds at most 65535 pairs
    PccvArgs b = a;
    b.npairs = a.npairs - p0 < 65535 ? a.npairs - p0 : 65535;
    if (a.desc) {
      b.desc = a.desc + p0;
    } else {
      b.pairs = a.pairs + p0;
      b.y = a.y + (int64_t)p0 * a.ldy;
    }
    const dim3 grid(lb, b.npairs);
#define FPCC_PCCV_S(F, SS)                                                    \
    if (mode == 1) k_pcc1<F, SS><<<grid, kLagBlock, 0, st>>>(b);              \
    else if (mode == 2) k_pccv<2, F, SS><<<grid, kLagBlock, 0, st>>>(b);      \
    else k_pccv<0, F, SS><<<grid, kLagBlock, 0, st>>>(b);
#define FPCC_PCCV_FMT(F)                                                      \
    if (a.half == F) {                                                        \
      if (split) { FPCC_PCCV_S(F, 4) } else { FPCC_PCCV_S(F, 1) }             \
    }
    FPCC_PCCV_FMT(0)
    FPCC_PCCV_FMT(1)
    FPCC_PCCV_FMT(2)
#undef FPCC_PCCV_FMT
#undef FPCC_PCCV_S
  }
  return cudaGetLastError();
}

cudaError_t launch_sign_bits(const float* x, int64_t ldx, int nrows, int N, uint32_t* bits, int64_t ldb,
                             int pos_ge, const int8_t* sel, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if ((N + 255) / 256 > 65535) return cudaErrorInvalidValue;
  dim3 grid(nrows, (N + 255) / 256);
  k_sign_bits<<<grid, 256, 0, st>>>(x, ldx, N, bits, ldb, pos_ge, sel);
  return cudaGetLastError();
}

cudaError_t launch_cc1b_popcount(const Cc1bArgs& a, cudaStream_t st) {
  if (a.npairs <= 0 || a.L <= 0) return cudaSuccess;
  for (int p0 = 0; p0 < a.npairs; p0 += 65535) {   // grid.y holds at most 65535 pairs
    Cc1bArgs b = a;
    b.npairs = a.npairs - p0 < 65535 ? a.npairs - p0 : 65535;
    if (a.desc) {
      b.desc = a.desc + p0;
    } else {
      b.pairs = a.pairs + p0;
      if (b.y) b.y = a.y + (int64_t)p0 * a.ldy;
      if (b.num) b.num = a.num + (int64_t)p0 * a.ldy;
    }
    k_cc1b_popcount<<<dim3((a.L + 255) / 256, b.npairs), 256, 0, st>>>(b);
  }
  return cudaGetLastError();
}

}  // namespace fpcc
