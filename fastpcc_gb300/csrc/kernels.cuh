// Kernel argument blocks and launchers shared by the host engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fastpcc_gb300.h"
#include "fft_core.cuh"

namespace fpcc {

// GNCC normalisation of one lag (src/FFTapps.c:896-902): the overlap energies
// of x1[n11, n12) and x2[n21, n22) come from FP64 prefix sums (E[0] = 0, so one
// of the two is a plain load and only the other a difference), then
// v / sqrt(e1 e2) with FP32 reciprocal square roots when both energies lie in
// [1e-30, 1e30] (checked on the values rounded to FP32), else in FP64.  The
// GB300 issues FP64 at a small fraction of its FP32 rate: this form takes one
// FP64 subtraction per lag instead of two subtractions and four comparisons.
// Narrowing of the two energies uses energy_to_float below rather than a
// conversion instruction, which would run on the FP64 pipe as well.
__device__ __forceinline__ float energy_to_float(double d);

// A prefix sum as stored: E[0] may hold -0.0 (the flag of rows that carry
// normalisation tables), read as +0.0; every other prefix sum is >= 0.
__device__ __forceinline__ double energy_at(const double* E, int i) {
  return __longlong_as_double(__double_as_longlong(E[i]) & 0x7fffffffffffffffLL);
}

__device__ __forceinline__ float gncc_lag_norm(float v, const double* E1, const double* E2, int N, int lag) {
  double e1, e2;
  if (lag > 0) {
    e1 = energy_at(E1, N - lag);
    e2 = E2[N] - energy_at(E2, lag);
  } else {
    e1 = E1[N] - energy_at(E1, -lag);
    e2 = energy_at(E2, N + lag);
  }
  const float f1 = energy_to_float(e1), f2 = energy_to_float(e2);
  if (f1 >= 1e-30f && f2 >= 1e-30f && f1 <= 1e30f && f2 <= 1e30f) return v * (rsqrtf(f1) * rsqrtf(f2));
  return (float)((double)v / sqrt(e1 * e2));
}

// Normalisation tables of one energy row (written by the energy stage when
// the row has room for them, flagged by E[0] = -0.0): after the N + 1 prefix
// sums, 2 (N + 1) floats
//   T[n]         = 1/sqrt(prefix energy E[n])          (n = 0..N)
//   T[N + 1 + n] = 1/sqrt(suffix energy E[N] - E[n])   (n = 0..N)
// each the FP32 reciprocal square root of the energy narrowed as in
// gncc_lag_norm, or 0 where that energy lies outside [1e-30, 1e30].  A lag then
// costs two float loads and two multiplications, with results identical to
// gncc_lag_norm: the same reciprocal square roots of the same narrowed
// energies, multiplied in the same order, and gncc_lag_norm itself for any lag
// whose energies are out of range.
__device__ __forceinline__ float energy_table_entry(double e) {
  const float f = energy_to_float(e);
  return (f >= 1e-30f && f <= 1e30f) ? rsqrtf(f) : 0.0f;
}

// Holds the two rows by their table addresses (the sums sit N + 1 doubles
// before), so that it keeps no more registers live than the two row pointers.
struct GnccNorm {
  const float *T1, *T2;
  int N;
  bool tab;
  __device__ __forceinline__ void init(const double* e1, const double* e2, int n) {
    N = n;
    tab = (__double_as_longlong(e1[0]) < 0) && (__double_as_longlong(e2[0]) < 0);
    T1 = reinterpret_cast<const float*>(e1 + n + 1);
    T2 = reinterpret_cast<const float*>(e2 + n + 1);
  }
  __device__ __forceinline__ const double* E1() const { return reinterpret_cast<const double*>(T1) - (N + 1); }
  __device__ __forceinline__ const double* E2() const { return reinterpret_cast<const double*>(T2) - (N + 1); }
  // product of the two table entries of a lag: > 0, or 0 where gncc_lag_norm
  // has to take the lag (an energy out of the tables' range)
  __device__ __forceinline__ float table(int lag) const {
    const float r1 = lag > 0 ? T1[N - lag] : T1[N + 1 - lag];
    const float r2 = lag > 0 ? T2[N + 1 + lag] : T2[N + lag];
    return r1 * r2;
  }
  __device__ __forceinline__ float apply(float v, int lag) const {
    if (tab) {
      const float p = table(lag);
      if (p > 0.0f) return v * p;
    }
    return gncc_lag_norm(v, E1(), E2(), N, lag);
  }
};

// A double narrowed to float by truncating its significand (relative error
// below 2^-23), from the IEEE-754 fields with integer operations; magnitudes
// below the float normal range give +-0 and above it +-infinity, which the
// range check of gncc_lag_norm sends to its FP64 branch.
__device__ __forceinline__ float energy_to_float(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
  if (e <= 0) return __int_as_float((int)sign);
  if (e >= 255) return __int_as_float((int)(sign | 0x7f800000u));
  return __int_as_float((int)(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu)));
}

// One correlation of a packed launch (lengths and lags per entry).
using PairDesc = fpcc_pair_desc;

// Amplitude-normalisation rules of the reference.
enum AmpRule : int {
  AMP_F_REG = 0,   // AmpNormf  (src/FFTapps.c:178-205): x / (|x| + 1e-6 max|x|)
  AMP_D_REG = 1,   // AmpNorm   (src/FFTapps.c:147-175): x / sqrt(|x|^2 + 1e-6 max|x|^2)
  AMP_PURE = 2,    // GPU_AmpNormf with mabs = 0 (src/ccs_cuda.cu:212-232): x / |x|
  AMP_THRESH = 3,  // GPU_AmpNormf2 on the max (src/ccs_cuda.cu:190-210): x/|x| above 1e-6 max|x|^2
  AMP_SUMTHR = 4   // cuda_AmpNormf2 on the sum (src/ccs_cuda.cu:493-511): x/|x| above 1e-6 sum|x|^2
};

enum SpecFmt : int { SPEC_F32 = 0, SPEC_F16 = 1, SPEC_I16 = 2 };

// Station spectrum stage input modes.
enum SpecMode : int {
  SPEC_PHASE = 0,  // complex analytic signal rows -> amplitude-normalised phase signal
  SPEC_REAL = 1,   // real trace rows
  SPEC_SIGN = 2    // 1-bit signs of real trace rows
};

struct SpecArgs {
  const void* in;        // SPEC_PHASE: float2 rows; otherwise float rows
  int64_t ldin;
  int nrows;
  int N;                 // samples per row
  int Nz;                // transform length (on the size menu)
  int mode;              // SpecMode
  int rule;              // AmpRule (SPEC_PHASE)
  const float* rowstat;  // SPEC_PHASE: per-row max |a|^2, or sum |a|^2 for AMP_SUMTHR
  int sign_ge;           // SPEC_SIGN: 1 -> x >= 0 is +1, 0 -> x > 0 is +1
  int fmt;               // SpecFmt of the output
  void* out;             // nrows x ldo complex; SPEC_PHASE stores Nz bins, else 0..Nz/2
  int64_t ldo;
};

// Rows of one CWT scale: out[r][k] = IDFT_M(X[r] * F)[k], k < L (in-block, M on the menu).
struct CwtRowArgs {
  const float2* X;       // nrows x M spectra
  int nrows;
  int M;
  const float2* F;       // M-point kernel spectrum (with the 1/M)
  int L;
  float2* out;           // nrows x ldo
  int64_t ldo;
};

struct PairArgs {
  const void* spec;      // station spectra
  int64_t ldspec;
  int fmt;               // SpecFmt
  const int2* pairs;     // (station-1 row, station-2 row) per output row
  int npairs;
  int Nz;                // 2 * (menu length)
  int lag0;              // first lag
  int L;                 // number of lags
  float scale;           // output scale
  float* y;              // npairs x ldy
  int64_t ldy;
  int norm;              // 0 none, 1 GNCC energies (FP64 prefix sums), 2 overlap counts
  const double* energy;  // per station row: N+1 prefix sums of x^2
  int64_t ldE;
  int N;
  const PairDesc* desc;  // packed mode: per-pair rows, N, lags, output (the fields above unused)
};

// Per-row phase signal store for the direct-sum methods.
struct PhaseArgs {
  const float2* in;      // analytic signal rows
  int64_t ldin;
  int nrows;
  int N;                 // samples per row (the largest, with row_N)
  int rule;
  const float* rowstat;
  int fmt;               // 0: float2, 1: half2, 2: int16 of scale 1/32767
  void* out;
  int64_t ldo;
  const int64_t* row_in; // optional (device): row r starts at in + row_in[r] ...
  const int* row_N;      //   ... and has row_N[r] samples (rows of different lengths in one launch)
};

// Bin i of a spectrum row; for block-scaled int16 rows the bins follow the
// header and come back unscaled (the pair's scale product goes into the output).
template <int FMT>
__device__ __forceinline__ float2 load_bin(const void* base, int i) {
  if constexpr (FMT == SPEC_F16) {
    return __half22float2(reinterpret_cast<const __half2*>(base)[i]);
  } else if constexpr (FMT == SPEC_I16) {
    const short2 q = i16_row_bins(base)[i];
    return make_float2((float)q.x, (float)q.y);
  } else {
    return reinterpret_cast<const float2*>(base)[i];
  }
}

// Cross-spectrum bin at position p in [0, Nz).  Full storage holds Nz bins;
// Hermitian storage (real traces) holds bins 0..Nz/2.
template <int FMT, bool HERM>
__device__ __forceinline__ float2 zbin(const void* X1, const void* X2, int p, int Nz) {
  if constexpr (HERM) {
    const int h = Nz >> 1;
    if (p <= h) return cconjmul(load_bin<FMT>(X1, p), load_bin<FMT>(X2, p));
    return cconj(cconjmul(load_bin<FMT>(X1, Nz - p), load_bin<FMT>(X2, Nz - p)));
  } else {
    return cconjmul(load_bin<FMT>(X1, p), load_bin<FMT>(X2, p));
  }
}

bool spec_supported(int Nz);
bool pair_supported(int Nz);
// Tiled pair kernel (pairs_tiled.cu): half lengths R1 x 256 with R1 in {32, 40}.
bool pair_tiled_supported(int Nz);
cudaError_t launch_pairs_tiled(const PairArgs& a, cudaStream_t st);
// Which pair kernel runs a padded length that both forms support.
enum PairForm : int { PAIR_FORM_BLOCK = 1, PAIR_FORM_TILED = 2 };
int pair_form_get(int Nz);
int pair_form_set(int Nz, int form);   // 0, or -1 if the form does not support Nz
size_t spec_smem_bytes(int Nz);
size_t pair_smem_bytes(int Nz);

cudaError_t launch_spec(const SpecArgs& a, cudaStream_t st);
cudaError_t launch_cwt_rows(const CwtRowArgs& a, cudaStream_t st);
cudaError_t launch_pairs(const PairArgs& a, cudaStream_t st);
cudaError_t launch_phase_store(const PhaseArgs& a, cudaStream_t st);
// Block-scaled int16 rows (header + n short2, row stride ldo four-byte elements)
// from float2 rows of stride ldin.
cudaError_t launch_quantize_i16(const float2* in, int64_t ldin, int n, int nrows, void* out, int64_t ldo,
                                cudaStream_t st);

// Generic transforms for any 2,3,5-smooth length: one kernel per radix pass,
// reading `in` and writing `out` (rows of n complex, row stride ld).  The first
// pass may read real rows (real_in) of stride ldr.  tw is the device table
// exp(-2 pi i t / n), t in [0, n).
cudaError_t launch_gpass(int R, int dir, const void* in, bool real_in, int64_t ldr, float2* out, int64_t ld,
                         int n, int Ns, int nrows, const float2* tw, cudaStream_t st);
// Analytic mask with the 1/n of the inverse (src/FFTapps.c:63-67), in place.
cudaError_t launch_analytic_mask(float2* a, int64_t ld, int n, int nrows, cudaStream_t st);
// Per-row max |a|^2 and sum |a|^2.
cudaError_t launch_rowstats(const float2* a, int64_t ld, int n, int nrows, float* rmax, float* rsum,
                            cudaStream_t st);

// Bluestein's chirp-z transform for window lengths with a prime factor above 5:
// DFT_N(x)[k] = c[k] sum_j (x[j] c[j]) conj(c[k-j]),  c[n] = exp(dir pi i n^2 / N),
// with the convolution done by M-point DFTs (M >= 2N-1, 2,3,5-smooth).
cudaError_t launch_blue_pre(const void* in, bool real_in, int64_t ldin, float2* a, int64_t lda, int N, int M,
                            int dir, int mask, int nrows, cudaStream_t st);
cudaError_t launch_blue_mul(float2* a, int64_t lda, const float2* B, int M, int nrows, cudaStream_t st);
cudaError_t launch_blue_post(const float2* a, int64_t lda, float2* out, int64_t ldo, int N, int M, int dir,
                             int nrows, cudaStream_t st);
cudaError_t launch_blue_filter(float2* b, int N, int M, int dir, cudaStream_t st);

}  // namespace fpcc
