// Four-step transforms for lengths above the in-block menu (see large.cuh).
#include <float.h>

#include "large.cuh"

namespace fpcc {
namespace {

constexpr int kColVecs = 16;   // columns per column-kernel block
constexpr int kRowVecs = 8;    // rows per row-kernel block

__host__ __device__ constexpr int cpadded(int n) { return n + (n >> 5) + 1; }
__host__ __device__ constexpr int ctw_hi(int n) { return (n + 127) / 128; }

template <int... Rs>
constexpr int rlen(Radices<Rs...>) {
  return prod_radices<Rs...>();
}


// Bin i of a spectrum row (int16 rows: after the header, unscaled).
__device__ __forceinline__ float2 ld_bin(const void* base, int fmt, int64_t i) {
  if (fmt == SPEC_F16) return __half22float2(reinterpret_cast<const __half2*>(base)[i]);
  if (fmt == SPEC_I16) {
    const short2 q = i16_row_bins(base)[i];
    return make_float2((float)q.x, (float)q.y);
  }
  return reinterpret_cast<const float2*>(base)[i];
}

// Cross-spectrum bin p of a pair: herm 0 = full spectra, 1 = bins 0..Nz/2 of real
// traces, 2 = precomputed cross-spectrum rows (spec row = pair index).
__device__ __forceinline__ float2 pair_bin(const LargeArgs& a, int row, int p) {
  const int Nz = a.Nz;
  if (a.herm == 2) return ld_bin(a.spec, a.fmt, (int64_t)row * a.ldspec + p);
  const void* X1;
  const void* X2;
  if (a.desc) {
    X1 = a.desc[row].a;
    X2 = a.desc[row].b;
  } else {
    const int2 pr = a.pairs[row];
    const int64_t esz = (a.fmt == SPEC_F32) ? 8 : 4;
    X1 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.x * a.ldspec * esz;
    X2 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.y * a.ldspec * esz;
  }
  if (a.herm == 1 && p > (Nz >> 1)) {
    const int q = Nz - p;
    return cconj(cconjmul(ld_bin(X1, a.fmt, q), ld_bin(X2, a.fmt, q)));
  }
  return cconjmul(ld_bin(X1, a.fmt, p), ld_bin(X2, a.fmt, p));
}

// prow / frow: for COL_PRODUCT the input row and the filter row of `row`
// (row / filt_of_row_div and its remainder, computed once per block).  MODE is
// the column mode, a compile-time value so that a block's loads carry no branch
// between them (cols_gather issues them all before the first is used).
template <int MODE>
__device__ __forceinline__ float2 col_load(const LargeArgs& a, int row, int j, float eps, int prow, int frow) {
  switch (MODE) {
    case COL_REAL:
    case COL_SIGN: {
      const int jj = j - a.in_off;
      if (jj < 0 || jj >= a.N) return make_float2(0.f, 0.f);
      float v = __ldg(reinterpret_cast<const float*>(a.in) + (int64_t)row * a.ldin + jj);
      if (MODE == COL_SIGN) v = (a.sign_ge ? (v >= 0.0f) : (v > 0.0f)) ? 1.0f : -1.0f;
      return make_float2(v * a.in_scale, 0.f);
    }
    case COL_PHASE: {
      if (j >= a.N) return make_float2(0.f, 0.f);
      const float2 v = reinterpret_cast<const float2*>(a.in)[(int64_t)row * a.ldin + j];
      return cscale(v, factor_of(a.rule, v.x * v.x + v.y * v.y, eps));
    }
    case COL_COMPLEX:
      return reinterpret_cast<const float2*>(a.in)[(int64_t)row * a.ldin + j];
    case COL_NORMALISE: {
      const float2 v = reinterpret_cast<const float2*>(a.in)[(int64_t)row * a.ldin + j];
      return cscale(v, factor_of(a.rule, v.x * v.x + v.y * v.y, eps));
    }
    case COL_PRODUCT: {
      const float2 x = reinterpret_cast<const float2*>(a.in)[(int64_t)prow * a.ldin + j];
      float2 w = a.filt[(int64_t)frow * a.ldfilt + j];
      if (a.filt_conj) w.y = -w.y;
      return cscale(cmul(x, w), a.in_scale);
    }
    default: {  // COL_PAIR: F[j] = (H[j] + H[j+h]) + i w^j (H[j] - H[j+h]), w = exp(2 pi i / Nz)
      const int h = a.n;
      const int Nz = a.Nz;
      const float2 z0 = pair_bin(a, row, j);
      const float2 z3 = pair_bin(a, row, j == 0 ? 0 : Nz - j);
      const float2 z2 = pair_bin(a, row, j + h);
      const float2 z1 = pair_bin(a, row, h - j);
      const float2 Hk = cscale(cadd(z0, cconj(z3)), 0.5f);
      const float2 Hkh = cscale(cadd(z2, cconj(z1)), 0.5f);
      float s, c;
      sincospif((float)j / (float)h, &s, &c);   // exp(2 pi i j / Nz), Nz = 2h
      const float2 e = cadd(Hk, Hkh);
      const float2 o = cmul(make_float2(c, s), csub(Hk, Hkh));
      return make_float2(e.x - o.y, e.y + o.x);
    }
  }
}

// The PER = C N1 / T column elements of a thread (element e = threadIdx.x + i T
// is column e % C, point e / C), loaded into registers together.
template <int MODE, int PER, int T, int C>
__device__ __forceinline__ void cols_gather(const LargeArgs& a, int row, int c0, int n2, float eps, int prow, int frow,
                                            float2* buf) {
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = threadIdx.x + i * T;
    buf[i] = col_load<MODE>(a, row, (e / C) * n2 + c0 + e % C, eps, prow, frow);
  }
}

// BATCH: each thread's loads issued together (for the modes whose loads are
// several reads and arithmetic: the wavelet band product and the pair
// cross-spectrum); the other modes keep the loop, held to the registers of
// five 256-thread blocks per SM (more warps to hide the loads' latency).
template <int T, typename RAD, int DIR, bool BATCH>
__global__ void __launch_bounds__(T, BATCH ? 1 : 1280 / T) k_cols(LargeArgs a) {
  constexpr int N1 = rlen(RAD{});
  constexpr int C = kColVecs;
  constexpr int VS = cpadded(N1);
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* lo1 = s + C * VS;
  float2* hi1 = lo1 + 128;
  float2* loN = hi1 + ctw_hi(N1);
  float2* hiN = loN + 128;
  const int n = a.n, n2 = a.n2;
  build_twiddles(lo1, hi1, N1);
  build_twiddles(loN, hiN, n);
  const int row = blockIdx.y;
  const int c0 = blockIdx.x * C;
  const float eps = (a.cmode == COL_PHASE || a.cmode == COL_NORMALISE) ? eps_of(a.rule, a.rowstat[row]) : 0.f;
  const int prow = (a.cmode == COL_PRODUCT) ? row / a.filt_of_row_div : row;
  const int frow = (a.cmode == COL_PRODUCT) ? row - prow * a.filt_of_row_div : 0;
  static_assert((C * N1) % T == 0, "column block: whole elements per thread");
  constexpr int PER = C * N1 / T;
  if constexpr (BATCH) {
    float2 buf[PER];
    if (a.cmode == COL_PRODUCT) cols_gather<COL_PRODUCT, PER, T, C>(a, row, c0, n2, eps, prow, frow, buf);
    else cols_gather<COL_PAIR, PER, T, C>(a, row, c0, n2, eps, prow, frow, buf);
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int e = threadIdx.x + i * T;
      s[(e % C) * VS + PADI(e / C)] = buf[i];
    }
  } else {
    for (int e = threadIdx.x; e < C * N1; e += T) {
      const int j = (e / C) * n2 + c0 + e % C;
      float2 v;
      switch (a.cmode) {
        case COL_REAL: v = col_load<COL_REAL>(a, row, j, eps, prow, frow); break;
        case COL_SIGN: v = col_load<COL_SIGN>(a, row, j, eps, prow, frow); break;
        case COL_PHASE: v = col_load<COL_PHASE>(a, row, j, eps, prow, frow); break;
        case COL_COMPLEX: v = col_load<COL_COMPLEX>(a, row, j, eps, prow, frow); break;
        default: v = col_load<COL_NORMALISE>(a, row, j, eps, prow, frow); break;
      }
      s[(e % C) * VS + PADI(e / C)] = v;
    }
  }
  __syncthreads();
  ct_fft<DIR, T, C>(s, C, VS, TwTab{lo1, hi1}, RAD{});
  float2* out = a.T + (int64_t)row * n;
  const TwTab twN{loN, hiN};
  for (int e = threadIdx.x; e < C * N1; e += T) {
    const int c = e % C, k1 = e / C;
    const int j2 = c0 + c;
    // j2 < n2 and k1 < N1, so j2 k1 < n: the twiddle index needs no reduction
    float2 w = twiddle(twN, j2 * k1);
    if (DIR > 0) w.y = -w.y;
    out[(int64_t)k1 * n2 + j2] = cmul(s[c * VS + PADI(k1)], w);
  }
}

// Row blocks of 160-256 threads are held to the registers of 1280 threads per
// SM (eight blocks of 160): the row pass waits on its loads, and more resident
// warps hide more of that wait than the few registers spilled cost.
template <int T, typename RAD, int DIR>
__global__ void __launch_bounds__(T, (T >= 160 && T <= 256) ? 1280 / T : 1) k_rows(LargeArgs a) {
  constexpr int N2 = rlen(RAD{});
  constexpr int C = kRowVecs;
  constexpr int VS = cpadded(N2);
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* lo = s + C * VS;
  float2* hi = lo + 128;
  __shared__ float red[32];
  build_twiddles(lo, hi, N2);
  const int n = a.n, n1 = a.n1;
  const int row = blockIdx.y;
  const int r0 = blockIdx.x * C;
  const float2* in = a.T + (int64_t)row * n;
  {
    // every load of the thread first, then the stores into the tile
    static_assert((C * N2) % T == 0, "row block: whole elements per thread");
    constexpr int PER = C * N2 / T;
    float2 buf[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int e = threadIdx.x + i * T;
      buf[i] = in[(int64_t)(r0 + e / N2) * N2 + e % N2];
    }
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int e = threadIdx.x + i * T;
      s[(e / N2) * VS + PADI(e % N2)] = buf[i];
    }
  }
  __syncthreads();
  ct_fft<DIR, T, C>(s, C, VS, TwTab{lo, hi}, RAD{});
  // lag read-out (ROW_LAGS): the pair's lengths, scale, output row and energy
  // rows are the block's (one pair per blockIdx.y), found once
  int N = 0, lag0 = 0, L = 0;
  float scale = 0.f;
  float* yrow = nullptr;
  GnccNorm gn;
  const int Nz = 2 * n;
  if (a.rmode == ROW_LAGS) {
    const double* E1 = nullptr;
    const double* E2 = nullptr;
    if (a.desc) {
      const PairDesc& d = a.desc[row];
      N = d.N;
      lag0 = d.lag0;
      L = d.L;
      scale = d.scale != 0.0f ? d.scale : (a.norm == 0 ? 1.0f / ((float)Nz * (float)N) : (float)(1.0 / (double)Nz));
      if (a.fmt == SPEC_I16) scale *= i16_row_scale(d.a) * i16_row_scale(d.b);
      yrow = reinterpret_cast<float*>(d.y);
      if (a.norm == 1) { E1 = d.ea; E2 = d.eb; }
    } else {
      N = a.N;
      lag0 = a.lag0;
      L = a.L;
      scale = a.scale;
      yrow = a.y + (int64_t)row * a.ldy;
      // station rows of the pair: only with a pair list (precomputed cross-spectrum rows have none)
      if (a.herm != 2 && (a.fmt == SPEC_I16 || a.norm == 1)) {
        const int2 pr = a.pairs[row];
        if (a.fmt == SPEC_I16) {
          const char* sp = reinterpret_cast<const char*>(a.spec);
          scale *= i16_row_scale(sp + (int64_t)pr.x * a.ldspec * 4) * i16_row_scale(sp + (int64_t)pr.y * a.ldspec * 4);
        }
        if (a.norm == 1) {
          E1 = a.energy + (int64_t)pr.x * a.ldE;
          E2 = a.energy + (int64_t)pr.y * a.ldE;
        }
      }
    }
    if (a.norm == 1) gn.init(E1, E2, N);
  }
  float mx = 0.f;
  for (int e = threadIdx.x; e < C * N2; e += T) {
    const int c = e % C, k2 = e / C;
    const int k = (r0 + c) + n1 * k2;
    const float2 v = s[c * VS + PADI(k2)];
    if (a.rmode == ROW_SPEC) {
      if (a.out_half && k > (n >> 1)) continue;
      if (a.out_fmt == SPEC_F16)
        reinterpret_cast<__half2*>(a.out)[(int64_t)row * a.ldo + k] = __float22half2_rn(v);
      else
        reinterpret_cast<float2*>(a.out)[(int64_t)row * a.ldo + k] = v;
    } else if (a.rmode == ROW_COMPLEX) {
      reinterpret_cast<float2*>(a.out)[(int64_t)row * a.ldo + k] = v;
      mx = fmaxf(mx, v.x * v.x + v.y * v.y);
    } else {
      // y_full[2k] = Re z[k], y_full[2k+1] = Im z[k]; lag = idx or idx - Nz
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int idx = 2 * k + q;
        const int lag = (idx <= (Nz >> 1)) ? idx : idx - Nz;
        const int l = lag - lag0;
        if (l < 0 || l >= L) continue;
        float val = (q ? v.y : v.x) * scale;
        if (a.norm == 1) {
          val = gn.apply(val, lag);
        } else if (a.norm == 2) {
          val = val / (float)(N - abs(lag));
        }
        yrow[l] = val;
      }
    }
  }
  if (a.rmode == ROW_COMPLEX && a.rowmax) {
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
      float v = (threadIdx.x < T / 32) ? red[threadIdx.x] : 0.f;
      v = warp_max(v);
      if (threadIdx.x == 0) atomicMax(reinterpret_cast<int*>(a.rowmax) + row, __float_as_int(v));
    }
  }
}

template <typename K>
cudaError_t launch_k2(K kern, dim3 grid, int T, size_t smem, cudaStream_t st, const LargeArgs& a) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void* argv[] = {const_cast<LargeArgs*>(&a)};
  return cudaLaunchKernel((const void*)kern, grid, dim3(T), argv, smem, st);
}

// column sub-lengths and row sub-lengths with their radix schedules
#define FPCC_COL_MENU(X) X(32, 128, 8, 4) X(64, 128, 16, 4) X(128, 128, 16, 8) X(256, 256, 16, 16)
#define FPCC_ROW_MENU(X)                                                                               \
  X(64, 128, 16, 4) X(128, 128, 16, 8) X(256, 128, 16, 16) X(320, 160, 16, 4, 5) X(384, 192, 16, 8, 3) \
  X(512, 256, 16, 8, 4) X(640, 320, 16, 8, 5) X(768, 384, 16, 16, 3) X(1024, 512, 16, 16, 4)           \
  X(1280, 640, 16, 16, 5) X(1536, 768, 16, 8, 4, 3) X(2048, 1024, 16, 16, 8)

bool in_col_menu(int n) {
#define FPCC_C(SZ, T, ...) if (n == SZ) return true;
  FPCC_COL_MENU(FPCC_C)
#undef FPCC_C
  return false;
}
bool in_row_menu(int n) {
#define FPCC_R(SZ, T, ...) if (n == SZ) return true;
  FPCC_ROW_MENU(FPCC_R)
#undef FPCC_R
  return false;
}

}  // namespace

bool large_supported(int n, int* n1, int* n2) {
  for (int c : {256, 128, 64, 32}) {
    if (n % c == 0 && in_col_menu(c) && in_row_menu(n / c) && n / c >= kRowVecs) {
      *n1 = c;
      *n2 = n / c;
      return true;
    }
  }
  return false;
}

cudaError_t launch_large(const LargeArgs& a, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  if (a.nrows > 65535) return cudaErrorInvalidValue;
  cudaError_t e = cudaErrorInvalidValue;
  // column pass
  {
    const bool batch = (a.cmode == COL_PRODUCT || a.cmode == COL_PAIR);
    dim3 grid(a.n2 / kColVecs, a.nrows);
    const size_t smem = ((size_t)kColVecs * cpadded(a.n1) + 128 + ctw_hi(a.n1) + 128 + ctw_hi(a.n)) * sizeof(float2);
    bool done = false;
#define FPCC_CL(SZ, T, ...)                                                                            \
  if (!done && a.n1 == SZ) {                                                                         \
    if (batch)                                                                                        \
      e = (a.dir < 0) ? launch_k2(k_cols<T, Radices<__VA_ARGS__>, -1, true>, grid, T, smem, st, a)     \
                      : launch_k2(k_cols<T, Radices<__VA_ARGS__>, 1, true>, grid, T, smem, st, a);     \
    else                                                                                              \
      e = (a.dir < 0) ? launch_k2(k_cols<T, Radices<__VA_ARGS__>, -1, false>, grid, T, smem, st, a)    \
                      : launch_k2(k_cols<T, Radices<__VA_ARGS__>, 1, false>, grid, T, smem, st, a);    \
    done = true;                                                                                     \
  }
    FPCC_COL_MENU(FPCC_CL)
#undef FPCC_CL
    if (!done || e != cudaSuccess) return done ? e : cudaErrorInvalidValue;
  }
  // row pass
  {
    dim3 grid(a.n1 / kRowVecs, a.nrows);
    const size_t smem = ((size_t)kRowVecs * cpadded(a.n2) + 128 + ctw_hi(a.n2)) * sizeof(float2);
    bool done = false;
#define FPCC_RW(SZ, T, ...)                                                                            \
  if (!done && a.n2 == SZ) {                                                                         \
    e = (a.dir < 0) ? launch_k2(k_rows<T, Radices<__VA_ARGS__>, -1>, grid, T, smem, st, a)             \
                    : launch_k2(k_rows<T, Radices<__VA_ARGS__>, 1>, grid, T, smem, st, a);             \
    done = true;                                                                                     \
  }
    FPCC_ROW_MENU(FPCC_RW)
#undef FPCC_RW
    if (!done) return cudaErrorInvalidValue;
  }
  return e;
}

}  // namespace fpcc
