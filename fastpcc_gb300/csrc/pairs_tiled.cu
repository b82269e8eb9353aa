// Tiled pair kernel: the cross-spectrum stage of PCC2 / GNCC / 1-bit GNCC for
// half lengths H = R1 x 256 (reference src/FFTapps.c:851-856 for PCC2,
// :347 and :896-902 for GNCC, :1044-1052 for the 1-bit form).
//
// The H-point inverse transform of the packed Hermitian part F of Z = conj(X1) X2
// is split as H = R1 x M with M = 256 (decimation in frequency):
//   X[s + R1 q] = sum_j w_M^(j q) [ w_H^(j s) sum_r F[j + M r] w_R1^(r s) ].
// Stage 1: thread j (256 threads) builds its R1 inputs F[j + M r] straight from
//   the station spectra in registers (the group {k, H-k, H+k, Nz-k} yields F[k]
//   and F[H-k]; F[H-k] belongs to thread M-j, which sits in the same warp, so
//   the two threads each build half of the groups and swap the mirrored values
//   with one shuffle), transforms them with an R1-point DFT in registers,
//   applies w_H^(j s) (powers formed in registers) and writes row s, column j
//   of a shared-memory tile.
// Stage 2: warp w owns rows s in [R1/8 w, R1/8 (w+1)) and transforms each row
//   in place as 16 x 16 (two passes of radix-16 butterflies, one butterfly per
//   lane at a time, rows padded one point per 16 so that neither the strided
//   nor the contiguous pass has bank conflicts), synchronising only the warp;
//   the result is in digit-reversed order.
// Stage 3: the requested lags are read out of the tile (X[f] holds lags 2f and
//   2f+1) with the method's scale and normalisation.
// The block synchronises three times per correlation and two 256-thread
// blocks share an SM.  Blocks loop over correlations (grid = resident blocks),
// so the twiddle tables are built once per block.
#include "kernels.cuh"

namespace fpcc {
namespace {

constexpr int kTM = 256;          // second-stage length = threads per block
constexpr int kTRowStride = 271;  // tile row: 256 points + one pad per 16; odd stride spreads rows over banks

__host__ __device__ __forceinline__ constexpr int P16(int i) { return i + (i >> 4); }
// Padded position of output q of a row after the in-place 16 x 16 transform
// (X[k1 + 16 k2] sits at point k2 + 16 k1).
__device__ __forceinline__ int out_pos(int q) { return (q >> 4) + 17 * (q & 15); }

// In-register DFT of length A*B (A, B on the small-DFT list; B may be 1),
// natural order in and out: X[s2 + B s1] = sum_{r1} w_A^(r1 s1) w_AB^(r1 s2)
// sum_{r2} v[r1 + A r2] w_B^(r2 s2).
template <int A, int B, int DIR>
__device__ __forceinline__ void dft_ab(float2* v) {
  constexpr int R = A * B;
  float2 u[A][B];
  sfor<0, A>([&](auto i1) {
    constexpr int r1 = decltype(i1)::value;
    float2 t[B];
#pragma unroll
    for (int r2 = 0; r2 < B; r2++) t[r2] = v[r1 + A * r2];
    if constexpr (B > 1) dft<B, DIR>(t);
    sfor<0, B>([&](auto i2) {
      constexpr int s2 = decltype(i2)::value;
      u[r1][s2] = cmul_ct<r1 * s2, R, DIR>(t[dft_perm<B>(s2)]);
    });
  });
#pragma unroll
  for (int s2 = 0; s2 < B; s2++) {
    float2 t[A];
#pragma unroll
    for (int r1 = 0; r1 < A; r1++) t[r1] = u[r1][s2];
    dft<A, DIR>(t);
#pragma unroll
    for (int s1 = 0; s1 < A; s1++) v[s2 + B * s1] = t[dft_perm<A>(s1)];
  }
}

// Stage-1 DFT of R1 points as A x B (B = 1: one radix-16 DFT).
__host__ __device__ constexpr int split_a(int R1) { return R1 == 16 ? 16 : 8; }
__host__ __device__ constexpr int split_b(int R1) { return R1 == 16 ? 1 : R1 / 8; }

// In-place 256-point inverse DFT of each of the RW rows of a warp (rows at
// stride kTRowStride, points P16-padded), as 16 x 16 by decimation in frequency:
//   pass 1, butterfly n1: Y[n1][k1] = w_256^(n1 k1) sum_n2 x[n1 + 16 n2] w_16^(n2 k1),
//                         stored at point n1 + 16 k1;
//   pass 2, butterfly k1: X[k1 + 16 k2] = sum_n1 Y[n1][k1] w_16^(n1 k2), stored at k2 + 16 k1.
// A lane always has n1 (pass 1) and k1 (pass 2) equal to lane & 15, so its
// fifteen twiddles are loaded once.  wm: exp(+2 pi i t / 256).
// Half-warps take one row each; with an odd row count the last row's pass 1
// (lanes 0-15) and row 0's pass 2 (lanes 16-31) share one iteration, as one
// instruction stream with per-lane strides and twiddles, so no lane idles.
// edges: only the outputs q in [-32, 32) mod 256 are read afterwards (k2 in
// {14, 15, 0, 1}), so the other pass-2 iterations form those four of their
// sixteen: after the column DFTs and twiddles of the 4 x 4 split
// (k2 = k1' + 4 k2'), the sums over n2 for (k1', k2') = (0, 0), (1, 0), (2, 3)
// and (3, 3).
template <int RW>
__device__ __forceinline__ void warp_dft256(float2* rows0, const float2* __restrict__ wm, int lane, bool edges) {
  constexpr int PR = RW / 2;   // row pairs
  const int b = lane & 15;
  const int h = lane >> 4;
  float2 tw[16];
#pragma unroll
  for (int k = 1; k < 16; k++) tw[k] = wm[b * k];
#pragma unroll
  for (int u = 0; u < PR; u++) {
    float2* x = rows0 + ((lane + 32 * u) >> 4) * kTRowStride + b;   // P16(b + 16 r) = b + 17 r
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = x[17 * r];
    dft<16, 1>(v);
    x[0] = v[dft_perm<16>(0)];
#pragma unroll
    for (int k1 = 1; k1 < 16; k1++) x[17 * k1] = cmul(v[dft_perm<16>(k1)], tw[k1]);
  }
  __syncwarp();
  if constexpr (RW % 2 == 1) {
    // lanes 0-15: pass 1 of row RW-1 (stride 17, twiddles); lanes 16-31: pass 2
    // of row 0 (stride 1, all sixteen outputs)
    float2* x = h ? rows0 + 17 * b : rows0 + (RW - 1) * kTRowStride + b;
    const int ls = h ? 1 : 17;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = x[ls * r];
    dft<16, 1>(v);
    x[0] = v[dft_perm<16>(0)];
#pragma unroll
    for (int k = 1; k < 16; k++) x[ls * k] = cmul(v[dft_perm<16>(k)], h ? make_float2(1.f, 0.f) : tw[k]);
    __syncwarp();
  }
  constexpr int R0 = RW % 2;   // first row left for pass 2
#pragma unroll
  for (int u = 0; u < PR; u++) {
    float2* x = rows0 + (R0 + ((lane + 32 * u) >> 4)) * kTRowStride + 17 * b;   // P16(16 b + n) = 17 b + n
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = x[r];
    if (edges) {
      dft16_head<1>(v);
      x[0] = cadd(cadd(v[0], v[2]), cadd(v[1], v[3]));
      x[1] = cadd(cadd(v[4], v[6]), cadd(v[5], v[7]));
      // output 3 of a DFT4: (u0 - u2) - i (u1 - u3)
      x[14] = csub(csub(v[8], v[10]), cmul_i<1>(csub(v[9], v[11])));
      x[15] = csub(csub(v[12], v[14]), cmul_i<1>(csub(v[13], v[15])));
    } else {
      dft<16, 1>(v);
#pragma unroll
      for (int k2 = 0; k2 < 16; k2++) x[k2] = v[dft_perm<16>(k2)];
    }
  }
}

// Spectrum bins of one group {k, HL-k, HL+k, Nz-k} of both stations: X1 and X2
// at k and HL-k, and (full spectra) at HL+k and Nz-k (0 for k = 0).  Half
// spectra (real traces) hold bins 0..HL only; their other two cross-spectrum
// values are conjugates of the first two, exactly as zbin forms them.
template <bool HERM>
struct GroupBins {
  float2 v[HERM ? 4 : 8];
};

template <int FMT, bool HERM, int HL>
__device__ __forceinline__ void load_group(GroupBins<HERM>& g, const char* X1, const char* X2, int k) {
  g.v[0] = load_bin<FMT>(X1, k);
  g.v[1] = load_bin<FMT>(X2, k);
  g.v[2] = load_bin<FMT>(X1, HL - k);
  g.v[3] = load_bin<FMT>(X2, HL - k);
  if constexpr (!HERM) {
    const int k3 = (k == 0) ? 0 : 2 * HL - k;
    g.v[4] = load_bin<FMT>(X1, HL + k);
    g.v[5] = load_bin<FMT>(X2, HL + k);
    g.v[6] = load_bin<FMT>(X1, k3);
    g.v[7] = load_bin<FMT>(X2, k3);
  }
}

// Hermitian parts 2H[k] = Z[k] + conj(Z[Nz-k]) and 2H[k+HL] = Z[HL+k] + conj(Z[HL-k])
// of Z = conj(X1) X2 (the values zbin gives), each as one fused sum of products.
template <bool HERM>
__device__ __forceinline__ void group_h(const GroupBins<HERM>& g, int k, float2& Hk, float2& Hkh) {
  const float2 a0 = g.v[0], b0 = g.v[1], a1 = g.v[2], b1 = g.v[3];
  if constexpr (HERM) {
    // half spectra: Z[HL+k] = conj(Z[HL-k]) and Z[Nz-k] = conj(Z[k]) for k > 0
    // (Z[0] and Z[HL] are real: bins of real sequences)
    const float2 z0 = cconjmul(a0, b0);
    const float2 z1 = cconjmul(a1, b1);
    if (k == 0) {
      Hk = make_float2(z0.x + z0.x, 0.0f);
      Hkh = make_float2(z1.x + z1.x, 0.0f);
    } else {
      Hk = make_float2(z0.x + z0.x, z0.y + z0.y);
      Hkh = make_float2(z1.x + z1.x, -(z1.y + z1.y));
    }
  } else {
    // conj(a) b + conj(conj(c) d) = conj(a) b + c conj(d)
    const float2 a3 = g.v[6], b3 = g.v[7], a2 = g.v[4], b2 = g.v[5];
    Hk = make_float2(fmaf(a0.x, b0.x, fmaf(a0.y, b0.y, fmaf(a3.x, b3.x, a3.y * b3.y))),
                     fmaf(a0.x, b0.y, fmaf(-a0.y, b0.x, fmaf(a3.y, b3.x, -a3.x * b3.y))));
    Hkh = make_float2(fmaf(a2.x, b2.x, fmaf(a2.y, b2.y, fmaf(a1.x, b1.x, a1.y * b1.y))),
                      fmaf(a2.x, b2.y, fmaf(-a2.y, b2.x, fmaf(a1.y, b1.x, -a1.x * b1.y))));
  }
}

template <int R1>
constexpr size_t tiled_smem_elems() {
  return (size_t)R1 * kTRowStride + 128 + tw_hi_len(2 * R1 * kTM) + 128 + tw_hi_len(R1 * kTM) + kTM;
}

template <int R1, int FMT, bool HERM>
__global__ void __launch_bounds__(kTM, 2) k_pairs_tiled(PairArgs a) {
  constexpr int M = kTM;
  constexpr int HL = R1 * M;       // inverse transform length (half of Nz)
  constexpr int NZ = 2 * HL;
  constexpr int RW = R1 / 8;       // tile rows per warp
  static_assert(R1 % 8 == 0, "rows per warp");
  constexpr int A = split_a(R1), B = split_b(R1);
  static_assert(A * B == R1, "stage-1 split");
  extern __shared__ float4 smem_raw[];
  float2* rows = reinterpret_cast<float2*>(smem_raw);
  float2* zlo = rows + R1 * kTRowStride;
  float2* zhi = zlo + 128;
  float2* hlo = zhi + tw_hi_len(NZ);
  float2* hhi = hlo + 128;
  float2* wm = hhi + tw_hi_len(HL);
  build_twiddles(zlo, zhi, NZ);
  build_twiddles(hlo, hhi, HL);
  for (int t = threadIdx.x; t < M; t += M) {
    float s, c;
    sincospif(2.0f * (float)t / (float)M, &s, &c);   // exp(+2 pi i t / M)
    wm[t] = make_float2(c, s);
  }
  __syncthreads();
  const TwTab twZ{zlo, zhi}, twH{hlo, hhi};

  // thread -> column j; columns j and M - j share the lanes l and l ^ 16 of a warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j0 = 16 * warp + (lane & 15);
  const int j = (lane < 16) ? j0 : (j0 == 0 ? M / 2 : M - j0);
  const bool self = (j == 0) || (j == M / 2);
  const int src = self ? lane : (lane ^ 16);
  float2 wj = twiddle(twZ, j);   // exp(+2 pi i j / Nz)
  wj.y = -wj.y;
  float2* rows_w = rows + warp * RW * kTRowStride;
  constexpr int esz = (FMT == SPEC_F32) ? 8 : 4;

  // station rows of correlation p
  auto rows_of = [&](int p, const char*& X1, const char*& X2) {
    if (a.desc) {
      X1 = reinterpret_cast<const char*>(a.desc[p].a);
      X2 = reinterpret_cast<const char*>(a.desc[p].b);
    } else {
      const int2 pr = a.pairs[p];
      X1 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.x * a.ldspec * esz;
      X2 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.y * a.ldspec * esz;
    }
  };
  for (int p = blockIdx.x; p < a.npairs; p += gridDim.x) {
    const char* X1;
    const char* X2;
    rows_of(p, X1, X2);

    // ---- stage 1: packed inputs F[j + M r], r < R1
    // F[k] = (H[k] + H[k+HL]) + i w^k (H[k] - H[k+HL]) with H the Hermitian part of
    // Z and w = exp(2 pi i / Nz); the group {k, HL-k} reads Z at k, HL-k, HL+k, Nz-k.
    float2 v[R1];
    sfor<0, R1 / 2>([&](auto ir) {
      constexpr int r = decltype(ir)::value;
      const int k = j + M * r;
      GroupBins<HERM> g;
      load_group<FMT, HERM, HL>(g, X1, X2, k);
      float2 Hk, Hkh;
      group_h<HERM>(g, k, Hk, Hkh);
      const float2 w = cmul_ct<r, 2 * R1, 1>(wj);    // exp(2 pi i (j + M r) / Nz)
      const float2 e = cadd(Hk, Hkh);
      const float2 d = csub(Hk, Hkh);
      const float2 o = cmul(w, d);
      v[r] = make_float2(e.x - o.y, e.y + o.x);
      // F[HL-k] from the same group: H[HL-k] = conj(H[k+HL]) and w^(HL-k) = -conj(w^k),
      // so its odd part is conj(o): F[HL-k] = conj(e) + i conj(o)
      float2 mir = make_float2(e.x + o.y, o.x - e.y);
      mir.x = __shfl_sync(0xffffffffu, mir.x, src);
      mir.y = __shfl_sync(0xffffffffu, mir.y, src);
      v[R1 - 1 - r] = mir;   // F[(M - j) + M (R1-1-r)] of the partner column
    });
    if (j == 0) {
      // column 0 mirrors onto itself one slot further: F[HL - M r] = F[M (R1 - r)];
      // the group k = HL/2 supplies F[HL/2] alone
#pragma unroll
      for (int s = R1 - 1; s > R1 / 2; s--) v[s] = v[s - 1];
      const int k = HL / 2;
      const float2 z0 = zbin<FMT, HERM>(X1, X2, k, NZ);
      const float2 z2 = zbin<FMT, HERM>(X1, X2, HL + k, NZ);
      const float2 Hk = cadd(z0, cconj(z2));   // Z[Nz - k] = Z[HL + k], Z[HL - k] = Z[k]
      const float2 Hkh = cadd(z2, cconj(z0));
      const float2 w = cmul_ct<R1 / 2, 2 * R1, 1>(make_float2(1.0f, 0.0f));
      const float2 e = cadd(Hk, Hkh);
      const float2 d = csub(Hk, Hkh);
      const float2 o = cmul(w, d);
      v[R1 / 2] = make_float2(e.x - o.y, e.y + o.x);
    }
    dft_ab<A, B, 1>(v);
    {
      // w_H^(j s) for s = 8 a + b: w_H^(8 j a) from the table (j s < HL), then
      // seven running products by u = w_H^j = (w_Nz^j)^2 (few live registers)
      const float2 u = cmul(wj, wj);
#pragma unroll
      for (int a8 = 0; a8 < R1 / 8; a8++) {
        float2 T;
        if (a8 == 0) {
          T = u;
        } else {
          T = twiddle(twH, 8 * a8 * j);
          T.y = -T.y;
          v[8 * a8] = cmul(v[8 * a8], T);
          T = cmul(T, u);
        }
#pragma unroll
        for (int bb = 1; bb < 8; bb++) {
          v[8 * a8 + bb] = cmul(v[8 * a8 + bb], T);
          if (bb < 7) T = cmul(T, u);
        }
      }
    }
    __syncthreads();   // the previous correlation's lags have been read out of the tile
#pragma unroll
    for (int s = 0; s < R1; s++) rows[s * kTRowStride + P16(j)] = v[s];
    __syncthreads();

    // ---- stage 2: M-point transforms of the warp's rows; when every output f
    // that stage 3 reads lies within 32 R1 of 0 (lags within about +-64 R1),
    // the rows' last pass forms only the outputs q in [-32, 32)
    {
      const int lag0 = a.desc ? a.desc[p].lag0 : a.lag0;
      const int L = a.desc ? a.desc[p].L : a.L;
      const int idx0 = lag0 < 0 ? lag0 + NZ : lag0;
      const int f0 = (idx0 >> 1) >= HL / 2 ? (idx0 >> 1) - HL : (idx0 >> 1);
      const int nout = (L + (idx0 & 1) + 1) >> 1;
      warp_dft256<RW>(rows_w, wm, lane, f0 >= -32 * R1 && f0 + nout <= 32 * R1);
    }
    __syncthreads();

    // ---- stage 3: the requested lags out of the tile
    float* y;
    const double* E1 = nullptr;
    const double* E2 = nullptr;
    int N, lag0, L;
    float scale;
    if (a.desc) {
      const PairDesc& dd = a.desc[p];
      y = reinterpret_cast<float*>(dd.y);
      if (a.norm == 1) { E1 = dd.ea; E2 = dd.eb; }
      N = dd.N;
      lag0 = dd.lag0;
      L = dd.L;
      scale = dd.scale != 0.0f ? dd.scale
                               : (a.norm == 0 ? 1.0f / ((float)NZ * (float)N) : (float)(1.0 / (double)NZ));
    } else {
      const int2 pr = a.pairs[p];
      y = a.y + (int64_t)p * a.ldy;
      if (a.norm == 1) {
        E1 = a.energy + (int64_t)pr.x * a.ldE;
        E2 = a.energy + (int64_t)pr.y * a.ldE;
      }
      N = a.N;
      lag0 = a.lag0;
      L = a.L;
      scale = a.scale;
    }
    if constexpr (FMT == SPEC_I16) scale *= i16_row_scale(X1) * i16_row_scale(X2);
    // X[f] holds the lags of indices 2f (real part) and 2f + 1 (imaginary part),
    // index = lag mod Nz; output m covers lag numbers 2m - e and 2m - e + 1
    // GNCC takes Hermitian spectra: the tables (GnccNorm) in those
    // instantiations; the full-spectrum ones keep the plain form, which holds
    // fewer registers
    GnccNorm gn;
    if constexpr (HERM) {
      if (a.norm == 1) gn.init(E1, E2, N);
    }
    const float hs = 0.5f * scale;
    const int idx0 = lag0 < 0 ? lag0 + NZ : lag0;
    const int e = idx0 & 1;
    const int nout = (L + e + 1) >> 1;
    // GNCC: a lag the tables cannot take (energies out of their range, or rows
    // without tables) is stored unnormalised and fixed after the loop, which
    // keeps the FP64 branch out of the loop's registers
    bool fix = false;
    auto put = [&](int l, float val) {
      const int lag = lag0 + l;
      val *= hs;
      if (a.norm == 1) {
        if constexpr (HERM) {
          const float pr = gn.tab ? gn.table(lag) : 0.0f;
          if (pr > 0.0f) val *= pr;
          else fix = true;
        } else {
          val = gncc_lag_norm(val, E1, E2, N, lag);
        }
      } else if (a.norm == 2) {
        val = val / (float)(N - abs(lag));
      }
      y[l] = val;
    };
#pragma unroll 2
    for (int m = threadIdx.x; m < nout; m += M) {
      int f = (idx0 >> 1) + m;
      if (f >= HL) f -= HL;
      const int q = f / R1;
      const float2 zz = rows[(f - q * R1) * kTRowStride + out_pos(q)];
      const int l = 2 * m - e;
      if (l >= 0) put(l, zz.x);
      if (l + 1 < L) put(l + 1, zz.y);
    }
    if constexpr (HERM) {
      if (fix) {
        // this thread's lags again: the ones the tables could not take
        for (int m = threadIdx.x; m < nout; m += M)
          for (int h = 0; h < 2; h++) {
            const int l = 2 * m - e + h;
            if (l < 0 || l >= L) continue;
            const int lag = lag0 + l;
            if (!(gn.tab && gn.table(lag) > 0.0f)) y[l] = gncc_lag_norm(y[l], E1, E2, N, lag);
          }
      }
    }
  }
}

int g_sms[64] = {0};

int resident_blocks(int dev, const void* kern, size_t smem) {
  if (dev < 0 || dev >= 64) return 152 * 2;
  if (g_sms[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    g_sms[dev] = n;
  }
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kTM, smem) != cudaSuccess || per <= 0) per = 1;
  return g_sms[dev] * per;
}

template <int R1, int FMT, bool HERM>
cudaError_t launch_tiled_t(const PairArgs& a, cudaStream_t st) {
  auto kern = k_pairs_tiled<R1, FMT, HERM>;
  const size_t smem = tiled_smem_elems<R1>() * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  const int cap = resident_blocks(dev, (const void*)kern, smem);
  const int grid = a.npairs < cap ? a.npairs : cap;
  void* argv[] = {const_cast<PairArgs*>(&a)};
  return cudaLaunchKernel((const void*)kern, dim3(grid), dim3(kTM), argv, smem, st);
}

template <int R1>
cudaError_t launch_tiled_r(const PairArgs& a, cudaStream_t st) {
  const bool herm = (a.norm != 0);
  if (a.fmt == SPEC_I16) return herm ? cudaErrorInvalidValue : launch_tiled_t<R1, SPEC_I16, false>(a, st);
  if (a.fmt == SPEC_F16) return herm ? launch_tiled_t<R1, SPEC_F16, true>(a, st) : launch_tiled_t<R1, SPEC_F16, false>(a, st);
  return herm ? launch_tiled_t<R1, SPEC_F32, true>(a, st) : launch_tiled_t<R1, SPEC_F32, false>(a, st);
}

}  // namespace

bool pair_tiled_supported(int Nz) { return Nz == 2 * 40 * kTM || Nz == 2 * 32 * kTM; }

cudaError_t launch_pairs_tiled(const PairArgs& a, cudaStream_t st) {
  if (a.npairs <= 0) return cudaSuccess;
  switch (a.Nz) {
    case 2 * 40 * kTM: return launch_tiled_r<40>(a, st);
    case 2 * 32 * kTM: return launch_tiled_r<32>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fpcc
