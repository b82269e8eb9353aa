// Wavelet phase cross-correlation (reference tspcc2_set, src/FFTapps.c:1076-1255,
// and its GPU twin cuda_tspcc2_set_freq, src/ccs_cuda.cu:898-1036).
//
// Station stage (per station window, all scales):
//   X   = DFT_Nz(x / Nz placed at offset Ls0)                          (:1185-1197)
//   B_s = IDFT_Nz(X * W_s),  W_s = DFT_Nz of the wavelet taps placed
//         circularly around index 0                                     (:1137-1149,1204-1205)
//   P_s = DFT_Nz(amplitude-normalised B_s)                              (:1206-1207)
// Pair stage (per pair window):
//   Y = sum_s conj(P1_s) P2_s / (scale_s Nz)                            (:1217-1218)
//   y = C Re IDFT_Nz(Y) at the lags, C = 1/(K0 N)                       (:1220-1224)
// All transforms use the four-step kernels; P_s is the cached station product.
// Any length >= N + M + Ls0 gives the reference's values (every operation is a
// linear convolution inside that support), so the planner may pick a shorter
// length than the reference's power of two.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/fastpcc_gb300.h"
#include "engine.h"
#include "large.cuh"
#include "wavelet.h"
#include "wpcc.h"

namespace fpcc {

namespace {

__global__ void __launch_bounds__(256) k_wpcc_accum(const void* __restrict__ P, int fmt, int S, int Nz,
                                                    const int2* __restrict__ pairs, int npairs,
                                                    const float* __restrict__ a_s, float2* __restrict__ Y) {
  const int p = blockIdx.y;
  const int2 pr = pairs[p];
  const int64_t row = (int64_t)S * Nz;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < Nz; k += gridDim.x * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int s = 0; s < S; s++) {
      float2 u, v;
      const int64_t o1 = pr.x * row + (int64_t)s * Nz + k, o2 = pr.y * row + (int64_t)s * Nz + k;
      if (fmt == SPEC_F16) {
        u = __half22float2(reinterpret_cast<const __half2*>(P)[o1]);
        v = __half22float2(reinterpret_cast<const __half2*>(P)[o2]);
      } else {
        u = reinterpret_cast<const float2*>(P)[o1];
        v = reinterpret_cast<const float2*>(P)[o2];
      }
      const float w = a_s[s];
      acc.x = fmaf(w, fmaf(u.x, v.x, u.y * v.y), acc.x);
      acc.y = fmaf(w, fmaf(u.x, v.y, -u.y * v.x), acc.y);
    }
    Y[(int64_t)p * Nz + k] = acc;
  }
}

}  // namespace

// A usable WPCC length: both Nz and Nz/2 run as four-step transforms.
static bool wpcc_len_ok(int nz) {
  int a, b;
  return nz > 0 && nz % 2 == 0 && large_supported(nz, &a, &b) && large_supported(nz / 2, &a, &b);
}

int wpcc_choose_nz(const WpccSetup& su, unsigned N, int nz_mode) {
  if (nz_mode >= 2) return wpcc_len_ok(nz_mode) && (unsigned)nz_mode >= N + su.M + su.Ls0 ? nz_mode : -1;
  bool capped = false;
  for (unsigned s = 0; s < su.wf.S; s++) capped |= (su.wf.Ls[s] >= su.Nz0);
  if (nz_mode == 0 || capped) return wpcc_len_ok((int)su.Nz_ref) ? (int)su.Nz_ref : -1;
  const int need = (int)(N + su.M + su.Ls0);
  for (int nz : smooth235_in(need, (int)su.Nz_ref))
    if (!(nz & 1) && wpcc_len_ok(nz)) return nz;
  return wpcc_len_ok((int)su.Nz_ref) ? (int)su.Nz_ref : -1;
}

cudaError_t wpcc_filters(const WaveletFamily& wf, int Nz, float2* d_W, float2* d_tmp_T, float2* d_stage,
                         cudaStream_t st) {
  const unsigned S = wf.S;
  std::vector<float2> h((size_t)S * Nz);
  std::memset(h.data(), 0, h.size() * sizeof(float2));
  for (unsigned s = 0; s < S; s++) {
    // taps[c..Ls) at 0.., taps[0..c) at Nz-c.. (src/FFTapps.c:1143-1145)
    const int c = wf.center[s];
    const int L = (int)wf.Ls[s];
    float2* f = h.data() + (size_t)s * Nz;
    for (int n = 0; n < L - c; n++)
      f[n] = make_float2((float)wf.taps[s][c + n].real(), (float)wf.taps[s][c + n].imag());
    for (int n = 0; n < c; n++)
      f[Nz - c + n] = make_float2((float)wf.taps[s][n].real(), (float)wf.taps[s][n].imag());
  }
  cudaError_t e = cudaMemcpyAsync(d_stage, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  int n1, n2;
  large_supported(Nz, &n1, &n2);
  LargeArgs a{};
  a.n = Nz; a.n1 = n1; a.n2 = n2; a.dir = -1; a.nrows = (int)S;
  a.cmode = COL_COMPLEX; a.in = d_stage; a.ldin = Nz; a.N = Nz; a.in_scale = 1.f;
  a.T = d_tmp_T;
  a.rmode = ROW_SPEC; a.out = d_W; a.ldo = Nz; a.out_fmt = SPEC_F32; a.out_half = 0;
  e = launch_large(a, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);   // h must outlive the copy
}

cudaError_t wpcc_station(const WpccPlanDev& pl, const float* d_x, int64_t ldx, int nrows, void* d_P, int fmt,
                         float2* d_X, float2* d_T, float2* d_band, float* d_rowmax, int chunk_sw, cudaStream_t st) {
  const int Nz = pl.Nz, S = pl.S;
  int n1, n2;
  large_supported(Nz, &n1, &n2);
  const size_t pesz = (fmt == SPEC_F16) ? 4 : 8;
  cudaError_t e;
  for (int r0 = 0; r0 < nrows; r0 += chunk_sw) {
    const int cnt = (nrows - r0) < chunk_sw ? (nrows - r0) : chunk_sw;
    // X = DFT(x / Nz at offset Ls0)
    LargeArgs a{};
    a.n = Nz; a.n1 = n1; a.n2 = n2; a.dir = -1; a.nrows = cnt;
    a.cmode = COL_REAL; a.in = d_x + (size_t)r0 * ldx; a.ldin = ldx; a.N = pl.N; a.in_off = pl.Ls0;
    a.in_scale = 1.0f / (float)Nz;
    a.T = d_T;
    a.rmode = ROW_COMPLEX; a.out = d_X; a.ldo = Nz; a.rowmax = nullptr;
    if ((e = launch_large(a, st)) != cudaSuccess) return e;
    // bands: rows (window, scale)
    const int rows = cnt * S;
    if ((e = cudaMemsetAsync(d_rowmax, 0, (size_t)rows * sizeof(float), st)) != cudaSuccess) return e;
    LargeArgs b{};
    b.n = Nz; b.n1 = n1; b.n2 = n2; b.dir = +1; b.nrows = rows;
    b.cmode = COL_PRODUCT; b.in = d_X; b.ldin = Nz; b.filt = pl.d_W; b.ldfilt = Nz; b.filt_of_row_div = S;
    b.filt_conj = pl.filt_conj; b.in_scale = 1.0f; b.N = Nz;
    b.T = d_T;
    b.rmode = ROW_COMPLEX; b.out = d_band; b.ldo = Nz; b.rowmax = d_rowmax;
    if ((e = launch_large(b, st)) != cudaSuccess) return e;
    // phase spectra
    LargeArgs c{};
    c.n = Nz; c.n1 = n1; c.n2 = n2; c.dir = -1; c.nrows = rows;
    c.cmode = COL_NORMALISE; c.in = d_band; c.ldin = Nz; c.rule = pl.rule; c.rowstat = d_rowmax; c.N = Nz;
    c.T = d_T;
    c.rmode = ROW_SPEC; c.out = (char*)d_P + (size_t)r0 * S * Nz * pesz; c.ldo = Nz; c.out_fmt = fmt; c.out_half = 0;
    if ((e = launch_large(c, st)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t wpcc_pairs(const WpccPlanDev& pl, const void* d_P, int fmt, const int2* d_pairs, int npairs,
                       float* d_y, int64_t ldy, float2* d_Y, float2* d_T, int chunk_p, cudaStream_t st) {
  const int Nz = pl.Nz, h = Nz / 2;
  int n1, n2;
  large_supported(h, &n1, &n2);
  cudaError_t e;
  for (int p0 = 0; p0 < npairs; p0 += chunk_p) {
    const int cnt = (npairs - p0) < chunk_p ? (npairs - p0) : chunk_p;
    dim3 grid((Nz + 255) / 256 < 512 ? (Nz + 255) / 256 : 512, cnt);
    k_wpcc_accum<<<grid, 256, 0, st>>>(d_P, fmt, pl.S, Nz, d_pairs + p0, cnt, pl.d_a, d_Y);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    LargeArgs a{};
    a.n = h; a.n1 = n1; a.n2 = n2; a.dir = +1; a.nrows = cnt;
    a.cmode = COL_PAIR; a.spec = d_Y; a.ldspec = Nz; a.fmt = SPEC_F32; a.herm = 2; a.Nz = Nz;
    a.T = d_T;
    a.rmode = ROW_LAGS; a.lag0 = pl.lag0; a.L = pl.L; a.scale = pl.C; a.norm = 0; a.N = pl.N;
    a.y = d_y + (size_t)p0 * ldy; a.ldy = ldy;
    if ((e = launch_large(a, st)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace fpcc
