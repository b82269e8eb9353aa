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
// B_s and P_s of a (window, scale) row run on a thread-block cluster that holds
// the row in its blocks' shared memories where Nz is on that kernel's menu
// (k_wpcc_rows below), else as four-step kernels like every other transform
// here; P_s is the cached station product.
// Any length >= N + M + Ls0 gives the reference's values (every operation is a
// linear convolution inside that support), so the planner may pick a shorter
// length than the reference's power of two.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
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

// ---------------------------------------------------------------- whole rows on a cluster
// The band and phase-spectrum transforms of one (window, scale) row, N = R Q
// points, on a cluster of R = 4 or 8 blocks whose shared memories hold the
// row between the transforms (no global-memory round trip):
//   inverse:           z_k[f] = w_N^(+k f) sum_j Y[f + Q j] w_R^(+k j),  Y = X W_s
//                      (block k reads the band at f in [k Q/R, (k+1) Q/R) only
//                      and stores z_r[f] of every r into block r),
//                      x[R m + k] = IDFT_Q(z_k)[m]                      (in place)
//   normalise:         x *= factor(|x|^2, eps(max over the R blocks))
//   forward, block k:  Z_k = DFT_Q(x[R m + k]),  then
//                      P[f + Q j] = sum_r w_R^(-r j) w_N^(-r f) Z_r[f]   (Z_r read from block r;
//                      block k writes every j at its share of f)
// The same arithmetic as the four-step passes (`launch_large` with the band
// product, the row maximum, the normalising load and the spectrum store) in
// another order of the FFT's butterflies.
template <int... Rs>
__host__ __device__ constexpr int prod_radices_of(Radices<Rs...>) {
  return prod_radices<Rs...>();
}

constexpr int kRowThreads = 1024;

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// all threads of all blocks of the cluster: shared-memory writes before it are seen by
// the cluster's reads after it
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// address of the same shared-memory location in block `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 cluster_ld2(uint32_t addr) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}
__device__ __forceinline__ void cluster_st2(uint32_t addr, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float cluster_ld(uint32_t addr) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}
// v * i^q
__device__ __forceinline__ float2 rot_quarter(float2 v, int q) {
  switch (q & 3) {
    case 0: return v;
    case 1: return make_float2(-v.y, v.x);
    case 2: return make_float2(-v.x, -v.y);
    default: return make_float2(v.y, -v.x);
  }
}
// v * w_R^q = v * exp(2 pi i q / R) for R = 4 or 8
template <int R>
__device__ __forceinline__ float2 rot_root(float2 v, int q) {
  static_assert(R == 4 || R == 8, "cluster sizes");
  if constexpr (R == 4) {
    return rot_quarter(v, q);
  } else {
    const float2 t = rot_quarter(v, (q & 7) >> 1);
    if (!(q & 1)) return t;
    const float h = 0.70710678118654752440f;   // w_8 = (1 + i) / sqrt(2)
    return make_float2(h * (t.x - t.y), h * (t.x + t.y));
  }
}

struct WpccRowArgs {
  const float2* X;     // window spectra of the chunk, Nz per row
  const float2* W;     // S x Nz wavelet spectra
  int S, filt_conj, rule, fmt;
  void* out;           // phase spectra, row = window * S + scale, Nz per row (fmt F32 / F16)
};

inline int row_smem_floats2(int R, int Q) {
  return padded_len(Q) + 128 + tw_hi_len(Q) + 128 + tw_hi_len(R * Q) + 17;
}

template <int R, typename RADQ>
__global__ void __cluster_dims__(R, 1, 1) __launch_bounds__(kRowThreads, 1) k_wpcc_rows(WpccRowArgs a) {
  constexpr int kRowRanks = R;
  constexpr int Q = prod_radices_of(RADQ{});
  constexpr int N = kRowRanks * Q;
  constexpr int T = kRowThreads;
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* qlo = s + padded_len(Q);
  float2* qhi = qlo + 128;
  float2* nlo = qhi + tw_hi_len(Q);
  float2* nhi = nlo + 128;
  float* red = reinterpret_cast<float*>(nhi + tw_hi_len(N));   // 33 floats
  const int k = (int)cluster_rank();
  const int row = blockIdx.x / kRowRanks;
  const float2* Xr = a.X + (int64_t)(row / a.S) * N;
  const float2* Wr = a.W + (int64_t)(row % a.S) * N;
  build_twiddles(qlo, qhi, Q);
  build_twiddles(nlo, nhi, N);
  __syncthreads();
  const TwTab twN{nlo, nhi};
  cluster_sync();   // every block of the cluster is running: its shared memory can be written
  // inverse transform: the R decimations z_r of the band Y = X W_s at this
  // block's share of f (two points per thread at a time, so that 4 R loads
  // are in flight), each stored into block r
  uint32_t base[kRowRanks];
#pragma unroll
  for (int r = 0; r < kRowRanks; r++) base[r] = cluster_addr(s, (uint32_t)r);
  constexpr int QB = Q / kRowRanks;
  static_assert(Q % kRowRanks == 0, "share of the row");
#pragma unroll 2
  for (int f = k * QB + (int)threadIdx.x; f < (k + 1) * QB; f += T) {
    float2 y[kRowRanks];
#pragma unroll
    for (int j = 0; j < kRowRanks; j++) {
      float2 w = __ldg(Wr + f + Q * j);
      if (a.filt_conj) w.y = -w.y;
      y[j] = cmul(__ldg(Xr + f + Q * j), w);
    }
#pragma unroll
    for (int r = 0; r < kRowRanks; r++) {
      float2 acc = y[0];
#pragma unroll
      for (int j = 1; j < kRowRanks; j++) acc = cadd(acc, rot_root<R>(y[j], r * j));
      if (r) {
        float2 t = twiddle(twN, r * f);   // exp(-2 pi i r f / N); r f < N
        t.y = -t.y;
        acc = cmul(acc, t);
      }
      cluster_st2(base[r] + (uint32_t)PADI(f) * 8u, acc);
    }
  }
  cluster_sync();   // every block's z_k complete
  ct_fft<+1, T, 1>(s, 1, 0, TwTab{qlo, qhi}, RADQ{});
  // the row's maximum |x|^2 over the R blocks
  float mx = 0.f;
  for (int i = threadIdx.x; i < Q; i += T) {
    const float2 v = s[PADI(i)];
    mx = fmaxf(mx, v.x * v.x + v.y * v.y);
  }
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = (threadIdx.x < T / 32) ? red[threadIdx.x] : 0.f;
    v = warp_max(v);
    if (threadIdx.x == 0) red[32] = v;
  }
  cluster_sync();
  float gm = 0.f;
#pragma unroll
  for (int r = 0; r < kRowRanks; r++) gm = fmaxf(gm, cluster_ld(cluster_addr(red + 32, (uint32_t)r)));
  const float eps = eps_of(a.rule, gm);
  for (int i = threadIdx.x; i < Q; i += T) {
    const float2 v = s[PADI(i)];
    s[PADI(i)] = cscale(v, factor_of(a.rule, v.x * v.x + v.y * v.y, eps));
  }
  __syncthreads();
  ct_fft<-1, T, 1>(s, 1, 0, TwTab{qlo, qhi}, RADQ{});
  cluster_sync();   // every block's Z_r complete (and its maximum read)
  // the spectrum at this block's share of f in all R output parts j, from
  // the R blocks' Z_r[f]
  const int64_t o = (int64_t)row * N;
#pragma unroll 2
  for (int f = k * QB + (int)threadIdx.x; f < (k + 1) * QB; f += T) {
    float2 z[kRowRanks];
    z[0] = cluster_ld2(base[0] + (uint32_t)PADI(f) * 8u);
#pragma unroll
    for (int r = 1; r < kRowRanks; r++) z[r] = cmul(cluster_ld2(base[r] + (uint32_t)PADI(f) * 8u), twiddle(twN, r * f));
#pragma unroll
    for (int j = 0; j < kRowRanks; j++) {
      float2 acc = z[0];
#pragma unroll
      for (int r = 1; r < kRowRanks; r++) acc = cadd(acc, rot_root<R>(z[r], -r * j));
      if (a.fmt == SPEC_F16) reinterpret_cast<__half2*>(a.out)[o + f + (int64_t)Q * j] = __float22half2_rn(acc);
      else reinterpret_cast<float2*>(a.out)[o + f + (int64_t)Q * j] = acc;
    }
  }
  cluster_sync();   // no block leaves while the others read its shared memory
}

// The cluster kernel for row length Nz (Nz = R Q with R = 4 or 8 blocks and Q
// on its menu), or null; `smem` and `ranks` receive its dynamic shared memory
// and cluster size.  The first call for a length sets the kernel's
// shared-memory limit and checks that a cluster of such blocks can be
// resident.
using RowKernel = void (*)(WpccRowArgs);
RowKernel row_kernel(int Nz, size_t* smem, int* ranks) {
  struct Entry { RowKernel fn; int R, Q; size_t smem; int ok; };
  static Entry menu[6] = {{k_wpcc_rows<4, Radices<16, 16, 16, 4>>, 4, 16384, 0, -1},
                          {k_wpcc_rows<4, Radices<8, 8, 8, 8, 5>>, 4, 20480, 0, -1},
                          {k_wpcc_rows<4, Radices<8, 8, 8, 8, 6>>, 4, 24576, 0, -1},
                          {k_wpcc_rows<8, Radices<16, 16, 16, 4>>, 8, 16384, 0, -1},
                          {k_wpcc_rows<8, Radices<8, 8, 8, 8, 5>>, 8, 20480, 0, -1},
                          {k_wpcc_rows<8, Radices<8, 8, 8, 8, 6>>, 8, 24576, 0, -1}};
  if (const char* e = getenv("FPCC_WPCC_CLUSTER"))
    if (e[0] == '0') return nullptr;
  // one first-use check per entry, whichever host thread gets there first
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  for (Entry& en : menu) {
    if (Nz != en.R * en.Q) continue;
    if (en.ok < 0) {
      en.smem = (size_t)row_smem_floats2(en.R, en.Q) * sizeof(float2);
      en.ok = 0;
      if (cudaFuncSetAttribute(en.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)en.smem) == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)en.R);
        cfg.blockDim = dim3(kRowThreads);
        cfg.dynamicSmemBytes = en.smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)en.R;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, en.fn, &cfg) == cudaSuccess && n > 0) en.ok = 1;
      }
      cudaGetLastError();
    }
    if (en.ok != 1) return nullptr;
    *smem = en.smem;
    *ranks = en.R;
    return en.fn;
  }
  return nullptr;
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
    size_t rsmem = 0;
    int ranks = 0;
    if (RowKernel rk = row_kernel(Nz, &rsmem, &ranks)) {
      // whole rows on clusters of four or eight blocks
      WpccRowArgs r{};
      r.X = d_X; r.W = pl.d_W; r.S = S; r.filt_conj = pl.filt_conj; r.rule = pl.rule; r.fmt = fmt;
      r.out = (char*)d_P + (size_t)r0 * S * Nz * pesz;
      rk<<<dim3((unsigned)rows * (unsigned)ranks), kRowThreads, rsmem, st>>>(r);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      continue;
    }
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
