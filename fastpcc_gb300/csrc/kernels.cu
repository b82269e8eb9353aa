// FFT-based correlation kernels (PCC2, GNCC, 1-bit GNCC) and the generic
// transform passes.
//
// Station spectrum stage, one block per station window, length Nz on the size
// menu (reference src/FFTapps.c):
//   SPEC_PHASE : analytic signal -> amplitude normalisation (:178-205 or the GPU
//                rules of src/ccs_cuda.cu) -> zero pad -> DFT_Nz, all Nz bins
//   SPEC_REAL  : trace -> zero pad -> DFT_Nz, bins 0..Nz/2              (:940-946)
//   SPEC_SIGN  : 1-bit signs (:1037,1042) -> zero pad -> DFT_Nz, bins 0..Nz/2
// Pair stage, one block per (station pair, window):
//   Z = conj(X1) X2 (:851, :347), y = Re IDFT_Nz(Z) at the requested lags, as one
//   complex IDFT of Nz/2 points of the packed Hermitian part of Z; scaled
//   (:832,855-856) and, for GNCC / 1-bit, divided by the overlap norms (:372-429).
// Generic passes: one radix-R Stockham pass per launch over all rows, for window
// lengths N that are not on the menu (the N-point analytic signal, :104-124).
#include <float.h>

#include <atomic>

#include <cooperative_groups.h>

#include "kernels.cuh"
#include "menu.cuh"

namespace cg = cooperative_groups;

namespace fpcc {

namespace {

__device__ __forceinline__ bool f_isnormal_pos(float v) { return v >= FLT_MIN && v <= FLT_MAX; }

// Reference threshold / regulariser from the row statistic.
__device__ __forceinline__ float amp_eps(int rule, float ref) {
  if (rule == AMP_F_REG) return (float)(1e-6 * sqrt((double)ref));   // src/FFTapps.c:191
  if (rule == AMP_PURE) return 0.0f;                                  // src/ccs_cuda.cu:582
  return 1e-6f * ref;                                                 // :160, ccs_cuda.cu:197
}

// Factor that maps a sample of squared modulus m2 to its phase-signal value.
__device__ __forceinline__ float amp_factor(int rule, float m2, float eps) {
  float f;
  if (rule == AMP_F_REG) {
    f = 1.0f / (sqrtf(m2) + eps);   // src/FFTapps.c:196-203
    return f_isnormal_pos(f) ? f : 0.0f;
  }
  if (rule == AMP_D_REG) {
    f = rsqrtf(m2 + eps);           // src/FFTapps.c:166-173
    return f_isnormal_pos(f) ? f : 0.0f;
  }
  return (m2 > eps) ? rsqrtf(m2) : 0.0f;   // src/ccs_cuda.cu:201-208, 223-230
}

// v / sqrt(e1 e2) for the overlap energies e1, e2 (exact FP64 differences of the
// prefix sums): FP32 reciprocal square roots in the normal range, FP64 outside it.

template <int... Rs>
constexpr int rad_len(Radices<Rs...>) {
  return prod_radices<Rs...>();
}

// ------------------------------------------------------------ station spectra
template <int T, typename RAD>
__global__ void __launch_bounds__(T, 1) k_spec(SpecArgs a) {
  constexpr int NZ = rad_len(RAD{});
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* lo = s + padded_len(NZ);
  float2* hi = lo + 128;
  build_twiddles(lo, hi, NZ);
  const int row = blockIdx.x;
  const int N = a.N;
  if (a.mode == SPEC_PHASE) {
    const float2* x = reinterpret_cast<const float2*>(a.in) + (int64_t)row * a.ldin;
    const int rule = a.rule;
    const float eps = amp_eps(rule, a.rowstat[row]);
    for (int n = threadIdx.x; n < N; n += T) {
      const float2 v = x[n];
      s[PADI(n)] = cscale(v, amp_factor(rule, v.x * v.x + v.y * v.y, eps));
    }
  } else {
    const float* x = reinterpret_cast<const float*>(a.in) + (int64_t)row * a.ldin;
    const bool sgn = (a.mode == SPEC_SIGN);
    const bool ge = a.sign_ge != 0;
    for (int n = threadIdx.x; n < N; n += T) {
      float v = __ldg(x + n);
      if (sgn) v = (ge ? (v >= 0.0f) : (v > 0.0f)) ? 1.0f : -1.0f;
      s[PADI(n)] = make_float2(v, 0.0f);
    }
  }
  for (int n = N + threadIdx.x; n < NZ; n += T) s[PADI(n)] = make_float2(0.0f, 0.0f);
  __syncthreads();
  ct_fft<-1, T, 1>(s, 1, 0, TwTab{lo, hi}, RAD{});
  const int nout = (a.mode == SPEC_PHASE) ? NZ : (NZ / 2 + 1);
  if (a.fmt == SPEC_I16) {
    __shared__ float scratch[32];
    store_i16_row<T>(s, nout, reinterpret_cast<char*>(a.out) + (int64_t)row * a.ldo * 4, scratch);
  } else if (a.fmt == SPEC_F16) {
    __half2* o = reinterpret_cast<__half2*>(a.out) + (int64_t)row * a.ldo;
    for (int k = threadIdx.x; k < nout; k += T) o[k] = __float22half2_rn(s[PADI(k)]);
  } else {
    float2* o = reinterpret_cast<float2*>(a.out) + (int64_t)row * a.ldo;
    for (int k = threadIdx.x; k < nout; k += T) o[k] = s[PADI(k)];
  }
}

// ------------------------------------------------------------ CWT rows
// One block per row: X[row][m] * F[m] in shared memory, the inverse transform
// (unnormalised; F carries the 1/M), the first L values stored (stride ldo).
template <int T, typename RAD>
__global__ void __launch_bounds__(T, 1) k_cwt_rows(CwtRowArgs a) {
  constexpr int NZ = rad_len(RAD{});
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* lo = s + padded_len(NZ);
  float2* hi = lo + 128;
  build_twiddles(lo, hi, NZ);
  const int row = blockIdx.x;
  const float2* x = a.X + (int64_t)row * NZ;
  for (int m = threadIdx.x; m < NZ; m += T) {
    const float2 u = x[m], f = __ldg(a.F + m);
    s[PADI(m)] = make_float2(u.x * f.x - u.y * f.y, u.x * f.y + u.y * f.x);
  }
  __syncthreads();
  ct_fft<+1, T, 1>(s, 1, 0, TwTab{lo, hi}, RAD{});
  float2* o = a.out + (int64_t)row * a.ldo;
  for (int k = threadIdx.x; k < a.L; k += T) o[k] = s[PADI(k)];
}

// ------------------------------------------------------------ pairs
// Block size of the pair kernel for a half length H: enough threads that every
// pass stages at most 16-24 complex values per thread.
__host__ __device__ constexpr int pair_threads(int H) {
  return H / 10 < 128 ? 128 : (H / 10 > 1024 ? 1024 : ((H / 10 + 31) / 32) * 32);
}

// Pair kernel: one block per pair; blocks are issued in pair order, so blocks
// running together work on neighbouring pairs, which share station spectra in L2.
// Two transform buffers (ping-pong passes) when they fit one block's shared memory.
__host__ __device__ constexpr bool pair_pingpong(int H) {
  return (2LL * (H + (H >> 5) + 1) + 128 + (H + 127) / 128 + 128 + (2 * H + 127) / 128) * 8 <= 227LL * 1024;
}

template <int T, typename RAD, int FMT, bool HERM>
__global__ void __launch_bounds__(T, 1) k_pairs(PairArgs a) {
  constexpr int H = rad_len(RAD{});
  constexpr int NZ = 2 * H;
  constexpr bool PP = pair_pingpong(H);
  extern __shared__ float4 smem_raw[];
  float2* s = reinterpret_cast<float2*>(smem_raw);
  float2* s2 = s + (PP ? padded_len(H) : 0);
  float2* hlo = s2 + padded_len(H);
  float2* hhi = hlo + 128;
  float2* zlo = hhi + tw_hi_len(H);
  float2* zhi = zlo + 128;
  build_twiddles(hlo, hhi, H);
  build_twiddles(zlo, zhi, NZ);
  __syncthreads();
  const TwTab twZ{zlo, zhi};
  constexpr int esz = (FMT == SPEC_F32) ? 8 : 4;
  {
    const int p = blockIdx.x;
    const char* X1;
    const char* X2;
    if (a.desc) {
      X1 = reinterpret_cast<const char*>(a.desc[p].a);
      X2 = reinterpret_cast<const char*>(a.desc[p].b);
    } else {
      const int2 pr = a.pairs[p];
      X1 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.x * a.ldspec * esz;
      X2 = reinterpret_cast<const char*>(a.spec) + (int64_t)pr.y * a.ldspec * esz;
    }

    // F[k] = (H[k] + H[k+h]) + i w^k (H[k] - H[k+h]), H = Hermitian part of Z,
    // w = exp(2 pi i / Nz); the group {k, h-k} reads Z at k, h-k, h+k, Nz-k.
    // 2H is formed (the 1/2 goes into the output scale) and w^(h-k) = -conj(w^k).
#pragma unroll 1
    for (int k = threadIdx.x; k <= (H >> 1); k += T) {
      const int k2 = H - k;
      const float2 z0 = zbin<FMT, HERM>(X1, X2, k, NZ);
      const float2 z1 = zbin<FMT, HERM>(X1, X2, k2, NZ);
      const float2 z2 = zbin<FMT, HERM>(X1, X2, H + k, NZ);
      const float2 z3 = zbin<FMT, HERM>(X1, X2, (k == 0) ? 0 : NZ - k, NZ);
      const float2 Hk = cadd(z0, cconj(z3));
      const float2 Hkh = cadd(z2, cconj(z1));
      float2 w = twiddle(twZ, k);
      w.y = -w.y;
      const float2 e = cadd(Hk, Hkh);
      const float2 d = csub(Hk, Hkh);
      const float2 o = cmul(w, d);
      s[PADI(k)] = make_float2(e.x - o.y, e.y + o.x);
      if (k2 != k && k2 < H) {
        // H[k2] = conj(H[k+h]), H[k2+h] = conj(H[k]); w^k2 = -conj(w^k)
        const float2 w2 = make_float2(-w.x, w.y);
        const float2 e2 = cconj(e);
        const float2 o2 = cmul(w2, make_float2(-d.x, d.y));
        s[PADI(k2)] = make_float2(e2.x - o2.y, e2.y + o2.x);
      }
    }
    __syncthreads();
    const float2* res = s;
    if constexpr (PP) {
      res = pp_fft<+1, T>(s, s2, TwTab{hlo, hhi}, RAD{});
    } else {
      ct_fft<+1, T, 1>(s, 1, 0, TwTab{hlo, hhi}, RAD{});
    }

    float* y;
    const double* E1 = nullptr;
    const double* E2 = nullptr;
    int N, lag0, L;
    float scale;
    if (a.desc) {
      const PairDesc& d = a.desc[p];
      y = reinterpret_cast<float*>(d.y);
      if (a.norm == 1) { E1 = d.ea; E2 = d.eb; }
      N = d.N;
      lag0 = d.lag0;
      L = d.L;
      scale = d.scale != 0.0f ? d.scale
                              : (a.norm == 0 ? 1.0f / ((float)NZ * (float)N) : (float)(1.0 / (double)NZ));
      if constexpr (FMT == SPEC_I16) scale *= i16_row_scale(d.a) * i16_row_scale(d.b);
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
      if constexpr (FMT == SPEC_I16) {
        const char* sp = reinterpret_cast<const char*>(a.spec);
        scale *= i16_row_scale(sp + (int64_t)pr.x * a.ldspec * 4) * i16_row_scale(sp + (int64_t)pr.y * a.ldspec * 4);
      }
    }
    GnccNorm gn;
    if (a.norm == 1) gn.init(E1, E2, N);
    for (int l = threadIdx.x; l < L; l += T) {
      const int lag = lag0 + l;
      const int idx = lag < 0 ? lag + NZ : lag;
      const float2 zz = res[PADI(idx >> 1)];
      float v = ((idx & 1) ? zz.y : zz.x) * (0.5f * scale);
      if (a.norm == 1) {
        v = gn.apply(v, lag);
      } else if (a.norm == 2) {
        v = v / (float)(N - abs(lag));
      }
      y[l] = v;
    }
  }
}

// ------------------------------------------------------------ phase store
__global__ void __launch_bounds__(256) k_phase_store(PhaseArgs a) {
  const int row = blockIdx.x;
  const int n = blockIdx.y * blockDim.x + threadIdx.x;
  if (n >= (a.row_N ? a.row_N[row] : a.N)) return;
  const float eps = amp_eps(a.rule, a.rowstat[row]);
  const float2 v = a.row_in ? a.in[a.row_in[row] + n] : a.in[(int64_t)row * a.ldin + n];
  const float2 p = cscale(v, amp_factor(a.rule, v.x * v.x + v.y * v.y, eps));
  if (a.fmt == SPEC_I16)   // |p| <= 1: fixed scale 1/32767
    reinterpret_cast<short2*>(a.out)[(int64_t)row * a.ldo + n] = make_short2(i16_quant(p.x, kI16Max),
                                                                              i16_quant(p.y, kI16Max));
  else if (a.fmt == SPEC_F16) reinterpret_cast<__half2*>(a.out)[(int64_t)row * a.ldo + n] = __float22half2_rn(p);
  else reinterpret_cast<float2*>(a.out)[(int64_t)row * a.ldo + n] = p;
}

// ------------------------------------------------------------ int16 rows
// One cluster of kQCluster blocks per row: each block takes a segment, the
// blocks exchange their segment maxima through distributed shared memory
// (hardware cluster barriers), and each writes its segment of the block-scaled
// int16 row; block 0 writes the header.  The row maximum does not depend on the
// split, so the row is the same as one block would write.
constexpr int kQCluster = 8;

__global__ void __cluster_dims__(kQCluster, 1, 1) __launch_bounds__(256)
    k_quantize_i16(const float2* __restrict__ in, int64_t ldin, int n, char* __restrict__ out, int64_t ldo_bytes) {
  __shared__ float scratch[32];
  __shared__ float seg_max;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int seg = (n + kQCluster - 1) / kQCluster;
  const int k0 = rank * seg, k1 = min(n, k0 + seg);
  const float2* r = in + (int64_t)blockIdx.y * ldin;
  float m = 0.0f;
  for (int k = k0 + threadIdx.x; k < k1; k += 256) m = fmaxf(m, fmaxf(fabsf(r[k].x), fabsf(r[k].y)));
  m = block_max(m, scratch);
  if (threadIdx.x == 0) seg_max = m;
  cluster.sync();
  if (threadIdx.x < 32) {
    float v = (threadIdx.x < kQCluster) ? *cluster.map_shared_rank(&seg_max, (unsigned)threadIdx.x) : 0.0f;
    v = warp_max(v);
    if (threadIdx.x == 0) scratch[0] = v;
  }
  cluster.sync();   // every block has read the others' maxima before any exits
  m = scratch[0];
  const float inv = (m > 0.0f) ? kI16Max / m : 0.0f;
  char* row = out + (int64_t)blockIdx.y * ldo_bytes;
  if (rank == 0 && threadIdx.x < 4) reinterpret_cast<float*>(row)[threadIdx.x] = (threadIdx.x == 0) ? m / kI16Max : 0.0f;
  short2* o = reinterpret_cast<short2*>(row + kI16Header);
  for (int k = k0 + threadIdx.x; k < k1; k += 256) o[k] = make_short2(i16_quant(r[k].x, inv), i16_quant(r[k].y, inv));
}

// ------------------------------------------------------------ generic passes
template <int R, int DIR, bool REAL_IN>
__global__ void __launch_bounds__(256) k_gpass(const void* __restrict__ in, int64_t ldr, float2* __restrict__ out,
                                               int64_t ld, int n, int Ns, int nrows,
                                               const float2* __restrict__ tw) {
  const int m = n / R;
  const int64_t total = (int64_t)m * nrows;
  const int tstride = n / (Ns * R);
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(g / m);
    const int j = (int)(g - (int64_t)row * m);
    float2 v[R];
    if constexpr (REAL_IN) {
      const float* x = reinterpret_cast<const float*>(in) + (int64_t)row * ldr;
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = make_float2(__ldg(x + j + r * m), 0.0f);
    } else {
      const float2* x = reinterpret_cast<const float2*>(in) + (int64_t)row * ld;
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = x[j + r * m];
    }
    const int k = j % Ns;
    if (k != 0) {
      float2 w1 = __ldg(tw + k * tstride);
      if (DIR > 0) w1.y = -w1.y;
      float2 w = w1;
#pragma unroll
      for (int r = 1; r < R; r++) {
        v[r] = cmul(v[r], w);
        if (r + 1 < R) w = cmul(w, w1);
      }
    }
    dft<R, DIR>(v);
    float2* o = out + (int64_t)row * ld + (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) o[r * Ns] = v[dft_perm<R>(r)];
  }
}

__global__ void k_analytic_mask(float2* a, int64_t ld, int n, int nrows) {
  const int row = blockIdx.x;
  const float d = 1.0f / (float)n;
  const int half = (n + 1) >> 1;
  for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < n; k += gridDim.y * blockDim.x) {
    float f;
    if (k == 0) f = d;
    else if (k < half) f = 2.0f * d;
    else if (!(n & 1) && k == (n >> 1)) f = d;
    else f = 0.0f;
    float2* p = a + (int64_t)row * ld + k;
    *p = cscale(*p, f);
  }
}

__global__ void __launch_bounds__(256) k_rowstats(const float2* a, int64_t ld, int n, float* rmax, float* rsum) {
  __shared__ float sm[32], ss[32];
  const float2* r = a + (int64_t)blockIdx.x * ld;
  float mx = 0.0f, sum = 0.0f;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const float2 v = r[k];
    const float m2 = v.x * v.x + v.y * v.y;
    mx = fmaxf(mx, m2);
    sum += m2;
  }
  mx = warp_max(mx);
  sum = warp_sum(sum);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sm[w] = mx; ss[w] = sum; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    mx = (l < nw) ? sm[l] : 0.0f;
    sum = (l < nw) ? ss[l] : 0.0f;
    mx = warp_max(mx);
    sum = warp_sum(sum);
    if (l == 0) {
      if (rmax) rmax[blockIdx.x] = mx;
      if (rsum) rsum[blockIdx.x] = sum;
    }
  }
}

// ------------------------------------------------------------ Bluestein helpers
// chirp c[n] = exp(dir * pi * i * n^2 / N) with n^2 reduced mod 2N exactly.
__device__ __forceinline__ float2 chirp(int64_t n, int N, int dir) {
  const int64_t r = (n * n) % (2 * (int64_t)N);
  double s, c;
  sincospi((double)dir * (double)r / (double)N, &s, &c);
  return make_float2((float)c, (float)s);
}

// a[j] = in[j] * c_dir[j] (j < N), 0 for N <= j < M.  in: real (real_in) or complex rows,
// optionally multiplied first by the analytic mask (mask_n = N) with its 1/N.
__global__ void k_blue_pre(const void* __restrict__ in, bool real_in, int64_t ldin, float2* __restrict__ a,
                           int64_t lda, int N, int M, int dir, int mask) {
  const int row = blockIdx.y;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (j < N) {
      if (real_in) v = make_float2(reinterpret_cast<const float*>(in)[(int64_t)row * ldin + j], 0.f);
      else v = reinterpret_cast<const float2*>(in)[(int64_t)row * ldin + j];
      if (mask) {
        const float d = 1.0f / (float)N;
        const int half = (N + 1) >> 1;
        float f;
        if (j == 0) f = d;
        else if (j < half) f = 2.0f * d;
        else if (!(N & 1) && j == (N >> 1)) f = d;
        else f = 0.0f;
        v = cscale(v, f);
      }
      v = cmul(v, chirp(j, N, dir));
    }
    a[(int64_t)row * lda + j] = v;
  }
}

// a[k] *= B[k] (one filter spectrum for all rows)
__global__ void k_blue_mul(float2* __restrict__ a, int64_t lda, const float2* __restrict__ B, int M) {
  const int row = blockIdx.y;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < M; k += gridDim.x * blockDim.x)
    a[(int64_t)row * lda + k] = cmul(a[(int64_t)row * lda + k], B[k]);
}

// out[k] = c_dir[k] * a[k] / M, k < N
__global__ void k_blue_post(const float2* __restrict__ a, int64_t lda, float2* __restrict__ out, int64_t ldo, int N,
                            int M, int dir) {
  const int row = blockIdx.y;
  const float inv = 1.0f / (float)M;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x)
    out[(int64_t)row * ldo + k] = cscale(cmul(a[(int64_t)row * lda + k], chirp(k, N, dir)), inv);
}

// filter b[j] = conj-chirp for |j| < N, placed circularly in M points
__global__ void k_blue_filter(float2* __restrict__ b, int N, int M, int dir) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (j < N) v = chirp(j, N, -dir);
    else if (j > M - N) v = chirp(M - j, N, -dir);
    b[j] = v;
  }
}

template <typename K>
cudaError_t launch_k(K kern, int grid, int T, size_t smem, cudaStream_t st, const void* args) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void* argv[] = {const_cast<void*>(args)};
  return cudaLaunchKernel((const void*)kern, dim3(grid), dim3(T), argv, smem, st);
}

}  // namespace

// ---------------------------------------------------------------- host side
bool spec_supported(int Nz) { return on_menu(Nz); }
bool pair_supported(int Nz) { return (Nz % 2 == 0) && on_menu(Nz / 2); }

size_t spec_smem_bytes(int Nz) {
  return ((size_t)padded_len(Nz) + 128 + tw_hi_len(Nz)) * sizeof(float2);
}

size_t pair_smem_bytes(int Nz) {
  const int h = Nz / 2;
  const size_t bufs = pair_pingpong(h) ? 2 : 1;
  return (bufs * padded_len(h) + 128 + tw_hi_len(h) + 128 + tw_hi_len(Nz)) * sizeof(float2);
}

cudaError_t launch_spec(const SpecArgs& a, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  const size_t smem = spec_smem_bytes(a.Nz);
  switch (a.Nz) {
#define FPCC_SPEC_CASE(SZ, T, ...) \
  case SZ: return launch_k(k_spec<T, Radices<__VA_ARGS__>>, a.nrows, T, smem, st, &a);
    FPCC_SIZE_MENU(FPCC_SPEC_CASE)
#undef FPCC_SPEC_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_cwt_rows(const CwtRowArgs& a, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  if (a.L > a.M) return cudaErrorInvalidValue;
  const size_t smem = spec_smem_bytes(a.M);
  switch (a.M) {
#define FPCC_CWT_CASE(SZ, T, ...) \
  case SZ: return launch_k(k_cwt_rows<T, Radices<__VA_ARGS__>>, a.nrows, T, smem, st, &a);
    FPCC_SIZE_MENU(FPCC_CWT_CASE)
#undef FPCC_CWT_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <int FMT, bool HERM>
static cudaError_t launch_pairs_t(const PairArgs& a, cudaStream_t st) {
  const size_t smem = pair_smem_bytes(a.Nz);
  switch (a.Nz / 2) {
#define FPCC_PAIR_CASE(SZ, T, ...)                                                                   \
  case SZ:                                                                                         \
    return launch_k(k_pairs<pair_threads(SZ), Radices<__VA_ARGS__>, FMT, HERM>, a.npairs, pair_threads(SZ), \
                    smem, st, &a);
    FPCC_SIZE_MENU(FPCC_PAIR_CASE)
#undef FPCC_PAIR_CASE
    default: return cudaErrorInvalidValue;
  }
}

// Pair-kernel form per padded length: the tiled kernel where it exists, unless
// set otherwise (autotuner, fpcc_pair_form).  Lengths are few; a fixed table
// with atomic entries is enough.
namespace {
constexpr int kFormSlots = 64;
std::atomic<int> g_form_nz[kFormSlots];
std::atomic<int> g_form_val[kFormSlots];
}  // namespace

int pair_form_get(int Nz) {
  for (int i = 0; i < kFormSlots; i++) {
    const int n = g_form_nz[i].load(std::memory_order_acquire);
    if (n == 0) break;
    if (n == Nz) return g_form_val[i].load(std::memory_order_relaxed);
  }
  return pair_tiled_supported(Nz) ? PAIR_FORM_TILED : PAIR_FORM_BLOCK;
}

int pair_form_set(int Nz, int form) {
  if (form != PAIR_FORM_BLOCK && form != PAIR_FORM_TILED) return -1;
  if (form == PAIR_FORM_TILED && !pair_tiled_supported(Nz)) return -1;
  if (form == PAIR_FORM_BLOCK && !pair_supported(Nz)) return -1;
  for (int i = 0; i < kFormSlots; i++) {
    int n = g_form_nz[i].load(std::memory_order_acquire);
    if (n == 0) {
      g_form_val[i].store(form, std::memory_order_relaxed);
      int expect = 0;
      if (g_form_nz[i].compare_exchange_strong(expect, Nz, std::memory_order_acq_rel)) return 0;
      n = expect;
    }
    if (n == Nz) {
      g_form_val[i].store(form, std::memory_order_relaxed);
      return 0;
    }
  }
  return -1;
}

cudaError_t launch_pairs(const PairArgs& a, cudaStream_t st) {
  if (a.npairs <= 0) return cudaSuccess;
  if (pair_tiled_supported(a.Nz) && pair_form_get(a.Nz) == PAIR_FORM_TILED) return launch_pairs_tiled(a, st);
  if (!pair_supported(a.Nz)) return cudaErrorInvalidValue;
  const bool herm = (a.norm != 0);
  if (a.fmt == SPEC_I16) return herm ? cudaErrorInvalidValue : launch_pairs_t<SPEC_I16, false>(a, st);
  if (a.fmt == SPEC_F16) return herm ? launch_pairs_t<SPEC_F16, true>(a, st) : launch_pairs_t<SPEC_F16, false>(a, st);
  return herm ? launch_pairs_t<SPEC_F32, true>(a, st) : launch_pairs_t<SPEC_F32, false>(a, st);
}

cudaError_t launch_quantize_i16(const float2* in, int64_t ldin, int n, int nrows, void* out, int64_t ldo,
                                cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  for (int r0 = 0; r0 < nrows; r0 += 65535) {
    const int nr = nrows - r0 < 65535 ? nrows - r0 : 65535;
    k_quantize_i16<<<dim3(kQCluster, nr), 256, 0, st>>>(in + (int64_t)r0 * ldin, ldin, n,
                                                        reinterpret_cast<char*>(out) + (int64_t)r0 * ldo * 4, ldo * 4);
  }
  return cudaGetLastError();
}

cudaError_t launch_phase_store(const PhaseArgs& a, cudaStream_t st) {
  if (a.nrows <= 0) return cudaSuccess;
  if ((a.N + 255) / 256 > 65535) return cudaErrorInvalidValue;
  dim3 grid(a.nrows, (a.N + 255) / 256);
  k_phase_store<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

static int grid_for(int64_t work) {
  int64_t b = (work + 255) / 256;
  const int64_t cap = 152 * 16;   // a few waves of 256-thread blocks on 152 SMs
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

cudaError_t launch_gpass(int R, int dir, const void* in, bool real_in, int64_t ldr, float2* out, int64_t ld, int n,
                         int Ns, int nrows, const float2* tw, cudaStream_t st) {
  const int grid = grid_for((int64_t)(n / R) * nrows);
#define FPCC_GP(RR)                                                                                   \
  if (R == RR) {                                                                                      \
    if (real_in) {                                                                                    \
      if (dir < 0) k_gpass<RR, -1, true><<<grid, 256, 0, st>>>(in, ldr, out, ld, n, Ns, nrows, tw);  \
      else k_gpass<RR, 1, true><<<grid, 256, 0, st>>>(in, ldr, out, ld, n, Ns, nrows, tw);           \
    } else {                                                                                          \
      if (dir < 0) k_gpass<RR, -1, false><<<grid, 256, 0, st>>>(in, ldr, out, ld, n, Ns, nrows, tw); \
      else k_gpass<RR, 1, false><<<grid, 256, 0, st>>>(in, ldr, out, ld, n, Ns, nrows, tw);          \
    }                                                                                                 \
    return cudaGetLastError();                                                                        \
  }
  FPCC_GP(16)
  FPCC_GP(8)
  FPCC_GP(5)
  FPCC_GP(4)
  FPCC_GP(3)
  FPCC_GP(2)
#undef FPCC_GP
  return cudaErrorInvalidValue;
}

cudaError_t launch_analytic_mask(float2* a, int64_t ld, int n, int nrows, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  dim3 grid(nrows, (n + 255) / 256 < 64 ? (n + 255) / 256 : 64);
  k_analytic_mask<<<grid, 256, 0, st>>>(a, ld, n, nrows);
  return cudaGetLastError();
}

cudaError_t launch_rowstats(const float2* a, int64_t ld, int n, int nrows, float* rmax, float* rsum,
                            cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  k_rowstats<<<nrows, 256, 0, st>>>(a, ld, n, rmax, rsum);
  return cudaGetLastError();
}

}  // namespace fpcc

namespace fpcc {

static dim3 rows_grid(int n, int nrows) {
  int gx = (n + 255) / 256;
  if (gx > 256) gx = 256;
  return dim3(gx, nrows);
}

cudaError_t launch_blue_pre(const void* in, bool real_in, int64_t ldin, float2* a, int64_t lda, int N, int M,
                            int dir, int mask, int nrows, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_blue_pre<<<rows_grid(M, nrows), 256, 0, st>>>(in, real_in, ldin, a, lda, N, M, dir, mask);
  return cudaGetLastError();
}

cudaError_t launch_blue_mul(float2* a, int64_t lda, const float2* B, int M, int nrows, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_blue_mul<<<rows_grid(M, nrows), 256, 0, st>>>(a, lda, B, M);
  return cudaGetLastError();
}

cudaError_t launch_blue_post(const float2* a, int64_t lda, float2* out, int64_t ldo, int N, int M, int dir,
                             int nrows, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  if (nrows > 65535) return cudaErrorInvalidValue;
  k_blue_post<<<rows_grid(N, nrows), 256, 0, st>>>(a, lda, out, ldo, N, M, dir);
  return cudaGetLastError();
}

cudaError_t launch_blue_filter(float2* b, int N, int M, int dir, cudaStream_t st) {
  k_blue_filter<<<(M + 255) / 256 < 1024 ? (M + 255) / 256 : 1024, 256, 0, st>>>(b, N, M, dir);
  return cudaGetLastError();
}

}  // namespace fpcc
