// C ABI of the correlation engine: contexts, device-resident stages and the
// host-buffer entry points (batched and plain per-window drop-ins).
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <semaphore.h>
#include <cmath>
#include <string>
#include <algorithm>
#include <vector>
#include <type_traits>

#include "../../include/fastpcc_gb300.h"
#include "direct.cuh"
#include "engine.h"
#include "kernels.cuh"
#include "jit.h"
#include "large.cuh"
#include "menu.cuh"
#include "wavelet.h"
#include "wpcc.h"
#include "precise.cuh"
#include "multi.cuh"
#include "stack.cuh"

using namespace fpcc;

namespace {

thread_local std::string g_err;
std::atomic<int64_t> g_launches{0};

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(FPCC_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);       \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
};

}  // namespace

struct fpcc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool own_pool = true;             // false: the pool belongs to a server sharing it
  DevBuf dev[56];
  DevBuf pin[8];
  cudaStream_t stream2 = nullptr;   // second stream of the pipelined drop-ins
  cudaEvent_t chunk_ev[16] = {};    // pair-stage chunks whose results stream2 downloads
  cudaEvent_t up_ev[4] = {};        // station-row chunks that stream2 has uploaded
  cudaStream_t stream3 = nullptr;   // downloads of the first-use pipeline (uploads run on stream2)
  std::vector<cudaEvent_t> pipe_ev; // events of the first-use pipeline
  // the context's device buffers and caches come from a pool of its own, allocated
  // and freed in the order of `stream` (no device synchronisation when a buffer
  // grows); ord_ev orders them against the second stream when it exists
  cudaMemPool_t pool = nullptr;
  cudaEvent_t ord_ev = nullptr;
  std::map<int, float2*> twiddles;   // device tables exp(-2 pi i t/n), per n
  std::map<int, float2*> bluestein;  // per window length N: M-point filter spectra, forward then inverse
  std::map<int, double2*> twiddles64;   // FP64 tables exp(-2 pi i t/n)
  std::map<int, float4*> twiddles_df;   // double-float tables exp(-2 pi i t/n)
  // filter spectra of the packed path per (N, M, fp64): forward then inverse, M values each,
  // held in blocks of one batched computation
  std::map<std::tuple<int, int, int>, void*> multi_filters;
  std::vector<void*> multi_blocks;
  size_t multi_filter_bytes = 0;
  int precision = FPCC_ANALYTIC_AUTO;   // when analytic signals are computed in FP64
  std::mutex mu;
};

namespace {

// Stream-ordered allocation from the context's pool; when the second stream
// exists it waits for the allocation before it can touch the memory.
cudaError_t ctx_alloc(fpcc_ctx* c, void** p, size_t bytes) {
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return e;
  }
  if (c->stream2) {
    cudaEventRecord(c->ord_ev, c->stream);
    cudaStreamWaitEvent(c->stream2, c->ord_ev, 0);
  }
  return cudaSuccess;
}

// Stream-ordered free: after the work queued on `stream` (and on the second
// stream, when it exists) that may still read the memory.
void ctx_free(fpcc_ctx* c, void* p) {
  if (!p) return;
  if (c->stream2) {
    cudaEventRecord(c->ord_ev, c->stream2);
    cudaStreamWaitEvent(c->stream, c->ord_ev, 0);
  }
  cudaFreeAsync(p, c->stream);
}

int dev_buf(fpcc_ctx* c, int slot, size_t bytes, void** out) {
  DevBuf& b = c->dev[slot];
  if (b.n < bytes) {
    // a buffer that has to grow grows by half again at least, so that a run of
    // slowly increasing sizes (windows sorted by length) reallocates rarely
    const size_t nb = b.p ? std::max(bytes, b.n + b.n / 2) : bytes;
    ctx_free(c, b.p);
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = ctx_alloc(c, &b.p, nb);
    if (e != cudaSuccess && nb > bytes) {
      e = ctx_alloc(c, &b.p, bytes);
      if (e == cudaSuccess) b.n = bytes;
    } else if (e == cudaSuccess) {
      b.n = nb;
    }
    if (e != cudaSuccess) return fail(FPCC_ENOMEM, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
  }
  *out = b.p;
  return 0;
}

int pin_buf(fpcc_ctx* c, int slot, size_t bytes, void** out) {
  DevBuf& b = c->pin[slot];
  if (b.n < bytes) {
    if (b.p) {
      cudaStreamSynchronize(c->stream);
      cudaFreeHost(b.p);
    }
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = cudaMallocHost(&b.p, bytes);
    if (e != cudaSuccess) return fail(FPCC_ENOMEM, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    b.n = bytes;
  }
  *out = b.p;
  return 0;
}

void lag_window(int Lag1, int Lag2, int* lag0, int* L) {
  if (Lag2 >= Lag1) { *lag0 = Lag1; *L = Lag2 - Lag1 + 1; }
  else { *lag0 = Lag2; *L = Lag1 - Lag2 + 1; }
}

bool is_fft_method(int m) { return m == FPCC_PCC2 || m == FPCC_GNCC || m == FPCC_CC1B; }

int check_lags(int N, int Lag1, int Lag2) {
  if (N <= 0) return fail(FPCC_EARG, "N must be positive");
  if (abs(Lag1) >= N || abs(Lag2) >= N)
    return fail(FPCC_EARG, "|lag| must be below N (Lag1=%d Lag2=%d N=%d)", Lag1, Lag2, N);
  return 0;
}

fpcc_ctx* g_default = nullptr;
std::mutex g_default_mu;

int default_ctx(fpcc_ctx** out) {
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default) {
    int dev = 0;
    cudaGetDevice(&dev);
    int rc = fpcc_create(&g_default, dev);
    if (rc) return rc;
  }
  *out = g_default;
  return 0;
}

}  // namespace

// ============================================================== context
extern "C" int fpcc_create(fpcc_ctx** out, int device) {
  if (!out) return fail(FPCC_EARG, "null output pointer");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(FPCC_ECUDA, "no CUDA device available");
  if (device < 0 || device >= ndev) return fail(FPCC_EARG, "device %d out of range", device);
  CK(cudaSetDevice(device));
  fpcc_ctx* c = new fpcc_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  c->own_stream = true;
  cudaMemPoolProps pp = {};
  pp.allocType = cudaMemAllocationTypePinned;
  pp.location.type = cudaMemLocationTypeDevice;
  pp.location.id = device;
  uint64_t keep = UINT64_MAX;   // freed blocks stay mapped for the context's later buffers
  if ((e = cudaMemPoolCreate(&c->pool, &pp)) != cudaSuccess ||
      (e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ord_ev, cudaEventDisableTiming)) != cudaSuccess) {
    if (c->pool) cudaMemPoolDestroy(c->pool);
    cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(e, "memory pool");
  }
  *out = c;
  return 0;
}

namespace fpcc {
// The calling thread's message for fpcc_last_error (a server hands its worker's
// message to the thread that collects a failed request).
void set_last_error(const char* msg) { g_err = msg ? msg : ""; }

// For a server: a context made by fpcc_create and not used yet gives up its own
// pool and allocates from the server's.
int ctx_share_pool(fpcc_ctx* c, cudaMemPool_t pool) {
  if (c->own_pool) cudaMemPoolDestroy(c->pool);
  c->pool = pool;
  c->own_pool = false;
  return 0;
}
}  // namespace fpcc

extern "C" int fpcc_destroy(fpcc_ctx* c) {
  if (!c) return 0;
  cudaSetDevice(c->device);
  for (auto& b : c->dev) ctx_free(c, b.p);
  for (auto& kv : c->twiddles) ctx_free(c, kv.second);
  for (auto& kv : c->bluestein) ctx_free(c, kv.second);
  for (auto& kv : c->twiddles64) ctx_free(c, kv.second);
  for (auto& kv : c->twiddles_df) ctx_free(c, kv.second);
  for (void* b : c->multi_blocks) ctx_free(c, b);
  cudaStreamSynchronize(c->stream);
  if (c->stream2) cudaStreamSynchronize(c->stream2);
  for (auto& b : c->pin) if (b.p) cudaFreeHost(b.p);
  if (c->own_pool) cudaMemPoolDestroy(c->pool);
  cudaEventDestroy(c->ord_ev);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  for (cudaEvent_t e : c->chunk_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->up_ev)
    if (e) cudaEventDestroy(e);
  if (c->stream3) {
    cudaStreamSynchronize(c->stream3);
    cudaStreamDestroy(c->stream3);
  }
  for (cudaEvent_t e : c->pipe_ev) cudaEventDestroy(e);
  {
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (c == g_default) g_default = nullptr;
  }
  delete c;
  return 0;
}

extern "C" int fpcc_set_analytic_precision(fpcc_ctx* c, int mode) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (mode < FPCC_ANALYTIC_F32 || mode > FPCC_ANALYTIC_F64) return fail(FPCC_EARG, "unknown precision mode %d", mode);
  c->precision = mode;
  return 0;
}

extern "C" int fpcc_set_stream(fpcc_ctx* c, void* stream) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (stream == nullptr) {
    if (!c->own_stream) {
      CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
      c->own_stream = true;
    }
    return 0;
  }
  // the context's buffers were allocated and freed in the old stream's order
  cudaStreamSynchronize(c->stream);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return 0;
}

extern "C" void* fpcc_get_stream(fpcc_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int fpcc_sync(fpcc_ctx* c) {
  if (!c) return fail(FPCC_EARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" const char* fpcc_last_error(void) { return g_err.c_str(); }
extern "C" const char* fpcc_version(void) { return "fastpcc_gb300 0.1 (sm_103a)"; }
extern "C" int64_t fpcc_launch_count(void) { return g_launches.load(); }

// ============================================================== planning
extern "C" int fpcc_choose_nz(int N, int Lag1, int Lag2, int mode) {
  const int M = abs(Lag1) > abs(Lag2) ? abs(Lag1) : abs(Lag2);
  return choose_nz(N, M, mode);
}

extern "C" int fpcc_max_block_len(void) { return kMenu[kMenuLen - 1]; }

extern "C" int fpcc_pair_form(int Nz, int form) {
  if (form > 0 && pair_form_set(Nz, form) != 0) return FPCC_EUNSUP;
  if (!pair_supported(Nz) && !pair_tiled_supported(Nz)) return FPCC_EUNSUP;
  return pair_form_get(Nz);
}

extern "C" int64_t fpcc_station_row_bytes(int method, int N, int Nz, int fmt) {
  switch (method) {
    case FPCC_PCC2: return fmt == FPCC_I16 ? 16 + 4 * (int64_t)Nz : (int64_t)Nz * (fmt == FPCC_F16 ? 4 : 8);
    case FPCC_PCC1:
    case FPCC_PCCV: return (int64_t)N * (fmt == FPCC_F32 ? 8 : 4);
    case FPCC_GNCC:
    case FPCC_CC1B: return ((int64_t)Nz / 2 + 1) * 8;
    case FPCC_CC1B_POPCOUNT: return ((int64_t)N + 31) / 32 * 4;
    default: return -1;
  }
}

extern "C" int64_t fpcc_station_row_elems(int method, int N, int Nz) {
  switch (method) {
    case FPCC_PCC2: return Nz;
    case FPCC_PCC1:
    case FPCC_PCCV: return N;
    case FPCC_GNCC:
    case FPCC_CC1B: return Nz / 2 + 1;
    case FPCC_CC1B_POPCOUNT: return (N + 31) / 32;
    default: return -1;
  }
}

// ============================================================== device stages
namespace {

// Workspace slots of the context.
enum Slot { S_HOST_X = 0, S_STATION = 1, S_ENERGY = 2, S_PAIRS2 = 3, S_Y = 4, S_PAIRS = 5, S_ANA_A = 6,
            S_ANA_B = 7, S_RSTAT = 8, S_LARGE_T = 9, S_WP_X = 10, S_WP_BAND = 11, S_WP_RMAX = 12,
            S_WP_Y = 13, S_WP_STAGE = 14, S_BLUE_O = 23, S_P64_D = 24, S_P64_A = 25, S_P64_B = 26,
            S_P64_CNT = 27, S_I16_Q = 28, S_MULTI_A = 29, S_MULTI_B = 30, S_MULTI_AN = 31, S_EPART = 32,
            S_CONV_X = 33, S_CONV_Y = 34, S_STK_SPEC = 35, S_STK_A = 36, S_STK_B = 37, S_STK_X = 38,
            S_STK_T = 39, S_STK_T2 = 40, S_STK_Y = 41, S_STK_Y2 = 42, S_STK_R = 43, S_STK_AN = 44,
            S_HK_TAB = 45, S_PIPE_CNT = 46, S_GATHER_X = 47, S_GATHER_O = 48, S_GATHER_I = 49 };

constexpr size_t kLargeChunkBytes = size_t(512) << 20;   // four-step intermediate per chunk

// Station products of a length above the in-block menu: four-step forward DFT
// of each zero-padded row, in chunks of rows whose intermediate stays small.
int large_station(fpcc_ctx* c, int cmode, const void* in, size_t in_esz, int64_t ldin, int nrows, int N, int Nz,
                  int rule, const float* rowstat, int sign_ge, int fmt, int half, void* out, int64_t ldo) {
  int n1, n2;
  if (!large_supported(Nz, &n1, &n2)) return fail(FPCC_EUNSUP, "Nz=%d is not a supported transform length", Nz);
  int64_t chunk = (int64_t)(kLargeChunkBytes / ((size_t)Nz * sizeof(float2)));
  if (chunk < 1) chunk = 1;
  if (chunk > 65535) chunk = 65535;
  if (chunk > nrows) chunk = nrows;
  void* T = nullptr;
  int rc = dev_buf(c, S_LARGE_T, (size_t)chunk * Nz * sizeof(float2), &T);
  if (rc) return rc;
  // int16 rows: F32 spectra of the chunk first, then the block-scaled rows
  void* Q = nullptr;
  if (fmt == FPCC_I16 && (rc = dev_buf(c, S_I16_Q, (size_t)chunk * Nz * sizeof(float2), &Q))) return rc;
  const size_t out_esz = (fmt == FPCC_F32) ? 8 : 4;
  for (int r0 = 0; r0 < nrows; r0 += (int)chunk) {
    LargeArgs a{};
    a.n = Nz; a.n1 = n1; a.n2 = n2; a.dir = -1;
    a.nrows = (int)((nrows - r0) < chunk ? (nrows - r0) : chunk);
    a.cmode = cmode;
    a.in = (const char*)in + (size_t)r0 * ldin * in_esz;
    a.ldin = ldin; a.N = N; a.in_off = 0; a.rule = rule;
    a.rowstat = rowstat ? rowstat + r0 : nullptr;
    a.sign_ge = sign_ge; a.in_scale = 1.0f;
    a.T = (float2*)T;
    a.rmode = ROW_SPEC;
    if (fmt == FPCC_I16) {
      a.out = Q; a.ldo = Nz; a.out_fmt = FPCC_F32; a.out_half = half;
    } else {
      a.out = (char*)out + (size_t)r0 * ldo * out_esz;
      a.ldo = ldo; a.out_fmt = fmt; a.out_half = half;
    }
    CK(launch_large(a, c->stream));
    g_launches += 2;
    if (fmt == FPCC_I16) {
      CK(launch_quantize_i16((const float2*)Q, Nz, half ? Nz / 2 + 1 : Nz, a.nrows, (char*)out + (size_t)r0 * ldo * 4,
                             ldo, c->stream));
      g_launches++;
    }
  }
  return 0;
}

// Pair stage for Nz/2 above the in-block menu: four-step inverse transform of the
// packed Hermitian cross-spectrum, lags written from the row pass.
int large_pairs(fpcc_ctx* c, const PairArgs& q, int herm) {
  const int h = q.Nz / 2;
  int n1, n2;
  if (!large_supported(h, &n1, &n2)) return fail(FPCC_EUNSUP, "Nz=%d is not a supported correlation length", q.Nz);
  int64_t chunk = (int64_t)(kLargeChunkBytes / ((size_t)h * sizeof(float2)));
  if (chunk < 1) chunk = 1;
  if (chunk > 65535) chunk = 65535;
  if (chunk > q.npairs) chunk = q.npairs;
  void* T = nullptr;
  int rc = dev_buf(c, S_LARGE_T, (size_t)chunk * h * sizeof(float2), &T);
  if (rc) return rc;
  for (int p0 = 0; p0 < q.npairs; p0 += (int)chunk) {
    LargeArgs a{};
    a.n = h; a.n1 = n1; a.n2 = n2; a.dir = +1;
    a.nrows = (int)((q.npairs - p0) < chunk ? (q.npairs - p0) : chunk);
    a.cmode = COL_PAIR;
    a.spec = q.spec; a.ldspec = q.ldspec; a.fmt = q.fmt; a.herm = herm;
    if (q.desc) a.desc = q.desc + p0;
    else a.pairs = q.pairs + p0;
    a.Nz = q.Nz;
    a.T = (float2*)T;
    a.rmode = ROW_LAGS;
    a.lag0 = q.lag0; a.L = q.L; a.scale = q.scale; a.norm = q.norm;
    a.energy = q.energy; a.ldE = q.ldE; a.N = q.N;
    if (!q.desc) { a.y = q.y + (size_t)p0 * q.ldy; a.ldy = q.ldy; }
    CK(launch_large(a, c->stream));
    g_launches += 2;
  }
  return 0;
}

// Rows of 4-byte words: dst row didx[r] (r without didx) = src row sidx[r]
// (r without sidx), `words` words each; strides in words.
__global__ void k_rows_copy(const uint32_t* __restrict__ src, int64_t lds, const int* __restrict__ sidx,
                            uint32_t* __restrict__ dst, int64_t ldd, const int* __restrict__ didx, int64_t words) {
  const int r = blockIdx.y;
  const int64_t sr = sidx ? sidx[r] : r, dr = didx ? didx[r] : r;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < words; i += (int64_t)gridDim.x * blockDim.x)
    dst[dr * ldd + i] = src[sr * lds + i];
}

cudaError_t launch_rows_copy(const void* src, int64_t lds, const int* sidx, void* dst, int64_t ldd, const int* didx,
                             int nrows, int64_t words, cudaStream_t st) {
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(32, (words + 255) / 256));
  for (int r0 = 0; r0 < nrows; r0 += 65535) {
    const int n = std::min(65535, nrows - r0);
    k_rows_copy<<<dim3(gx, n), 256, 0, st>>>((const uint32_t*)src + (sidx ? 0 : r0 * lds), lds, sidx ? sidx + r0 : nullptr,
                                             (uint32_t*)dst + (didx ? 0 : r0 * ldd), ldd, didx ? didx + r0 : nullptr,
                                             words);
  }
  return cudaGetLastError();
}

// Twiddle table exp(-2 pi i t / n), t < n, computed on the device in FP64
// (sincospi of the exact fraction -2t/n) and stored as float2 or double2, in
// the context's stream order (no host loop, no synchronous upload).
__global__ void k_twiddles(float2* f, double2* d, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double sn, cs;
    sincospi(-2.0 * (double)t / (double)n, &sn, &cs);
    if (f) f[t] = make_float2((float)cs, (float)sn);
    if (d) d[t] = make_double2(cs, sn);
  }
}

cudaError_t launch_twiddles(float2* f, double2* d, int n, cudaStream_t st) {
  const int g = (int)std::min<int64_t>(1024, ((int64_t)n + 255) / 256);
  k_twiddles<<<g > 0 ? g : 1, 256, 0, st>>>(f, d, n);
  return cudaGetLastError();
}

int twiddle_table(fpcc_ctx* c, int n, const float2** out) {
  auto it = c->twiddles.find(n);
  if (it != c->twiddles.end()) { *out = it->second; return 0; }
  float2* d = nullptr;
  cudaError_t e = ctx_alloc(c, (void**)&d, (size_t)n * sizeof(float2));
  if (e != cudaSuccess) return fail(FPCC_ENOMEM, "twiddle table: %s", cudaGetErrorString(e));
  if ((e = launch_twiddles(d, nullptr, n, c->stream)) != cudaSuccess) {
    ctx_free(c, d);
    return cuda_fail(e, "twiddle table");
  }
  g_launches++;
  c->twiddles[n] = d;
  *out = d;
  return 0;
}

// Generic passes of one M-point transform over rows (ping-pong between A and B,
// starting from A); returns the buffer that holds the result.
int passes(fpcc_ctx* c, float2* A, float2* B, int M, int nrows, int dir, float2** result) {
  FftPlan p;
  if (!make_plan(M, &p)) return fail(FPCC_EUNSUP, "length %d is not 2,3,5-smooth", M);
  const float2* tw = nullptr;
  int rc = twiddle_table(c, M, &tw);
  if (rc) return rc;
  float2* bufs[2] = {A, B};
  int cur = 0, Ns = 1;
  for (int i = 0; i < p.npass; i++) {
    CK(launch_gpass(p.rad[i], dir, bufs[cur], false, M, bufs[cur ^ 1], M, M, Ns, nrows, tw, c->stream));
    g_launches++;
    cur ^= 1;
    Ns *= p.rad[i];
  }
  *result = bufs[cur];
  return 0;
}

// Transform length of Bluestein's method for windows of n/2 samples: the
// cheapest length >= n (by the pass cost model) that the generic passes run
// (2,3,5-smooth within the pass limit), searched up to 2n.
int smooth_at_least(int n) {
  static std::mutex mu;
  static std::map<int, int> memo;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = memo.find(n);
    if (it != memo.end()) return it->second;
  }
  int best = -1;
  double bc = 1e300;
  for (int m : smooth235_in(n, 2 * n + 64)) {
    FftPlan p;
    if (!make_plan(m, &p)) continue;
    const double c = plan_cost(m);
    if (c < bc) { bc = c; best = m; }
  }
  std::lock_guard<std::mutex> lk(mu);
  memo[n] = best;
  return best;
}

// ---------------------------------------------------------------- FP64 analytic signals
// Rows with at least FPCC_F64_ZERO_SAMPLES zero samples get FP64 analytic
// signals in the automatic mode (runs of zeros are where FP32 transforms lose
// the phase).
constexpr int kZeroSamples = FPCC_F64_ZERO_SAMPLES;

int twiddle64(fpcc_ctx* c, int n, const double2** out) {
  auto it = c->twiddles64.find(n);
  if (it != c->twiddles64.end()) { *out = it->second; return 0; }
  double2* d = nullptr;
  cudaError_t e = ctx_alloc(c, (void**)&d, (size_t)n * sizeof(double2));
  if (e != cudaSuccess) return fail(FPCC_ENOMEM, "FP64 twiddle table: %s", cudaGetErrorString(e));
  if ((e = launch_twiddles(nullptr, d, n, c->stream)) != cudaSuccess) {
    ctx_free(c, d);
    return cuda_fail(e, "FP64 twiddle table");
  }
  g_launches++;
  c->twiddles64[n] = d;
  *out = d;
  return 0;
}

// Radix-4/2/3/5 schedule of n (empty when n has another prime factor).
std::vector<int> radices64(int n) {
  std::vector<int> r;
  while (n % 4 == 0) { r.push_back(4); n /= 4; }
  if (n % 2 == 0) { r.push_back(2); n /= 2; }
  while (n % 3 == 0) { r.push_back(3); n /= 3; }
  while (n % 5 == 0) { r.push_back(5); n /= 5; }
  if (n != 1) r.clear();
  return r;
}

// n-point FP64 transforms of nrows rows held in A (ping-pong with B); *res gets the result.
int passes64(fpcc_ctx* c, double2* A, double2* B, int n, int nrows, int dir, double2** res) {
  const std::vector<int> rad = radices64(n);
  if (rad.empty() && n != 1) return fail(FPCC_EUNSUP, "length %d is not 2,3,5-smooth", n);
  const double2* tw = nullptr;
  int rc = twiddle64(c, n, &tw);
  if (rc) return rc;
  double2* bufs[2] = {A, B};
  int cur = 0, Ns = 1;
  for (int R : rad) {
    CK(launch_pass64(R, dir, bufs[cur], bufs[cur ^ 1], n, Ns, nrows, tw, c->stream));
    g_launches++;
    cur ^= 1;
    Ns *= R;
  }
  *res = bufs[cur];
  return 0;
}

// Double-float twiddle table of n points, from the FP64 table.
int twiddle_df(fpcc_ctx* c, int n, const float4** out) {
  auto it = c->twiddles_df.find(n);
  if (it != c->twiddles_df.end()) { *out = it->second; return 0; }
  const double2* t64 = nullptr;
  int rc = twiddle64(c, n, &t64);
  if (rc) return rc;
  float4* d = nullptr;
  cudaError_t e = ctx_alloc(c, (void**)&d, (size_t)n * sizeof(float4));
  if (e != cudaSuccess) return fail(FPCC_ENOMEM, "double-float twiddle table: %s", cudaGetErrorString(e));
  if ((e = launch_df_from_double(t64, d, n, c->stream)) != cudaSuccess) {
    ctx_free(c, d);
    return cuda_fail(e, "double-float twiddle table");
  }
  g_launches++;
  c->twiddles_df[n] = d;
  *out = d;
  return 0;
}

DfConsts df_consts() {
  auto split = [](double v) {
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
  };
  const double pi = 3.14159265358979323846;
  DfConsts k;
  k.s3 = split(std::sin(2 * pi / 3));
  k.c1 = split(std::cos(2 * pi / 5));
  k.c2 = split(std::cos(4 * pi / 5));
  k.s1 = split(std::sin(2 * pi / 5));
  k.s2 = split(std::sin(4 * pi / 5));
  k.c8 = split(std::cos(pi / 8));
  k.s8 = split(std::sin(pi / 8));
  k.r2 = split(std::sqrt(0.5));
  return k;
}

// n-point double-float transforms of nrows rows held in A (ping-pong with B).
int passes_df(fpcc_ctx* c, float4* A, float4* B, int n, int nrows, int dir, float4** res) {
  const std::vector<int> r64 = radices64(n);
  if (r64.empty() && n != 1) return fail(FPCC_EUNSUP, "length %d is not 2,3,5-smooth", n);
  // two consecutive radix-4 levels run as one radix-16 pass (half the global traffic)
  std::vector<int> rad;
  for (size_t i = 0; i < r64.size(); i++) {
    if (r64[i] == 4 && i + 1 < r64.size() && r64[i + 1] == 4) {
      rad.push_back(16);
      i++;
    } else {
      rad.push_back(r64[i]);
    }
  }
  const float4* tw = nullptr;
  int rc = twiddle_df(c, n, &tw);
  if (rc) return rc;
  static const DfConsts kc = df_consts();
  float4* bufs[2] = {A, B};
  int cur = 0, Ns = 1;
  for (int R : rad) {
    CK(launch_pass_df(R, dir, bufs[cur], bufs[cur ^ 1], n, Ns, nrows, tw, kc, c->stream));
    g_launches++;
    cur ^= 1;
    Ns *= R;
  }
  *res = bufs[cur];
  return 0;
}

// Rows whose analytic signals are to be computed in more than FP32 (double-float)
// under the context's mode.
int precise_rows(fpcc_ctx* c, const float* d_x, int64_t ldx, int nrows, int N, std::vector<int>* rows) {
  rows->clear();
  if (c->precision == FPCC_ANALYTIC_F32 || nrows <= 0) return 0;
  if (c->precision == FPCC_ANALYTIC_F64) {
    for (int r = 0; r < nrows; r++) rows->push_back(r);
    return 0;
  }
  void* cnt;
  int rc = dev_buf(c, S_P64_CNT, (size_t)nrows * sizeof(int), &cnt);
  if (rc) return rc;
  CK(launch_zero_count(d_x, ldx, N, nrows, (int*)cnt, c->stream));
  g_launches++;
  std::vector<int> h(nrows);
  CK(cudaMemcpyAsync(h.data(), cnt, (size_t)nrows * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int r = 0; r < nrows; r++)
    if (h[r] >= kZeroSamples) rows->push_back(r);
  return 0;
}

template <typename T>
int multi_group(fpcc_ctx* c, std::vector<MultiRow>& rows, int M);

// Overwrites the listed rows of the FP32 analytic signals `an` (stride ldan)
// with analytic signals of the same rows of x computed in double-float (the
// packed convolution stage: about 44 significant bits on the FP32 pipes),
// rounded to float2.
int refine_analytic(fpcc_ctx* c, const float* d_x, int64_t ldx, int N, const std::vector<int>& rows, float2* an,
                    int64_t ldan) {
  if (rows.empty()) return 0;
  std::vector<MultiRow> mr(rows.size());
  for (size_t i = 0; i < rows.size(); i++) {
    mr[i] = MultiRow{};
    mr[i].x = d_x + (int64_t)rows[i] * ldx;
    mr[i].out = an + (int64_t)rows[i] * ldan;
    mr[i].N = N;
  }
  return multi_group<float4>(c, mr, conv_class_len(N));
}

// Analytic signal for window lengths with a prime factor above 5, by Bluestein
// transforms (DFT_N then masked IDFT_N) on M-point generic passes.
int analytic_rows_bluestein(fpcc_ctx* c, const float* d_x, int64_t ldx, int nrows, int N, const float2** out,
                            const float** rmax, const float** rsum) {
  const int M = smooth_at_least(2 * N - 1);
  float2* Bf = nullptr;
  auto it = c->bluestein.find(N);
  if (it == c->bluestein.end()) {
    // filter spectra for both directions (computed once per N)
    CK(ctx_alloc(c, (void**)&Bf, (size_t)2 * M * sizeof(float2)));
    void* tmp;
    int rc = dev_buf(c, S_ANA_B, (size_t)2 * M * sizeof(float2), &tmp);
    if (rc) { ctx_free(c, Bf); return rc; }
    for (int d = 0; d < 2; d++) {
      const int dir = d ? +1 : -1;
      CK(launch_blue_filter(Bf + (size_t)d * M, N, M, dir, c->stream));
      float2* res = nullptr;
      if ((rc = passes(c, Bf + (size_t)d * M, (float2*)tmp, M, 1, -1, &res))) { ctx_free(c, Bf); return rc; }
      if (res != Bf + (size_t)d * M)
        CK(cudaMemcpyAsync(Bf + (size_t)d * M, res, (size_t)M * sizeof(float2), cudaMemcpyDeviceToDevice, c->stream));
    }
    c->bluestein[N] = Bf;
  } else {
    Bf = it->second;
  }
  void *A, *B, *O, *S;
  int rc;
  const size_t mb = (size_t)nrows * M * sizeof(float2);
  if ((rc = dev_buf(c, S_ANA_A, mb, &A)) || (rc = dev_buf(c, S_ANA_B, mb, &B)) ||
      (rc = dev_buf(c, S_BLUE_O, (size_t)nrows * N * sizeof(float2), &O)) ||
      (rc = dev_buf(c, S_RSTAT, (size_t)2 * nrows * sizeof(float), &S)))
    return rc;
  for (int d = 0; d < 2; d++) {
    const int dir = d ? +1 : -1;
    const void* src = d ? (const void*)O : (const void*)d_x;
    CK(launch_blue_pre(src, d == 0, d ? N : ldx, (float2*)A, M, N, M, dir, d, nrows, c->stream));
    float2* r1 = nullptr;
    if ((rc = passes(c, (float2*)A, (float2*)B, M, nrows, -1, &r1))) return rc;
    CK(launch_blue_mul(r1, M, Bf + (size_t)d * M, M, nrows, c->stream));
    float2* r2 = nullptr;
    float2* other = (r1 == (float2*)A) ? (float2*)B : (float2*)A;
    if ((rc = passes(c, r1, other, M, nrows, +1, &r2))) return rc;
    CK(launch_blue_post(r2, M, (float2*)O, N, N, M, dir, nrows, c->stream));
    g_launches += 3;
  }
  float* st = (float*)S;
  CK(launch_rowstats((const float2*)O, N, N, nrows, st, st + nrows, c->stream));
  g_launches++;
  *out = (const float2*)O;
  *rmax = st;
  *rsum = st + nrows;
  return 0;
}

// Analytic signal of nrows real rows (src/FFTapps.c:104-124): DFT_N, mask,
// IDFT_N, by generic passes.  Leaves the rows (stride N) in *out and the row
// statistics (max and sum of |a|^2) in *rmax / *rsum.
int analytic_rows(fpcc_ctx* c, const float* d_x, int64_t ldx, int nrows, int N, const float2** out,
                  const float** rmax, const float** rsum) {
  FftPlan p;
  if (!make_plan(N, &p)) return analytic_rows_bluestein(c, d_x, ldx, nrows, N, out, rmax, rsum);
  const float2* tw = nullptr;
  int rc = twiddle_table(c, N, &tw);
  if (rc) return rc;
  void *A, *B, *S;
  const size_t bytes = (size_t)nrows * N * sizeof(float2);
  if ((rc = dev_buf(c, S_ANA_A, bytes, &A)) || (rc = dev_buf(c, S_ANA_B, bytes, &B)) ||
      (rc = dev_buf(c, S_RSTAT, (size_t)2 * nrows * sizeof(float), &S)))
    return rc;
  float2* bufs[2] = {(float2*)A, (float2*)B};
  int cur = 0;   // buffer holding the current data (after the first pass)
  for (int dir = -1; dir <= 1; dir += 2) {
    int Ns = 1;
    for (int i = 0; i < p.npass; i++) {
      const int R = p.rad[i];
      const bool first = (dir < 0 && i == 0);
      float2* dst = first ? bufs[0] : bufs[cur ^ 1];
      const void* src = first ? (const void*)d_x : (const void*)bufs[cur];
      CK(launch_gpass(R, dir, src, first, ldx, dst, N, N, Ns, nrows, tw, c->stream));
      g_launches++;
      cur = first ? 0 : (cur ^ 1);
      Ns *= R;
    }
    if (p.npass == 0 && dir < 0) {
      // N == 1: copy the real sample in through a radix-free pass is not possible; unsupported
      return fail(FPCC_EUNSUP, "N=1");
    }
    if (dir < 0) {
      CK(launch_analytic_mask(bufs[cur], N, N, nrows, c->stream));
      g_launches++;
    }
  }
  float* st = (float*)S;
  CK(launch_rowstats(bufs[cur], N, N, nrows, st, st + nrows, c->stream));
  g_launches++;
  *out = bufs[cur];
  *rmax = st;
  *rsum = st + nrows;
  return 0;
}

// Analytic signals of nrows rows with the listed rows in FP64: when every row is
// listed the FP32 transforms are skipped altogether.
int analytic_rows_p64(fpcc_ctx* c, const float* d_x, int64_t ldx, int nrows, int N, const std::vector<int>& rows,
                      const float2** out, const float** rmax, const float** rsum) {
  if ((int)rows.size() != nrows || nrows == 0) {
    int rc = analytic_rows(c, d_x, ldx, nrows, N, out, rmax, rsum);
    if (rc || rows.empty()) return rc;
    rc = refine_analytic(c, d_x, ldx, N, rows, const_cast<float2*>(*out), N);
    if (rc) return rc;
  } else {
    void *A, *S;
    int rc;
    if ((rc = dev_buf(c, S_ANA_A, (size_t)nrows * N * sizeof(float2), &A)) ||
        (rc = dev_buf(c, S_RSTAT, (size_t)2 * nrows * sizeof(float), &S)))
      return rc;
    if ((rc = refine_analytic(c, d_x, ldx, N, rows, (float2*)A, N))) return rc;
    *out = (const float2*)A;
    *rmax = (const float*)S;
    *rsum = (const float*)S + nrows;
  }
  CK(launch_rowstats(*out, N, N, nrows, const_cast<float*>(*rmax), const_cast<float*>(*rsum), c->stream));
  g_launches++;
  return 0;
}

// ---------------------------------------------------------------- packed analytic signals

constexpr size_t kMultiFilterCache = (size_t)4 << 30;   // bytes of cached filter spectra per context

// Kernel spectra H_N = FFT_M(kernel) / M of every window length in Ns, for
// transforms of M points in precision T; returns a device pointer per entry of
// Ns.  The spectra are real (float for T = float2, double-float float2 for
// T = float4).  New lengths are computed together, two kernels per row of one
// batched double-float transform (launch_hk_rows), and cached in blocks; the
// cache is emptied first when it would grow past kMultiFilterCache.
template <typename T>
int multi_filters(fpcc_ctx* c, const std::vector<int>& Ns, int M, std::vector<const void*>& filt) {
  constexpr bool dfl = std::is_same<T, float4>::value;
  constexpr size_t hsz = dfl ? sizeof(float2) : sizeof(float);
  const int f64 = dfl ? 1 : 0;
  std::vector<int> missing;
  for (int N : Ns)
    if (!c->multi_filters.count(std::make_tuple(N, M, f64)) &&
        std::find(missing.begin(), missing.end(), N) == missing.end())
      missing.push_back(N);
  const size_t need = missing.size() * (size_t)M * hsz;
  if (need && c->multi_filter_bytes + need > kMultiFilterCache && c->multi_filter_bytes) {
    for (void* b : c->multi_blocks) ctx_free(c, b);   // in stream order: later work cannot read them
    c->multi_blocks.clear();
    c->multi_filters.clear();
    c->multi_filter_bytes = 0;
    missing.clear();
    for (int N : Ns)
      if (std::find(missing.begin(), missing.end(), N) == missing.end()) missing.push_back(N);
  }
  // lengths per batch: at most 128, and transform buffers of at most 256 MB each
  const size_t rows_max = std::max<size_t>(1, ((size_t)256 << 20) / ((size_t)M * sizeof(float4)));
  const size_t per = std::min<size_t>(128, 2 * rows_max);
  const int ldt = hk_table_len(M);
  for (size_t i0 = 0; i0 < missing.size(); i0 += per) {
    const int n = (int)std::min<size_t>(per, missing.size() - i0);
    const int rows = (n + 1) / 2;
    const std::vector<int> lens(missing.begin() + i0, missing.begin() + i0 + n);
    void *B, *A, *dN, *tab;
    int rc;
    if ((rc = dev_buf(c, S_MULTI_B, (size_t)rows * M * sizeof(float4), &B)) ||
        (rc = dev_buf(c, S_MULTI_A, (size_t)rows * M * sizeof(float4), &A)) ||
        (rc = dev_buf(c, S_P64_CNT, (size_t)n * sizeof(int), &dN)) ||
        (rc = dev_buf(c, S_HK_TAB, (size_t)n * ldt * sizeof(double2), &tab)))
      return rc;
    CK(cudaMemcpyAsync(dN, lens.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(launch_hk_rows((const int*)dN, n, (double2*)tab, (float4*)A, M, c->stream));
    void* block = nullptr;
    CK(ctx_alloc(c, &block, (size_t)n * M * hsz));
    c->multi_blocks.push_back(block);
    c->multi_filter_bytes += (size_t)n * M * hsz;
    float4* r = nullptr;
    if ((rc = passes_df(c, (float4*)A, (float4*)B, M, rows, -1, &r))) return rc;
    CK(launch_hk_extract(r, n, M, dfl, block, c->stream));
    g_launches += 3;
    for (int j = 0; j < n; j++)
      c->multi_filters[std::make_tuple(lens[j], M, f64)] = (char*)block + (size_t)j * M * hsz;
  }
  filt.resize(Ns.size());
  for (size_t i = 0; i < Ns.size(); i++) filt[i] = c->multi_filters.at(std::make_tuple(Ns[i], M, f64));
  return 0;
}

// Analytic signals of `rows` (all of length class M, precision T) into their
// out pointers, in chunks that keep each transform buffer under 512 MB: pairs of
// windows share a forward transform, each window gets its own inverse one.
template <typename T>
int multi_group(fpcc_ctx* c, std::vector<MultiRow>& rows, int M) {
  std::vector<int> Ns(rows.size());
  for (size_t i = 0; i < rows.size(); i++) Ns[i] = rows[i].N;
  std::vector<const void*> filt;
  int rc = multi_filters<T>(c, Ns, M, filt);
  if (rc) return rc;
  for (size_t i = 0; i < rows.size(); i++) rows[i].filt = filt[i];
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(4096, ((size_t)512 << 20) / ((size_t)M * sizeof(T))));
  for (size_t r0 = 0; r0 < rows.size(); r0 += chunk) {
    const int n = (int)std::min<size_t>(chunk, rows.size() - r0);
    const int np = (n + 1) / 2;
    void *A, *B, *d;
    if ((rc = dev_buf(c, S_MULTI_A, (size_t)n * M * sizeof(T), &A)) ||
        (rc = dev_buf(c, S_MULTI_B, (size_t)n * M * sizeof(T), &B)) ||
        (rc = dev_buf(c, S_P64_CNT, (size_t)n * sizeof(MultiRow), &d)))
      return rc;
    CK(cudaMemcpyAsync(d, rows.data() + r0, (size_t)n * sizeof(MultiRow), cudaMemcpyHostToDevice, c->stream));
    CK(launch_multi_exp((MultiRow*)d, n, c->stream));
    const MultiRow* dr = (const MultiRow*)d;
    constexpr bool dfl = std::is_same<T, float4>::value;
    auto tr = [&](T* in, T* other, int nr, int dir, T** res) -> int {
      if constexpr (dfl) return passes_df(c, (float4*)in, (float4*)other, M, nr, dir, (float4**)res);
      else return passes(c, (float2*)in, (float2*)other, M, nr, dir, (float2**)res);
    };
    T* z = nullptr;
    if constexpr (dfl) CK(launch_multi_load2_df(dr, n, (float4*)A, M, c->stream));
    else CK(launch_multi_load2<T>(dr, n, (T*)A, M, c->stream));
    if ((rc = tr((T*)A, (T*)B, np, -1, &z))) return rc;
    T* y = (z == (T*)A) ? (T*)B : (T*)A;
    if constexpr (dfl) CK(launch_multi_split_df(dr, n, (const float4*)z, (float4*)y, M, c->stream));
    else CK(launch_multi_split<T>(dr, n, z, y, M, c->stream));
    T* res = nullptr;
    if ((rc = tr(y, z, n, +1, &res))) return rc;
    if constexpr (dfl) CK(launch_multi_store_df(dr, n, (const float4*)res, M, c->stream));
    else CK(launch_multi_store<T>(dr, n, res, M, c->stream));
    g_launches += 3;
  }
  return 0;
}

}  // namespace

extern "C" int fpcc_station_stage_multi(fpcc_ctx* c, int method, const fpcc_station_row* h_rows, int nrows,
                                        int fmt, int rule, void* d_out, int64_t ldo) {
  if (!c || (!h_rows && nrows > 0) || !d_out) return fail(FPCC_EARG, "null argument");
  if (nrows <= 0) return 0;
  if (method != FPCC_PCC2 && method != FPCC_PCC1 && method != FPCC_PCCV)
    return fail(FPCC_EUNSUP, "the packed station stage serves the phase methods");
  if (fmt < FPCC_F32 || fmt > FPCC_I16) return fail(FPCC_EARG, "unknown storage format %d", fmt);
  for (int r = 1; r < nrows; r++)
    if (h_rows[r].N < h_rows[r - 1].N || (h_rows[r].N == h_rows[r - 1].N && h_rows[r].Nz < h_rows[r - 1].Nz))
      return fail(FPCC_EARG, "rows must be ordered by (N, Nz)");
  for (int r = 0; r < nrows; r++) {
    const auto& q = h_rows[r];
    if (q.N <= 0 || !q.d_x) return fail(FPCC_EARG, "row %d: bad window", r);
    if (method == FPCC_PCC2) {
      if (q.Nz < q.N || (q.Nz & 1)) return fail(FPCC_EARG, "row %d: Nz=%d must be even and >= N", r, q.Nz);
      if (fpcc_station_row_bytes(method, q.N, q.Nz, fmt) > ldo * (fmt == FPCC_F32 ? 8 : 4))
        return fail(FPCC_EARG, "row %d does not fit ldo", r);
    } else if (q.N > ldo) {
      return fail(FPCC_EARG, "row %d does not fit ldo", r);
    }
  }
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  // analytic signals, packed: row r at offset off[r] (float2)
  std::vector<int64_t> off(nrows + 1, 0);
  for (int r = 0; r < nrows; r++) off[r + 1] = off[r] + h_rows[r].N;
  void *an, *st;
  int rc;
  if ((rc = dev_buf(c, S_MULTI_AN, (size_t)off[nrows] * sizeof(float2), &an)) ||
      (rc = dev_buf(c, S_RSTAT, (size_t)2 * nrows * sizeof(float), &st)))
    return rc;
  std::map<std::pair<int, int>, std::vector<MultiRow>> groups;   // (M, fp64)
  std::vector<MultiRow> all(nrows);
  for (int r = 0; r < nrows; r++) {
    MultiRow m{};
    m.x = h_rows[r].d_x;
    m.out = (float2*)an + off[r];
    m.N = h_rows[r].N;
    all[r] = m;
    groups[{conv_class_len(m.N), h_rows[r].f64 ? 1 : 0}].push_back(m);
  }
  for (auto& kv : groups) {
    const int M = kv.first.first;
    // windows with gaps: double-float transforms (FP32 pipes, about 44 significant bits)
    rc = kv.first.second ? multi_group<float4>(c, kv.second, M) : multi_group<float2>(c, kv.second, M);
    if (rc) return rc;
  }
  void* dall;
  if ((rc = dev_buf(c, S_P64_CNT, (size_t)nrows * sizeof(MultiRow), &dall))) return rc;
  CK(cudaMemcpyAsync(dall, all.data(), (size_t)nrows * sizeof(MultiRow), cudaMemcpyHostToDevice, c->stream));
  float* rmax = (float*)st;
  float* rsum = rmax + nrows;
  CK(launch_multi_rowstats((const MultiRow*)dall, nrows, rmax, rsum, c->stream));
  g_launches++;
  const size_t oesz = fmt == FPCC_F32 ? 8 : 4;
  if (method != FPCC_PCC2) {
    // phase signals: one launch over every row, each with its own offset and length
    std::vector<int64_t> roff(off.begin(), off.begin() + nrows);
    std::vector<int> rN(nrows);
    int Nmax = 0;
    for (int r = 0; r < nrows; r++) { rN[r] = h_rows[r].N; Nmax = std::max(Nmax, rN[r]); }
    void* dmeta;
    if ((rc = dev_buf(c, S_CONV_X, (size_t)nrows * (sizeof(int64_t) + sizeof(int)), &dmeta))) return rc;
    CK(cudaMemcpyAsync(dmeta, roff.data(), (size_t)nrows * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync((char*)dmeta + (size_t)nrows * sizeof(int64_t), rN.data(), (size_t)nrows * sizeof(int),
                       cudaMemcpyHostToDevice, c->stream));
    PhaseArgs a{};
    a.in = (const float2*)an; a.ldin = 0; a.nrows = nrows; a.N = Nmax; a.rule = rule;
    a.rowstat = (rule == FPCC_AMP_SUMTHR) ? rsum : rmax; a.fmt = fmt; a.out = d_out; a.ldo = ldo;
    a.row_in = (const int64_t*)dmeta;
    a.row_N = (const int*)((char*)dmeta + (size_t)nrows * sizeof(int64_t));
    CK(launch_phase_store(a, c->stream));
    g_launches++;
    return 0;
  }
  // normalisation, zero padding and DFT_Nz per (N, Nz) run of rows
  for (int r0 = 0; r0 < nrows;) {
    int r1 = r0 + 1;
    while (r1 < nrows && h_rows[r1].N == h_rows[r0].N && h_rows[r1].Nz == h_rows[r0].Nz) r1++;
    const int N = h_rows[r0].N, Nz = h_rows[r0].Nz, n = r1 - r0;
    const float2* in = (const float2*)an + off[r0];
    const float* rs = ((rule == FPCC_AMP_SUMTHR) ? rsum : rmax) + r0;
    void* out = (char*)d_out + (size_t)r0 * ldo * oesz;
    if (method == FPCC_PCC2) {
      if (spec_supported(Nz)) {
        SpecArgs a{};
        a.in = in; a.ldin = N; a.nrows = n; a.N = N; a.Nz = Nz; a.mode = SPEC_PHASE; a.rule = rule;
        a.rowstat = rs; a.fmt = fmt; a.out = out; a.ldo = ldo;
        CK(launch_spec(a, c->stream));
        g_launches++;
      } else if ((rc = large_station(c, COL_PHASE, in, sizeof(float2), N, n, N, Nz, rule, rs, 0, fmt, 0, out, ldo))) {
        return rc;
      }
    } else {
      PhaseArgs a{};
      a.in = in; a.ldin = N; a.nrows = n; a.N = N; a.rule = rule; a.rowstat = rs;
      a.fmt = fmt; a.out = out; a.ldo = ldo;
      CK(launch_phase_store(a, c->stream));
      g_launches++;
    }
    r0 = r1;
  }
  return 0;
}

extern "C" int fpcc_station_stage(fpcc_ctx* c, int method, const float* d_x, int64_t ldx, int nrows, int N,
                                  int Nz, int fmt, int rule, void* d_out, int64_t ldo) {
  return fpcc_station_stage_ex(c, method, d_x, ldx, nrows, N, Nz, fmt, rule, d_out, ldo, nullptr, -1);
}

namespace {
int station_general(fpcc_ctx* c, int method, const float* d_x, int64_t ldx, int nrows, int N, int Nz, int fmt,
                    int rule, void* d_out, int64_t ldo, const std::vector<int>& p64);
}  // namespace

extern "C" int fpcc_station_stage_ex(fpcc_ctx* c, int method, const float* d_x, int64_t ldx, int nrows, int N,
                                     int Nz, int fmt, int rule, void* d_out, int64_t ldo, const int32_t* h_f64_rows,
                                     int n_f64_rows) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (nrows <= 0) return 0;
  if (N <= 0) return fail(FPCC_EARG, "N must be positive");
  int rc;
  if (method == FPCC_CC1B_POPCOUNT) {
    CK(launch_sign_bits(d_x, ldx, nrows, N, (uint32_t*)d_out, ldo, rule == FPCC_SIGN_GE ? 1 : 0, nullptr,
                        c->stream));
    g_launches++;
    return 0;
  }
  std::vector<int> p64;   // rows whose analytic signals are computed in FP64
  const bool phase_method = (method == FPCC_PCC1 || method == FPCC_PCCV || method == FPCC_PCC2);
  if (phase_method) {
    if (n_f64_rows >= 0) {
      for (int i = 0; i < n_f64_rows; i++) {
        if (!h_f64_rows || h_f64_rows[i] < 0 || h_f64_rows[i] >= nrows) return fail(FPCC_EARG, "bad FP64 row list");
        p64.push_back(h_f64_rows[i]);
      }
    } else if ((rc = precise_rows(c, d_x, ldx, nrows, N, &p64))) {
      return rc;
    }
    std::sort(p64.begin(), p64.end());
    p64.erase(std::unique(p64.begin(), p64.end()), p64.end());
  }
  if (method == FPCC_PCC1 || method == FPCC_PCCV) {
    const float2 *an; const float *rmax, *rsum;
    if ((rc = analytic_rows_p64(c, d_x, ldx, nrows, N, p64, &an, &rmax, &rsum))) return rc;
    PhaseArgs a{};
    a.in = an; a.ldin = N; a.nrows = nrows; a.N = N; a.rule = rule;
    a.rowstat = (rule == FPCC_AMP_SUMTHR) ? rsum : rmax;
    a.fmt = fmt; a.out = d_out; a.ldo = ldo;
    CK(launch_phase_store(a, c->stream));
    g_launches++;
    return 0;
  }
  if (method != FPCC_PCC2 && method != FPCC_GNCC && method != FPCC_CC1B)
    return fail(FPCC_EUNSUP, "method %d has no station stage", method);
  if (Nz < N || (Nz & 1)) return fail(FPCC_EARG, "Nz=%d must be even and >= N=%d", Nz, N);
  if ((method == FPCC_GNCC || method == FPCC_CC1B) && fmt != FPCC_F32)
    return fail(FPCC_EUNSUP, "real-trace spectra are stored in F32");
  if (fmt == FPCC_I16 && ldo < (int64_t)Nz + 4)
    return fail(FPCC_EARG, "int16 spectrum rows need ldo >= Nz + 4 (16-byte header)");
  if (!spec_supported(Nz)) {
    if (method == FPCC_PCC2) {
      const float2 *an; const float *rmax, *rsum;
      if ((rc = analytic_rows_p64(c, d_x, ldx, nrows, N, p64, &an, &rmax, &rsum))) return rc;
      return large_station(c, COL_PHASE, an, sizeof(float2), N, nrows, N, Nz, rule,
                           (rule == FPCC_AMP_SUMTHR) ? rsum : rmax, 0, fmt, 0, d_out, ldo);
    }
    return large_station(c, method == FPCC_GNCC ? COL_REAL : COL_SIGN, d_x, sizeof(float), ldx, nrows, N, Nz, 0,
                         nullptr, rule == FPCC_SIGN_GE ? 1 : 0, FPCC_F32, 1, d_out, ldo);
  }
  if (method == FPCC_PCC2 && (int)p64.size() < nrows) {
    // one fused kernel per station window, specialised at run time for (N, Nz);
    // windows with gaps (FP64 analytic signals) are then redone on their own
    // through the general path, so that every window's spectrum depends on that
    // window only, not on the others of the call (a call whose windows all have
    // gaps goes to the general path directly: no fused kernel to specialise)
    const cudaError_t e = launch_station_fused(d_x, ldx, nrows, N, Nz, rule, fmt, d_out, ldo, c->stream);
    if (e == cudaSuccess) {
      g_launches++;
      if (p64.empty()) return 0;
      const int np = (int)p64.size();
      const int64_t words = fpcc_station_row_bytes(method, N, Nz, fmt) / 4;
      const int64_t ldo_w = ldo * (fmt == FPCC_F32 ? 2 : 1);
      void *gx, *go, *gi;
      if ((rc = dev_buf(c, S_GATHER_X, (size_t)np * N * sizeof(float), &gx)) ||
          (rc = dev_buf(c, S_GATHER_O, (size_t)np * ldo_w * 4, &go)) ||
          (rc = dev_buf(c, S_GATHER_I, (size_t)np * sizeof(int), &gi)))
        return rc;
      CK(cudaMemcpyAsync(gi, p64.data(), (size_t)np * sizeof(int), cudaMemcpyHostToDevice, c->stream));
      CK(launch_rows_copy(d_x, ldx, (const int*)gi, gx, N, nullptr, np, N, c->stream));
      std::vector<int> all((size_t)np);
      for (int i = 0; i < np; i++) all[(size_t)i] = i;
      if ((rc = station_general(c, method, (const float*)gx, N, np, N, Nz, fmt, rule, go, ldo, all))) return rc;
      CK(launch_rows_copy(go, ldo_w, nullptr, d_out, ldo_w, (const int*)gi, np, words, c->stream));
      g_launches += 2;
      return 0;
    }
    if (e != cudaErrorNotSupported) return cuda_fail(e, "fused station kernel");
  }
  return station_general(c, method, d_x, ldx, nrows, N, Nz, fmt, rule, d_out, ldo, p64);
}

namespace {
// The station stage of PCC2 (analytic signals, FP64 for the rows in p64, then
// the phase spectra), GNCC and 1-bit (spectra of the real rows) by general
// radix passes.
int station_general(fpcc_ctx* c, int method, const float* d_x, int64_t ldx, int nrows, int N, int Nz, int fmt,
                    int rule, void* d_out, int64_t ldo, const std::vector<int>& p64) {
  int rc;
  SpecArgs a{};
  a.nrows = nrows; a.N = N; a.Nz = Nz; a.fmt = fmt; a.out = d_out; a.ldo = ldo;
  if (method == FPCC_PCC2) {
    const float2 *an; const float *rmax, *rsum;
    if ((rc = analytic_rows_p64(c, d_x, ldx, nrows, N, p64, &an, &rmax, &rsum))) return rc;
    a.in = an; a.ldin = N; a.mode = SPEC_PHASE; a.rule = rule;
    a.rowstat = (rule == FPCC_AMP_SUMTHR) ? rsum : rmax;
  } else {
    a.in = d_x; a.ldin = ldx;
    a.mode = (method == FPCC_GNCC) ? SPEC_REAL : SPEC_SIGN;
    a.sign_ge = (rule == FPCC_SIGN_GE) ? 1 : 0;
  }
  CK(launch_spec(a, c->stream));
  g_launches++;
  return 0;
}
}  // namespace

extern "C" int fpcc_energy_stage(fpcc_ctx* c, const float* d_x, int64_t ldx, int nrows, int N, double* d_E,
                                 int64_t ldE) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (nrows <= 0 || N <= 0) return 0;
  if (!d_x || !d_E || ldE < (int64_t)N + 1 || ldx < N) return fail(FPCC_EARG, "bad energy stage arguments");
  const int blk = std::min(nrows, 65535);   // rows per launch pair (grid y)
  void* part;
  int rc = dev_buf(c, S_EPART, (size_t)blk * energy_chunks(N) * sizeof(double), &part);
  if (rc) return rc;
  // rows with room for them also get the pair stage's normalisation tables
  const bool tables = ldE >= 2 * ((int64_t)N + 1);
  for (int r0 = 0; r0 < nrows; r0 += blk) {
    const int n = std::min(blk, nrows - r0);
    CK(launch_energy_prefix(d_x + (size_t)r0 * ldx, ldx, n, N, d_E + (size_t)r0 * ldE, ldE, (double*)part, tables,
                            c->stream));
    g_launches += tables ? 3 : 2;
  }
  return 0;
}

extern "C" int fpcc_pair_stage(fpcc_ctx* c, int method, const void* d_station, int64_t lds, int fmt,
                               const int32_t* d_pairs, int npairs, int N, int Nz, int Lag1, int Lag2, float v,
                               const double* d_E, int64_t ldE, float* d_y, int64_t ldy, int64_t* d_num) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (npairs <= 0) return 0;
  int rc = check_lags(N, Lag1, Lag2);
  if (rc) return rc;
  int lag0, L;
  lag_window(Lag1, Lag2, &lag0, &L);
  const int M = abs(Lag1) > abs(Lag2) ? abs(Lag1) : abs(Lag2);
  if (is_fft_method(method)) {
    if (Nz < N + M || (Nz & 1)) return fail(FPCC_EARG, "Nz=%d must be even and >= N+M=%d", Nz, N + M);
    PairArgs a{};
    a.spec = d_station;
    a.ldspec = lds;
    a.fmt = fmt;
    a.pairs = reinterpret_cast<const int2*>(d_pairs);
    a.npairs = npairs;
    a.Nz = Nz;
    const bool inblock = pair_supported(Nz);
    a.lag0 = lag0;
    a.L = L;
    a.y = d_y;
    a.ldy = ldy;
    a.N = N;
    if (method == FPCC_PCC2) {
      a.norm = 0;
      a.scale = 1.0f / ((float)Nz * (float)N);   // src/FFTapps.c:832
    } else if (method == FPCC_GNCC) {
      if (!d_E) return fail(FPCC_EARG, "GNCC needs the energy prefix sums");
      a.norm = 1;
      a.energy = d_E;
      a.ldE = ldE;
      a.scale = (float)(1.0 / (double)Nz);       // src/FFTapps.c:340
      if (fmt != FPCC_F32) return fail(FPCC_EUNSUP, "GNCC spectra are F32");
    } else {
      a.norm = 2;
      a.scale = (float)(1.0 / (double)Nz);       // src/FFTapps.c:357
      if (fmt != FPCC_F32) return fail(FPCC_EUNSUP, "1-bit spectra are F32");
    }
    if (!inblock) return large_pairs(c, a, method == FPCC_PCC2 ? 0 : 1);
    CK(launch_pairs(a, c->stream));
    g_launches++;
    return 0;
  }
  if (method == FPCC_PCC1 || method == FPCC_PCCV) {
    PccvArgs a{};
    a.phase = d_station;
    a.ldp = lds;
    a.half = fmt;
    a.pairs = reinterpret_cast<const int2*>(d_pairs);
    a.npairs = npairs;
    a.N = N;
    a.Lag1 = lag0;
    a.L = L;
    a.v = (method == FPCC_PCC1) ? 1.0f : v;
    // the PCC1 path and the GPU PCC_v path divide by 2(N-|lag|) (src/FFTapps.c:276,
    // src/ccs_cuda.cu:452); the CPU PCC_v path by 2^(v/2)(N-|lag|) (src/FFTapps.c:334)
    a.norm_gpu = 1;
    a.y = d_y;
    a.ldy = ldy;
    CK(launch_pccv(a, c->stream));
    g_launches++;
    return 0;
  }
  if (method == FPCC_CC1B_POPCOUNT) {
    Cc1bArgs a{};
    a.bits = (const uint32_t*)d_station;
    a.ldb = lds;
    a.pairs = reinterpret_cast<const int2*>(d_pairs);
    a.npairs = npairs;
    a.N = N;
    a.lag0 = lag0;
    a.L = L;
    a.y = d_y;
    a.num = reinterpret_cast<long long*>(d_num);
    a.ldy = ldy;
    CK(launch_cc1b_popcount(a, c->stream));
    g_launches++;
    return 0;
  }
  return fail(FPCC_EUNSUP, "method %d has no pair stage", method);
}

extern "C" int fpcc_pair_stage_packed(fpcc_ctx* c, int method, int fmt, int Nz, const fpcc_pair_desc* d_desc,
                                      int npairs, int maxL, float v, int numerators) {
  if (!c) return fail(FPCC_EARG, "null context");
  if (npairs <= 0) return 0;
  if (!d_desc || maxL <= 0) return fail(FPCC_EARG, "packed pair stage needs descriptors and maxL > 0");
  if (npairs > 0x7fffffff / 2) return fail(FPCC_EARG, "too many pairs");
  if (is_fft_method(method)) {
    if (Nz & 1) return fail(FPCC_EARG, "packed pair stage: Nz=%d must be even", Nz);
    if (method != FPCC_PCC2 && fmt != FPCC_F32) return fail(FPCC_EUNSUP, "GNCC and 1-bit spectra are F32");
    PairArgs a{};
    a.fmt = fmt;
    a.npairs = npairs;
    a.Nz = Nz;
    a.norm = method == FPCC_PCC2 ? 0 : (method == FPCC_GNCC ? 1 : 2);
    a.desc = d_desc;
    if (!pair_supported(Nz)) return large_pairs(c, a, method == FPCC_PCC2 ? 0 : 1);
    CK(launch_pairs(a, c->stream));
    g_launches++;
    return 0;
  }
  if (method == FPCC_PCC1 || method == FPCC_PCCV) {
    PccvArgs a{};
    a.half = fmt;
    a.npairs = npairs;
    a.L = maxL;
    a.v = (method == FPCC_PCC1) ? 1.0f : v;
    a.norm_gpu = 1;
    a.desc = d_desc;
    CK(launch_pccv(a, c->stream));
    g_launches++;
    return 0;
  }
  if (method == FPCC_CC1B_POPCOUNT) {
    Cc1bArgs a{};
    a.npairs = npairs;
    a.L = maxL;
    a.desc = d_desc;
    a.desc_num = numerators ? 1 : 0;
    CK(launch_cc1b_popcount(a, c->stream));
    g_launches++;
    return 0;
  }
  return fail(FPCC_EUNSUP, "method %d has no packed pair stage", method);
}

// ============================================================== host entry points
namespace {

struct Layout {
  int method, N, Nz, lag0, L, fmt;
  int64_t lds;      // station row elements
  size_t esz;       // station element bytes
  bool two_rules;   // 1-bit: station 1 and 2 rows use different sign rules
  // GNCC energy row: N + 1 FP64 prefix sums and the normalisation tables (2 (N + 1) floats)
  int64_t ldE() const { return 2 * ((int64_t)N + 1); }
};

int make_layout(int method, int N, int Lag1, int Lag2, int nz_mode, int fmt, Layout* o) {
  int rc = check_lags(N, Lag1, Lag2);
  if (rc) return rc;
  o->method = method;
  o->N = N;
  lag_window(Lag1, Lag2, &o->lag0, &o->L);
  o->Nz = is_fft_method(method) ? fpcc_choose_nz(N, Lag1, Lag2, nz_mode) : N;
  if (o->Nz <= 0) return fail(FPCC_EUNSUP, "no padded length for N=%d", N);
  if (method == FPCC_GNCC || method == FPCC_CC1B) fmt = FPCC_F32;
  o->fmt = fmt;
  if (fmt < FPCC_F32 || fmt > FPCC_I16) return fail(FPCC_EARG, "unknown storage format %d", fmt);
  o->esz = (method == FPCC_CC1B_POPCOUNT) ? 4 : (fmt == FPCC_F32 ? 8 : 4);
  const int64_t rb = fpcc_station_row_bytes(method, N, o->Nz, fmt);
  if (rb < 0) return fail(FPCC_EUNSUP, "method %d not available here", method);
  o->lds = rb / (int64_t)o->esz;
  o->two_rules = (method == FPCC_CC1B || method == FPCC_CC1B_POPCOUNT);
  return 0;
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// All pairs with pinned host buffers, in the order the pair list first uses
// the rows: the used rows are laid out on the device in first-use order (the
// pair list is rewritten onto that order), so that the rows of the first pairs
// go up first, each run of rows at one host stride as one strided copy; the
// station stage runs on contiguous chunks of those rows as they arrive (a small
// first chunk, then 768 rows), each chunk's gap counts come back on a third
// stream (the host never waits behind pair stages), the pairs whose rows are
// all transformed run in pieces, and each piece's results go down on the
// third stream once every row is up (the two directions share the host link,
// and downloads beside the uploads starve them) while later pieces compute.  Results are the same as through
// run_device: every row goes through the same station stage, with its FP64
// rows chosen by the same rule.  Returns 1, with nothing queued, when the pair
// list's first-use order breaks into too many runs (no row structure to use).
int run_first_use(fpcc_ctx* c, const Layout& Ly, float* d_x, int nsta, const int32_t* h_pairs, int32_t* d_p,
                  int npairs, float v, float* d_y, float* h_y, const float* h_x) {
  const int method = Ly.method;
  const int N = Ly.N;
  int rc;
  // the rewritten pair list goes straight into pinned staging for its upload
  void* hps = nullptr;
  if ((rc = pin_buf(c, 7, 2 * (size_t)npairs * sizeof(int32_t), &hps))) return rc;
  int32_t* hp = (int32_t*)hps;
  std::vector<int> pos((size_t)nsta, -1), order;
  order.reserve((size_t)nsta);
  std::vector<int> need((size_t)npairs);   // rows first used by pairs 0..i
  for (int i = 0; i < npairs; i++) {
    for (int h = 0; h < 2; h++) {
      const int r = h_pairs[2 * (size_t)i + h];
      if (r < 0 || r >= nsta) return fail(FPCC_EARG, "pair row index out of range");
      if (pos[(size_t)r] < 0) {
        pos[(size_t)r] = (int)order.size();
        order.push_back(r);
      }
      hp[2 * (size_t)i + h] = pos[(size_t)r];
    }
    need[(size_t)i] = (int)order.size();
  }
  const int nuse = (int)order.size();
  // runs of rows at one host stride (device rows contiguous)
  struct Run { int d0, r0, stride, len; };
  std::vector<Run> runs;
  for (int a = 0; a < nuse;) {
    int b = a + 1;
    int stride = b < nuse ? order[(size_t)b] - order[(size_t)a] : 1;
    if (stride < 1 || (int64_t)stride * N * (int64_t)sizeof(float) > (1 << 30)) stride = 0;
    if (stride) while (b < nuse && order[(size_t)b] - order[(size_t)b - 1] == stride) b++;
    else b = a + 1;
    runs.push_back({a, order[(size_t)a], stride ? stride : 1, b - a});
    a = b;
  }
  if (runs.size() > (size_t)std::max(64, nuse / 8)) return 1;
  // station chunks: rows [R[k], R[k+1]); the first one small so that results start early
  std::vector<int> R{0};
  for (int r = std::min(nuse, 256); ; r = std::min(nuse, r + 768)) {
    R.push_back(r);
    if (r == nuse) break;
  }
  const int nch = (int)R.size() - 1;
  void* d_st = nullptr;
  const size_t rowb = (size_t)Ly.lds * Ly.esz;
  if ((rc = dev_buf(c, S_STATION, (size_t)nuse * rowb, &d_st))) return rc;
  double* d_E = nullptr;
  if (method == FPCC_GNCC) {
    void* p = nullptr;
    if ((rc = dev_buf(c, S_ENERGY, (size_t)nuse * Ly.ldE() * sizeof(double), &p))) return rc;
    d_E = (double*)p;
  }
  const bool phase = (method == FPCC_PCC2 || method == FPCC_PCC1 || method == FPCC_PCCV);
  const bool counts = phase && c->precision == FPCC_ANALYTIC_AUTO;
  int* d_cnt = nullptr;
  int* h_cnt = nullptr;
  if (counts) {
    void *dp, *hp2;
    if ((rc = dev_buf(c, S_PIPE_CNT, (size_t)nuse * sizeof(int), &dp)) ||
        (rc = pin_buf(c, 6, (size_t)nuse * sizeof(int), &hp2)))
      return rc;
    d_cnt = (int*)dp;
    h_cnt = (int*)hp2;
  }
  if (!c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FPCC_ECUDA, "stream creation failed");
  if (!c->stream3 && cudaStreamCreateWithFlags(&c->stream3, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FPCC_ECUDA, "stream creation failed");
  // pieces of pairs: pair i is ready once rows [0, need[i]) are transformed
  const int cp = std::max(1024, std::min(8192, npairs / 32));
  std::vector<std::pair<int, int>> pieces;   // (first pair, chunk after which it is ready)
  for (int i = 0, k = 0; i < npairs;) {
    while (need[(size_t)i] > R[(size_t)k + 1]) k++;
    int j = i + 1;
    while (j < npairs && j - i < (pieces.empty() ? cp / 4 : cp) && need[(size_t)j] <= R[(size_t)k + 1]) j++;
    pieces.push_back({i, k});
    i = j;
  }
  pieces.push_back({npairs, nch});
  const size_t nev = 2 * (size_t)nch + pieces.size() + 1;
  while (c->pipe_ev.size() < nev) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(FPCC_ECUDA, "event creation failed");
    c->pipe_ev.push_back(e);
  }
  cudaEvent_t* ev_up = c->pipe_ev.data();          // chunk k uploaded
  cudaEvent_t* ev_cnt = ev_up + nch;               // chunk k's gap counts on the host
  cudaEvent_t* ev_pair = ev_cnt + nch;             // piece p computed
  cudaEvent_t ev_upall = ev_pair[pieces.size()];   // every row uploaded
  // the pair list, rewritten onto the device order, goes first on the main stream
  CK(cudaMemcpyAsync(d_p, hps, 2 * (size_t)npairs * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  // the copies follow everything queued on the main stream (buffer allocations included)
  CK(cudaEventRecord(c->ord_ev, c->stream));
  CK(cudaStreamWaitEvent(c->stream2, c->ord_ev, 0));
  CK(cudaStreamWaitEvent(c->stream3, c->ord_ev, 0));
  const size_t xrow = (size_t)N * sizeof(float);
  // uploads of every chunk, in order, each followed by its gap counts
  size_t ri = 0;
  for (int k = 0; k < nch; k++) {
    for (; ri < runs.size() && runs[ri].d0 < R[(size_t)k + 1]; ri++) {
      // a run may cross a chunk boundary: copy the part in this chunk, keep the rest
      Run& u = runs[ri];
      const int len = std::min(u.len, R[(size_t)k + 1] - u.d0);
      CK(cudaMemcpy2DAsync(d_x + (size_t)u.d0 * N, xrow, h_x + (size_t)u.r0 * N, xrow * u.stride, xrow, (size_t)len,
                           cudaMemcpyHostToDevice, c->stream2));
      if (len < u.len) {
        u.d0 += len;
        u.r0 += len * u.stride;
        u.len -= len;
        break;
      }
    }
    CK(cudaEventRecord(ev_up[k], c->stream2));
    if (counts) {
      // the gap counts on the third stream (idle until the downloads), so that
      // the uploads run back to back
      const int r0 = R[(size_t)k], n = R[(size_t)k + 1] - r0;
      CK(cudaStreamWaitEvent(c->stream3, ev_up[k], 0));
      CK(launch_zero_count(d_x + (size_t)r0 * N, N, N, n, d_cnt + r0, c->stream3));
      g_launches++;
      CK(cudaMemcpyAsync(h_cnt + r0, d_cnt + r0, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c->stream3));
      CK(cudaEventRecord(ev_cnt[k], c->stream3));
    }
  }
  // host-to-device and device-to-host copies share the host link, and a
  // download running beside the uploads leaves them a small part of it (the
  // last rows then arrive late and hold up the last pairs): the downloads start
  // once every row is up
  CK(cudaEventRecord(ev_upall, c->stream2));
  CK(cudaStreamWaitEvent(c->stream3, ev_upall, 0));
  size_t pi = 0;
  std::vector<int32_t> f64;
  for (int k = 0; k < nch; k++) {
    const int r0 = R[(size_t)k], n = R[(size_t)k + 1] - r0;
    CK(cudaStreamWaitEvent(c->stream, ev_up[k], 0));
    f64.clear();
    if (counts) {
      CK(cudaEventSynchronize(ev_cnt[k]));
      for (int i = 0; i < n; i++)
        if (h_cnt[r0 + i] >= kZeroSamples) f64.push_back(i);
    } else if (phase && c->precision == FPCC_ANALYTIC_F64) {
      for (int i = 0; i < n; i++) f64.push_back(i);
    }
    if ((rc = fpcc_station_stage_ex(c, method, d_x + (size_t)r0 * N, N, n, N, Ly.Nz, Ly.fmt, FPCC_AMP_F_REG,
                                    (char*)d_st + (size_t)r0 * rowb, Ly.lds, f64.data(), (int)f64.size())))
      return rc;
    if (d_E && (rc = fpcc_energy_stage(c, d_x + (size_t)r0 * N, N, n, N, d_E + (size_t)r0 * Ly.ldE(), Ly.ldE())))
      return rc;
    // the pieces ready after this chunk: compute, then download on the third stream
    for (; pi + 1 < pieces.size() && pieces[pi].second == k; pi++) {
      const int i0 = pieces[pi].first, np = pieces[pi + 1].first - i0;
      if ((rc = fpcc_pair_stage(c, method, d_st, Ly.lds, Ly.fmt, d_p + 2 * (size_t)i0, np, N, Ly.Nz, Ly.lag0,
                                Ly.lag0 + Ly.L - 1, v, d_E, Ly.ldE(), d_y + (size_t)i0 * Ly.L, Ly.L, nullptr)))
        return rc;
      CK(cudaEventRecord(ev_pair[pi], c->stream));
      CK(cudaStreamWaitEvent(c->stream3, ev_pair[pi], 0));
      CK(cudaMemcpyAsync(h_y + (size_t)i0 * Ly.L, d_y + (size_t)i0 * Ly.L, (size_t)np * Ly.L * sizeof(float),
                         cudaMemcpyDeviceToHost, c->stream3));
    }
  }
  CK(cudaStreamSynchronize(c->stream3));
  return 0;
}

// Station stage then pair stage on the context stream.  For the 1-bit methods
// the sign rule depends on the role of the trace (src/FFTapps.c:1037,1042):
// split >= 0 gives rows [0, split) the station-1 rule and the rest the station-2
// rule; split < 0 computes both variants (rows [0,nsta) and [nsta,2 nsta)) and
// expects each pair's station-2 index to point into the second half.
// Station stage(s), then the pair stage.  With h_x (the station windows in host
// memory, one method rule), the windows go up in four row chunks on the second
// stream and the station stage of each chunk starts as soon as its rows have
// arrived.  With h_y (FP32 results wanted in host memory) and enough pairs, the
// pair stage runs in chunks of consecutive pairs and the second stream
// downloads each chunk's rows once its kernels are done, so the download of one
// chunk overlaps the correlation of the next; every kernel is queued before the
// first download, so pageable host memory (whose copies return only when done)
// does not hold back the launches.
int run_device(fpcc_ctx* c, const Layout& Ly, const float* d_x, int nsta, const int32_t* d_pairs, int npairs,
               float v, float* d_y, int64_t* d_num, int split, float* h_y = nullptr, const float* h_x = nullptr) {
  void* d_st = nullptr;
  int rc;
  const int method = Ly.method;
  const bool both = Ly.two_rules && split < 0;
  const int nrows_st = both ? 2 * nsta : nsta;
  if ((rc = dev_buf(c, S_STATION, (size_t)nrows_st * Ly.lds * Ly.esz, &d_st))) return rc;
  char* base = (char*)d_st;
  const size_t rowb = (size_t)Ly.lds * Ly.esz;
  if (Ly.two_rules) {
    const int n1 = both ? nsta : split;
    if (n1 > 0 && (rc = fpcc_station_stage(c, method, d_x, Ly.N, n1, Ly.N, Ly.Nz, Ly.fmt, FPCC_SIGN_GE, base,
                                           Ly.lds)))
      return rc;
    if (both) {
      if ((rc = fpcc_station_stage(c, method, d_x, Ly.N, nsta, Ly.N, Ly.Nz, Ly.fmt, FPCC_SIGN_GT,
                                   base + (size_t)nsta * rowb, Ly.lds)))
        return rc;
    } else if (nsta - split > 0) {
      if ((rc = fpcc_station_stage(c, method, d_x + (size_t)split * Ly.N, Ly.N, nsta - split, Ly.N, Ly.Nz, Ly.fmt,
                                   FPCC_SIGN_GT, base + (size_t)split * rowb, Ly.lds)))
        return rc;
    }
  } else if (h_x) {
    if (!c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess)
      return fail(FPCC_ECUDA, "stream creation failed");
    for (int k = 0; k < 4; k++)
      if (!c->up_ev[k] && cudaEventCreateWithFlags(&c->up_ev[k], cudaEventDisableTiming) != cudaSuccess)
        return fail(FPCC_ECUDA, "event creation failed");
    // the uploads follow everything queued on the main stream (buffer allocations included)
    CK(cudaEventRecord(c->ord_ev, c->stream));
    CK(cudaStreamWaitEvent(c->stream2, c->ord_ev, 0));
    const int per = (nsta + 3) / 4;
    for (int k = 0; k < 4; k++) {
      const int r0 = k * per, n = std::min(per, nsta - r0);
      if (n <= 0) break;
      CK(cudaMemcpyAsync((float*)d_x + (size_t)r0 * Ly.N, h_x + (size_t)r0 * Ly.N, (size_t)n * Ly.N * sizeof(float),
                         cudaMemcpyHostToDevice, c->stream2));
      CK(cudaEventRecord(c->up_ev[k], c->stream2));
      CK(cudaStreamWaitEvent(c->stream, c->up_ev[k], 0));
      if ((rc = fpcc_station_stage(c, method, d_x + (size_t)r0 * Ly.N, Ly.N, n, Ly.N, Ly.Nz, Ly.fmt, FPCC_AMP_F_REG,
                                   base + (size_t)r0 * rowb, Ly.lds)))
        return rc;
    }
  } else {
    if ((rc = fpcc_station_stage(c, method, d_x, Ly.N, nsta, Ly.N, Ly.Nz, Ly.fmt, FPCC_AMP_F_REG, d_st, Ly.lds)))
      return rc;
  }
  double* d_E = nullptr;
  if (method == FPCC_GNCC) {
    void* p = nullptr;
    if ((rc = dev_buf(c, S_ENERGY, (size_t)nsta * Ly.ldE() * sizeof(double), &p))) return rc;
    d_E = (double*)p;
    if ((rc = fpcc_energy_stage(c, d_x, Ly.N, nsta, Ly.N, d_E, Ly.ldE()))) return rc;
  }
  if (!h_y)
    return fpcc_pair_stage(c, method, d_st, Ly.lds, Ly.fmt, d_pairs, npairs, Ly.N, Ly.Nz, Ly.lag0,
                           Ly.lag0 + Ly.L - 1, v, d_E, Ly.ldE(), d_y, Ly.L, d_num);
  // chunks of about 6000 correlations (at most 16): the first download starts
  // after a short first chunk, and the rest overlap the following chunks
  const int nch = (int)std::max<int64_t>(1, std::min<int64_t>(16, npairs / 6000));
  if (nch > 1 && !c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FPCC_ECUDA, "stream creation failed");
  for (int k = 0; k < nch; k++)
    if (!c->chunk_ev[k] && cudaEventCreateWithFlags(&c->chunk_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return fail(FPCC_ECUDA, "event creation failed");
  const int per = (npairs + nch - 1) / nch;
  for (int k = 0; k < nch; k++) {
    const int i0 = k * per, n = std::min(per, npairs - i0);
    if (n <= 0) break;
    if ((rc = fpcc_pair_stage(c, method, d_st, Ly.lds, Ly.fmt, d_pairs + 2 * (size_t)i0, n, Ly.N, Ly.Nz, Ly.lag0,
                              Ly.lag0 + Ly.L - 1, v, d_E, Ly.ldE(), d_y + (size_t)i0 * Ly.L, Ly.L, nullptr)))
      return rc;
    CK(cudaEventRecord(c->chunk_ev[k], c->stream));
  }
  cudaStream_t dl = nch > 1 ? c->stream2 : c->stream;
  for (int k = 0; k < nch; k++) {
    const int i0 = k * per, n = std::min(per, npairs - i0);
    if (n <= 0) break;
    CK(cudaStreamWaitEvent(dl, c->chunk_ev[k], 0));
    CK(cudaMemcpyAsync(h_y + (size_t)i0 * Ly.L, d_y + (size_t)i0 * Ly.L, (size_t)n * Ly.L * sizeof(float),
                       cudaMemcpyDeviceToHost, dl));
  }
  CK(cudaStreamSynchronize(dl));
  return 0;
}

int host_windows(int method, float** y, int64_t** num, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1,
                 int Lag2, float v, int nz_mode, int fmt, bool plain) {
  if (!x1 || !x2 || (!y && !num)) return fail(FPCC_EARG, "null row arrays");
  if (Tr == 0) return 0;
  fpcc_ctx* c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  Layout Ly;
  if ((rc = make_layout(method, (int)N, Lag1, Lag2, nz_mode, fmt, &Ly))) return rc;
  const unsigned nwin = plain ? 1u : Tr;   // windows per launch sequence
  const size_t xbytes = (size_t)2 * nwin * N * sizeof(float);
  const size_t ybytes = (size_t)nwin * Ly.L * (num ? sizeof(int64_t) : sizeof(float));
  void *h_x, *h_y, *d_x, *d_y, *d_pairs;
  if ((rc = pin_buf(c, 0, xbytes, &h_x)) || (rc = pin_buf(c, 1, ybytes, &h_y))) return rc;
  if ((rc = dev_buf(c, S_HOST_X, xbytes, &d_x)) || (rc = dev_buf(c, S_Y, ybytes, &d_y)) ||
      (rc = dev_buf(c, S_PAIRS, (size_t)2 * nwin * sizeof(int32_t), &d_pairs)))
    return rc;
  std::vector<int32_t> pairs(2 * nwin);
  for (unsigned t = 0; t < nwin; t++) { pairs[2 * t] = (int32_t)t; pairs[2 * t + 1] = (int32_t)(nwin + t); }
  CK(cudaMemcpyAsync(d_pairs, pairs.data(), pairs.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  for (unsigned t0 = 0; t0 < Tr; t0 += nwin) {
    float* hx = (float*)h_x;
    for (unsigned t = 0; t < nwin; t++) {
      memcpy(hx + (size_t)t * N, x1[t0 + t], N * sizeof(float));
      memcpy(hx + (size_t)(nwin + t) * N, x2[t0 + t], N * sizeof(float));
    }
    CK(cudaMemcpyAsync(d_x, h_x, xbytes, cudaMemcpyHostToDevice, c->stream));
    if (num) {
      if ((rc = run_device(c, Ly, (const float*)d_x, 2 * nwin, (const int32_t*)d_pairs, nwin, v, nullptr,
                           (int64_t*)d_y, (int)nwin)))
        return rc;
    } else {
      if ((rc = run_device(c, Ly, (const float*)d_x, 2 * nwin, (const int32_t*)d_pairs, nwin, v, (float*)d_y,
                           nullptr, (int)nwin)))
        return rc;
    }
    CK(cudaMemcpyAsync(h_y, d_y, ybytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (unsigned t = 0; t < nwin; t++) {
      if (num) memcpy(num[t0 + t], (int64_t*)h_y + (size_t)t * Ly.L, Ly.L * sizeof(int64_t));
      else memcpy(y[t0 + t], (float*)h_y + (size_t)t * Ly.L, Ly.L * sizeof(float));
    }
  }
  return 0;
}

}  // namespace

extern "C" int fpcc_host_batched(int method, float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1,
                                 int Lag2, float v, int nz_mode, int fmt) {
  return host_windows(method, y, nullptr, x1, x2, N, Tr, Lag1, Lag2, v, nz_mode, fmt, false);
}

extern "C" int fpcc_host_plain(int method, float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1,
                               int Lag2, float v, int nz_mode, int fmt) {
  return host_windows(method, y, nullptr, x1, x2, N, Tr, Lag1, Lag2, v, nz_mode, fmt, true);
}

extern "C" int fpcc_allpairs_host(fpcc_ctx* c, int method, const float* h_x, int nsta, int N, const int32_t* h_pairs,
                                  int npairs, int Lag1, int Lag2, float v, int nz_mode, int fmt, float* h_y) {
  if (!c || !h_x || !h_pairs || !h_y) return fail(FPCC_EARG, "null argument");
  if (nsta < 0 || npairs < 0) return fail(FPCC_EARG, "negative count");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  Layout Ly;
  int rc = make_layout(method, N, Lag1, Lag2, nz_mode, fmt, &Ly);
  if (rc) return rc;
  // pinned buffers and one-rule methods try the first-use path, which checks
  // the row indices as it reads the pair list; every other call checks them here
  const bool first_use = !Ly.two_rules && npairs >= 2048 && is_pinned(h_x) && is_pinned(h_y);
  if (!first_use)
    for (size_t i = 0; i < 2 * (size_t)npairs; i++)
      if (h_pairs[i] < 0 || h_pairs[i] >= nsta) return fail(FPCC_EARG, "pair row index out of range");
  const size_t xbytes = (size_t)nsta * N * sizeof(float);
  const size_t ybytes = (size_t)npairs * Ly.L * sizeof(float);
  const size_t pbytes = (size_t)npairs * 2 * sizeof(int32_t);
  void *d_x, *d_y, *d_p;
  if ((rc = dev_buf(c, S_HOST_X, xbytes, &d_x)) || (rc = dev_buf(c, S_Y, ybytes, &d_y)) ||
      (rc = dev_buf(c, S_PAIRS, pbytes, &d_p)))
    return rc;
  if (Ly.two_rules) {
    // station 2 of each pair reads the station-2-rule variant (second half of the rows)
    CK(cudaMemcpyAsync(d_x, h_x, xbytes, cudaMemcpyHostToDevice, c->stream));
    std::vector<int32_t> hp(h_pairs, h_pairs + 2 * (size_t)npairs);
    for (int i = 0; i < npairs; i++) hp[2 * i + 1] += nsta;
    CK(cudaMemcpyAsync(d_p, hp.data(), pbytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  // one-rule methods with pinned buffers: rows in first-use order when the pair
  // list has that structure (it uploads its own rewritten pair list); otherwise
  // the windows go up in chunks that the station stage consumes as they arrive
  rc = 1;
  if (first_use)
    rc = run_first_use(c, Ly, (float*)d_x, nsta, h_pairs, (int32_t*)d_p, npairs, v, (float*)d_y, h_y, h_x);
  if (rc < 0 || (rc > 1)) return rc;
  if (rc == 1) {
    if (!Ly.two_rules) CK(cudaMemcpyAsync(d_p, h_pairs, pbytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = run_device(c, Ly, (const float*)d_x, nsta, (const int32_t*)d_p, npairs, v, (float*)d_y, nullptr, -1,
                         h_y, Ly.two_rules ? nullptr : h_x)))
      return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

// Drop-in siblings of the reference's per-pair GPU calls (plain form).
extern "C" int pcc2_highlevel(float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1, int Lag2) {
  return host_windows(FPCC_PCC2, y, nullptr, x1, x2, N, Tr, Lag1, Lag2, 2.0f, FPCC_NZ_FAST, FPCC_F32, true);
}
extern "C" int ccgn_highlevel(float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1, int Lag2) {
  return host_windows(FPCC_GNCC, y, nullptr, x1, x2, N, Tr, Lag1, Lag2, 0.0f, FPCC_NZ_FAST, FPCC_F32, true);
}
extern "C" int cc1b_highlevel(float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1, int Lag2) {
  return host_windows(FPCC_CC1B, y, nullptr, x1, x2, N, Tr, Lag1, Lag2, 0.0f, FPCC_NZ_FAST, FPCC_F32, true);
}
extern "C" int cc1b_popcount_highlevel(int64_t** num, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1,
                                       int Lag2) {
  return host_windows(FPCC_CC1B_POPCOUNT, nullptr, num, x1, x2, N, Tr, Lag1, Lag2, 0.0f, FPCC_NZ_FAST, FPCC_F32,
                      true);
}

// ============================================================== wavelet PCC
struct fpcc_wpcc_plan {
  fpcc::WpccSetup su;
  fpcc::WpccPlanDev dev;
  float2* W = nullptr;
  float* a = nullptr;
  int device = 0;
};

namespace {

int wpcc_plan_build(fpcc_ctx* c, const WaveletFamily& wf, int Nz, unsigned N, int lag0, int L, double C, int rule,
                    int filt_conj, fpcc_wpcc_plan* p) {
  int n1, n2;
  if (!large_supported(Nz, &n1, &n2) || !large_supported(Nz / 2, &n1, &n2))
    return fail(FPCC_EUNSUP, "WPCC length Nz=%d is not supported", Nz);
  const unsigned S = wf.S;
  CK(cudaMalloc(&p->W, (size_t)S * Nz * sizeof(float2)));
  CK(cudaMalloc(&p->a, (size_t)S * sizeof(float)));
  std::vector<float> a(S);
  for (unsigned s = 0; s < S; s++) a[s] = (float)(1.0 / (wf.scale[s] * (double)Nz));   // src/FFTapps.c:1217
  CK(cudaMemcpyAsync(p->a, a.data(), S * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  void *T, *stage;
  int rc;
  if ((rc = dev_buf(c, S_LARGE_T, (size_t)S * Nz * sizeof(float2), &T)) ||
      (rc = dev_buf(c, S_WP_STAGE, (size_t)S * Nz * sizeof(float2), &stage)))
    return rc;
  CK(wpcc_filters(wf, Nz, p->W, (float2*)T, (float2*)stage, c->stream));
  g_launches += 2;
  p->dev.N = (int)N;
  p->dev.Nz = Nz;
  p->dev.S = (int)S;
  p->dev.Ls0 = (int)wf.Ls[S - 1];
  p->dev.lag0 = lag0;
  p->dev.L = L;
  p->dev.rule = rule;
  p->dev.filt_conj = filt_conj;
  p->dev.C = (float)C;
  p->dev.d_W = p->W;
  p->dev.d_a = p->a;
  cudaGetDevice(&p->device);
  return 0;
}

int wpcc_station_run(fpcc_ctx* c, const fpcc_wpcc_plan* p, const float* d_x, int64_t ldx, int nrows, void* d_P,
                     int fmt) {
  const int Nz = p->dev.Nz, S = p->dev.S;
  int chunk = (int)(kLargeChunkBytes / ((size_t)S * Nz * sizeof(float2)));
  if (chunk < 1) chunk = 1;
  if (chunk * S > 65535) chunk = 65535 / S;
  if (chunk > nrows) chunk = nrows;
  void *X, *T, *band, *rmax;
  int rc;
  if ((rc = dev_buf(c, S_WP_X, (size_t)chunk * Nz * sizeof(float2), &X)) ||
      (rc = dev_buf(c, S_LARGE_T, (size_t)chunk * S * Nz * sizeof(float2), &T)) ||
      (rc = dev_buf(c, S_WP_BAND, (size_t)chunk * S * Nz * sizeof(float2), &band)) ||
      (rc = dev_buf(c, S_WP_RMAX, (size_t)chunk * S * sizeof(float), &rmax)))
    return rc;
  CK(wpcc_station(p->dev, d_x, ldx, nrows, d_P, fmt, (float2*)X, (float2*)T, (float2*)band, (float*)rmax, chunk,
                  c->stream));
  g_launches += 6 * ((nrows + chunk - 1) / chunk);
  return 0;
}

int wpcc_pairs_run(fpcc_ctx* c, const fpcc_wpcc_plan* p, const void* d_P, int fmt, const int32_t* d_pairs,
                   int npairs, float* d_y, int64_t ldy) {
  const int Nz = p->dev.Nz;
  int chunk = (int)(kLargeChunkBytes / ((size_t)Nz * sizeof(float2)));
  if (chunk < 1) chunk = 1;
  if (chunk > 65535) chunk = 65535;
  if (chunk > npairs) chunk = npairs;
  void *Y, *T;
  int rc;
  if ((rc = dev_buf(c, S_WP_Y, (size_t)chunk * Nz * sizeof(float2), &Y)) ||
      (rc = dev_buf(c, S_LARGE_T, (size_t)chunk * (Nz / 2) * sizeof(float2), &T)))
    return rc;
  CK(wpcc_pairs(p->dev, d_P, fmt, reinterpret_cast<const int2*>(d_pairs), npairs, d_y, ldy, (float2*)Y,
                (float2*)T, chunk, c->stream));
  g_launches += 3 * ((npairs + chunk - 1) / chunk);
  return 0;
}

// x1, x2 rows -> y rows through the WPCC plan (one batched pass over all windows).
int wpcc_host_rows(fpcc_ctx* c, const fpcc_wpcc_plan* p, float** y, float** x1, float** x2, unsigned N,
                   unsigned Tr) {
  const int L = p->dev.L, S = p->dev.S, Nz = p->dev.Nz;
  const size_t xbytes = (size_t)2 * Tr * N * sizeof(float);
  const size_t ybytes = (size_t)Tr * L * sizeof(float);
  void *h_x, *h_y, *d_x, *d_y, *d_pairs, *d_P;
  int rc;
  if ((rc = pin_buf(c, 0, xbytes, &h_x)) || (rc = pin_buf(c, 1, ybytes, &h_y))) return rc;
  if ((rc = dev_buf(c, S_HOST_X, xbytes, &d_x)) || (rc = dev_buf(c, S_Y, ybytes, &d_y)) ||
      (rc = dev_buf(c, S_PAIRS, (size_t)2 * Tr * sizeof(int32_t), &d_pairs)) ||
      (rc = dev_buf(c, S_STATION, (size_t)2 * Tr * S * Nz * sizeof(float2), &d_P)))
    return rc;
  float* hx = (float*)h_x;
  for (unsigned t = 0; t < Tr; t++) {
    memcpy(hx + (size_t)t * N, x1[t], N * sizeof(float));
    memcpy(hx + (size_t)(Tr + t) * N, x2[t], N * sizeof(float));
  }
  std::vector<int32_t> pairs(2 * Tr);
  for (unsigned t = 0; t < Tr; t++) { pairs[2 * t] = (int32_t)t; pairs[2 * t + 1] = (int32_t)(Tr + t); }
  CK(cudaMemcpyAsync(d_x, h_x, xbytes, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_pairs, pairs.data(), pairs.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  if ((rc = wpcc_station_run(c, p, (const float*)d_x, N, 2 * (int)Tr, d_P, FPCC_F32))) return rc;
  if ((rc = wpcc_pairs_run(c, p, d_P, FPCC_F32, (const int32_t*)d_pairs, (int)Tr, (float*)d_y, L))) return rc;
  CK(cudaMemcpyAsync(h_y, d_y, ybytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (unsigned t = 0; t < Tr; t++) memcpy(y[t], (float*)h_y + (size_t)t * L, L * sizeof(float));
  return 0;
}

}  // namespace

extern "C" int fpcc_wpcc_plan_create(fpcc_ctx* c, fpcc_wpcc_plan** out, unsigned N, int Lag1, int Lag2, double pmin,
                                     double pmax, unsigned V, int type, double op1, int rule, int nz_mode) {
  if (!c || !out) return fail(FPCC_EARG, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  fpcc_wpcc_plan* p = new fpcc_wpcc_plan();
  if (wpcc_setup(N, Lag1, Lag2, pmin, pmax, V, type, op1, &p->su) != 0) {
    delete p;
    return fail(FPCC_EARG, "invalid WPCC parameters (lags below N, pmin/pmax > 0, type -1/-2/-3)");
  }
  const int Nz = wpcc_choose_nz(p->su, N, nz_mode);
  if (Nz <= 0) {
    delete p;
    return fail(FPCC_EUNSUP, "no supported WPCC transform length");
  }
  int lag0, L;
  lag_window(Lag1, Lag2, &lag0, &L);
  int rc = wpcc_plan_build(c, p->su.wf, Nz, N, lag0, L, p->su.C, rule, 0, p);
  if (rc) {
    cudaFree(p->W);
    cudaFree(p->a);
    delete p;
    return rc;
  }
  *out = p;
  return 0;
}

extern "C" int fpcc_wpcc_plan_set_band(fpcc_wpcc_plan* p, int s_lo, int s_hi) {
  if (!p) return fail(FPCC_EARG, "null plan");
  const int S = p->dev.S;
  std::vector<float> a(S, 0.0f);
  for (int s = 0; s < S; s++)
    if (s >= s_lo && s < s_hi) a[s] = (float)(1.0 / (p->su.wf.scale.empty() ? 1.0 : p->su.wf.scale[s]) / p->dev.Nz);
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->device);
  const cudaError_t e = cudaMemcpy(p->a, a.data(), S * sizeof(float), cudaMemcpyHostToDevice);
  cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "band weights");
  return 0;
}

extern "C" int fpcc_wpcc_plan_set_lags(fpcc_wpcc_plan* p, int Lag1, int Lag2) {
  if (!p) return fail(FPCC_EARG, "null plan");
  const int N = p->dev.N;
  int rc = check_lags(N, Lag1, Lag2);
  if (rc) return rc;
  const int M = abs(Lag1) > abs(Lag2) ? abs(Lag1) : abs(Lag2);
  bool capped = false;
  for (unsigned s = 0; s < p->su.wf.S; s++) capped |= (p->su.wf.Ls[s] >= p->su.Nz0);
  // exact for any length holding the data, the lags and the longest wavelet; a
  // family whose lengths hit the cap is the reference's only for lags giving
  // the same cap 2^ceil(log2(N+M))
  const unsigned cap = 1u << (unsigned)std::ceil(std::log2((double)(N + M)));
  if (capped ? cap != p->su.Nz0 : N + M + (int)p->su.Ls0 > p->dev.Nz)
    return fail(FPCC_EARG, "lags up to %d do not fit the plan's length Nz=%d", M, p->dev.Nz);
  lag_window(Lag1, Lag2, &p->dev.lag0, &p->dev.L);
  return 0;
}

extern "C" int fpcc_wpcc_plan_info(const fpcc_wpcc_plan* p, int* Nz, int* S, int* L) {
  if (!p) return fail(FPCC_EARG, "null plan");
  if (Nz) *Nz = p->dev.Nz;
  if (S) *S = p->dev.S;
  if (L) *L = p->dev.L;
  return 0;
}

extern "C" int fpcc_wpcc_plan_destroy(fpcc_wpcc_plan* p) {
  if (!p) return 0;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->device);
  cudaDeviceSynchronize();
  cudaFree(p->W);
  cudaFree(p->a);
  cudaSetDevice(cur);
  delete p;
  return 0;
}

extern "C" int fpcc_wpcc_station_stage(fpcc_ctx* c, const fpcc_wpcc_plan* p, const float* d_x, int64_t ldx,
                                       int nrows, void* d_P, int fmt) {
  if (!c || !p) return fail(FPCC_EARG, "null argument");
  if (fmt != FPCC_F32 && fmt != FPCC_F16) return fail(FPCC_EUNSUP, "wavelet spectra are stored in F32 or F16");
  if (nrows <= 0) return 0;
  return wpcc_station_run(c, p, d_x, ldx, nrows, d_P, fmt);
}

extern "C" int fpcc_wpcc_pair_stage(fpcc_ctx* c, const fpcc_wpcc_plan* p, const void* d_P, int fmt,
                                    const int32_t* d_pairs, int npairs, float* d_y, int64_t ldy) {
  if (!c || !p) return fail(FPCC_EARG, "null argument");
  if (fmt != FPCC_F32 && fmt != FPCC_F16) return fail(FPCC_EUNSUP, "wavelet spectra are stored in F32 or F16");
  if (npairs <= 0) return 0;
  return wpcc_pairs_run(c, p, d_P, fmt, d_pairs, npairs, d_y, ldy);
}

extern "C" int fpcc_wpcc_host(float** y, float** x1, float** x2, unsigned N, unsigned Tr, int Lag1, int Lag2,
                              double pmin, double pmax, unsigned V, int type, double op1, int rule, int nz_mode) {
  if (!y || !x1 || !x2) return fail(FPCC_EARG, "null row arrays");
  if (Tr == 0) return 0;
  fpcc_ctx* c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return rc;
  fpcc_wpcc_plan* p = nullptr;
  if ((rc = fpcc_wpcc_plan_create(c, &p, N, Lag1, Lag2, pmin, pmax, V, type, op1, rule, nz_mode))) return rc;
  {
    std::lock_guard<std::mutex> lk(c->mu);
    rc = wpcc_host_rows(c, p, y, x1, x2, N, Tr);
  }
  fpcc_wpcc_plan_destroy(p);
  return rc;
}

// ============================================================== reference GPU boundary
// The four entry points of the reference's src/ccs_cuda.h with its signatures.
namespace {

enum CcSlot { S_CC_AN = 15, S_CC_PH = 17, S_CC_Y = 19, S_CC_ZERO = 21 };

// PCC_v on analytic signals produced concurrently by the caller: windows are
// consumed in groups of 16 (the reference's 16 streams, src/ccs_cuda.cu:570-592)
// on two alternating streams with double-buffered pinned staging, so the copy
// of one group overlaps the kernels of the previous one.
int pcc_from_analytic(float** y, const float2* const* x1, const float2* const* x2, int N, unsigned Tr, float v,
                      int Lag1, int Lag2, sem_t* anok, bool pcc1) {
  if (!y || !x1 || !x2 || N <= 0) return FPCC_ECUDA;
  // lag handling of src/ccs_cuda.cu:544-551
  int L = abs(Lag2 - Lag1 + 1);
  if (Lag2 > N) L -= (Lag2 - N);
  const int l1 = (Lag1 >= -N) ? 0 : -(Lag1 + N);
  if (L <= 0 || Tr == 0) return 0;
  fpcc_ctx* c = nullptr;
  if (default_ctx(&c)) return FPCC_ECUDA;
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return FPCC_ECUDA;
  if (!c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess) return FPCC_ECUDA;
  const unsigned G = 16;
  const size_t xb = (size_t)2 * G * N * sizeof(float2);
  const size_t yb = (size_t)G * L * sizeof(float);
  void *hx[2], *hy[2], *dx[2], *dp[2], *dy[2], *zero, *dpairs;
  for (int k = 0; k < 2; k++) {
    if (pin_buf(c, 2 + k, xb, &hx[k]) || pin_buf(c, 4 + k, yb, &hy[k]) || dev_buf(c, S_CC_AN + k, xb, &dx[k]) ||
        dev_buf(c, S_CC_PH + k, xb, &dp[k]) || dev_buf(c, S_CC_Y + k, yb, &dy[k]))
      return FPCC_ECUDA;
  }
  if (dev_buf(c, S_CC_ZERO, (size_t)2 * G * sizeof(float), &zero) ||
      dev_buf(c, S_PAIRS, (size_t)2 * G * sizeof(int32_t), &dpairs))
    return FPCC_ECUDA;
  std::vector<int32_t> pr(2 * G);
  for (unsigned t = 0; t < G; t++) { pr[2 * t] = (int32_t)t; pr[2 * t + 1] = (int32_t)(G + t); }
  cudaStream_t st[2] = {c->stream, c->stream2};
  if (cudaMemsetAsync(zero, 0, 2 * G * sizeof(float), st[0]) != cudaSuccess ||
      cudaMemcpyAsync(dpairs, pr.data(), pr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st[0]) != cudaSuccess ||
      cudaStreamSynchronize(st[0]) != cudaSuccess)
    return FPCC_ECUDA;
  unsigned pending_base[2] = {0, 0}, pending_n[2] = {0, 0};
  auto drain = [&](int k) -> int {
    if (!pending_n[k]) return 0;
    if (cudaStreamSynchronize(st[k]) != cudaSuccess) return FPCC_ECUDA;
    for (unsigned t = 0; t < pending_n[k]; t++)
      for (int l = l1; l < L; l++) y[pending_base[k] + t][l] = ((float*)hy[k])[(size_t)t * L + l];
    pending_n[k] = 0;
    return 0;
  };
  unsigned grp = 0;
  for (unsigned t0 = 0; t0 < Tr; t0 += G, grp++) {
    const int k = grp & 1;
    if (drain(k)) return FPCC_ECUDA;
    const unsigned n = (Tr - t0) < G ? (Tr - t0) : G;
    float2* h = (float2*)hx[k];
    for (unsigned t = 0; t < n; t++) {
      if (anok) sem_wait(&anok[t0 + t]);   // src/ccs_cuda.cu:575,693
      memcpy(h + (size_t)t * N, x1[t0 + t], (size_t)N * sizeof(float2));
      memcpy(h + (size_t)(G + t) * N, x2[t0 + t], (size_t)N * sizeof(float2));
    }
    if (cudaMemcpyAsync(dx[k], hx[k], xb, cudaMemcpyHostToDevice, st[k]) != cudaSuccess) return FPCC_ECUDA;
    PhaseArgs a{};
    a.in = (const float2*)dx[k]; a.ldin = N; a.nrows = 2 * G; a.N = N; a.rule = AMP_PURE;
    a.rowstat = (const float*)zero; a.fmt = 0; a.out = dp[k]; a.ldo = N;
    if (launch_phase_store(a, st[k]) != cudaSuccess) return FPCC_ECUDA;
    PccvArgs q{};
    q.phase = dp[k]; q.ldp = N; q.half = 0; q.pairs = (const int2*)dpairs; q.npairs = (int)n; q.N = N;
    q.Lag1 = Lag1; q.L = L; q.v = pcc1 ? 1.0f : v; q.norm_gpu = 1; q.y = (float*)dy[k]; q.ldy = L;
    if (launch_pccv(q, st[k]) != cudaSuccess) return FPCC_ECUDA;
    if (cudaMemcpyAsync(hy[k], dy[k], (size_t)n * L * sizeof(float), cudaMemcpyDeviceToHost, st[k]) != cudaSuccess)
      return FPCC_ECUDA;
    g_launches += 2;
    pending_base[k] = t0;
    pending_n[k] = n;
  }
  if (drain(0) || drain(1)) return FPCC_ECUDA;
  return 0;
}

}  // namespace

extern "C" int pcc_highlevel(float** y, float2** x1, float2** x2, int N, unsigned int Tr, float v, int Lag1, int Lag2,
                             sem_t* anok) {
  return pcc_from_analytic(y, x1, x2, N, Tr, v, Lag1, Lag2, anok, false) ? -1 : 0;
}

extern "C" int pcc1_highlevel(float** y, float2** x1, float2** x2, int N, unsigned int Tr, int Lag1, int Lag2,
                              sem_t* anok) {
  return pcc_from_analytic(y, x1, x2, N, Tr, 1.0f, Lag1, Lag2, anok, true) ? -1 : 0;
}

// Raw traces in: analytic signals on the GPU, amplitude threshold 1e-6 of the
// sum of |x|^2 (cuda_AmpNormf2, src/ccs_cuda.cu:493-511), PCC1.  The reference's
// GPU_analytic (src/ccs_cuda.cu:13-30) does not apply the one-sided mask of
// src/FFTapps.c:114-118; this one applies that mask.
extern "C" void pcc1_highlevel2(float** y, float** x1, float** x2, int N, unsigned int Tr, int Lag1, int Lag2) {
  if (!y || !x1 || !x2 || N <= 0 || Tr == 0) return;
  int L = abs(Lag2 - Lag1 + 1);
  if (Lag2 > N) L -= (Lag2 - N);
  const int l1 = (Lag1 >= -N) ? 0 : -(Lag1 + N);
  if (L <= 0) return;
  fpcc_ctx* c = nullptr;
  if (default_ctx(&c)) return;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const size_t xb = (size_t)2 * Tr * N * sizeof(float), yb = (size_t)Tr * L * sizeof(float);
  void *hx, *hy, *dx, *dy, *dp, *dpairs;
  if (pin_buf(c, 0, xb, &hx) || pin_buf(c, 1, yb, &hy) || dev_buf(c, S_HOST_X, xb, &dx) ||
      dev_buf(c, S_Y, yb, &dy) || dev_buf(c, S_STATION, (size_t)2 * Tr * N * sizeof(float2), &dp) ||
      dev_buf(c, S_PAIRS, (size_t)2 * Tr * sizeof(int32_t), &dpairs))
    return;
  float* h = (float*)hx;
  for (unsigned t = 0; t < Tr; t++) {
    memcpy(h + (size_t)t * N, x1[t], N * sizeof(float));
    memcpy(h + (size_t)(Tr + t) * N, x2[t], N * sizeof(float));
  }
  std::vector<int32_t> pr(2 * Tr);
  for (unsigned t = 0; t < Tr; t++) { pr[2 * t] = (int32_t)t; pr[2 * t + 1] = (int32_t)(Tr + t); }
  if (cudaMemcpyAsync(dx, hx, xb, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return;
  if (cudaMemcpyAsync(dpairs, pr.data(), pr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    return;
  const float2* an;
  const float *rmax, *rsum;
  if (analytic_rows(c, (const float*)dx, N, 2 * (int)Tr, N, &an, &rmax, &rsum)) return;
  PhaseArgs a{};
  a.in = an; a.ldin = N; a.nrows = 2 * (int)Tr; a.N = N; a.rule = AMP_SUMTHR; a.rowstat = rsum;
  a.fmt = 0; a.out = dp; a.ldo = N;
  if (launch_phase_store(a, c->stream) != cudaSuccess) return;
  PccvArgs q{};
  q.phase = dp; q.ldp = N; q.pairs = (const int2*)dpairs; q.npairs = (int)Tr; q.N = N; q.Lag1 = Lag1; q.L = L;
  q.v = 1.0f; q.norm_gpu = 1; q.y = (float*)dy; q.ldy = L;
  if (launch_pccv(q, c->stream) != cudaSuccess) return;
  g_launches += 2;
  if (cudaMemcpyAsync(hy, dy, yb, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return;
  for (unsigned t = 0; t < Tr; t++)
    for (int l = l1; l < L; l++) y[t][l] = ((float*)hy)[(size_t)t * L + l];
}

// WPCC with the caller's wavelet family, the GPU path's conventions: bands from
// conj(W_s) (GPU_prod, src/ccs_cuda.cu:874-884) and the threshold normalisation
// on the band maximum (cuda_AmpNormf3, :513-531).
extern "C" int cuda_tspcc2_set_freq(float** y0, float** x01, float** x02, unsigned int N, unsigned int Tr,
                                    unsigned int Nz, const int Lag1, const int Lag2, unsigned int S, double* scale,
                                    double2** wc, unsigned int* Ls, int* center, unsigned int* Down_smp, float C) {
  if (!y0 || !x01 || !x02 || !scale || !wc || !Ls || !center || !Down_smp || S == 0) return -1;
  for (unsigned s = 0; s < S; s++)
    if (Down_smp[s] != 1) return -2;   // src/ccs_cuda.cu:940-941
  WaveletFamily wf;
  wf.S = S;
  wf.scale.assign(scale, scale + S);
  wf.Ls.assign(Ls, Ls + S);
  wf.center.assign(center, center + S);
  wf.taps.resize(S);
  for (unsigned s = 0; s < S; s++) {
    wf.taps[s].resize(Ls[s]);
    for (unsigned n = 0; n < Ls[s]; n++) wf.taps[s][n] = std::complex<double>(wc[s][n].x, wc[s][n].y);
  }
  int lag0, L;
  lag_window(Lag1, Lag2, &lag0, &L);
  fpcc_ctx* c = nullptr;
  if (default_ctx(&c)) return -1;
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return -1;
  fpcc_wpcc_plan p;
  if (wpcc_plan_build(c, wf, (int)Nz, N, lag0, L, (double)C, AMP_THRESH, 1, &p)) {
    cudaFree(p.W);
    cudaFree(p.a);
    return -1;
  }
  const int rc = wpcc_host_rows(c, &p, y0, x01, x02, N, Tr);
  cudaStreamSynchronize(c->stream);
  cudaFree(p.W);
  cudaFree(p.a);
  return rc ? -1 : 0;
}

// ============================================================== stacks over windows
namespace {

// M-point spectra (FFT / M, float2) of the L-periodic CWT kernels of every scale:
// rows [0, S): forward (conjugate taps at offsets c - l), rows [S, 2S): the
// reconstruction (taps at offsets l - c).
int stack_spectra(fpcc_ctx* c, const WaveletFamily& wf, int L, int M, float2** out) {
  const int S = (int)wf.S;
  std::vector<double2> h((size_t)2 * S * M, make_double2(0.0, 0.0));
  for (int s = 0; s < S; s++) {
    double2* f = h.data() + (size_t)s * M;
    double2* r = h.data() + (size_t)(S + s) * M;
    const int cs = wf.center[s];
    for (int l = 0; l < (int)wf.Ls[s]; l++) {
      const std::complex<double> w = wf.taps[s][l];
      // index of offset d in the layout: d mod L placed at [0, L) or, for the
      // negative representative, at M - (L - d mod L)
      auto at = [&](int d) {
        int k = d % L;
        if (k < 0) k += L;
        return k;
      };
      const int kf = at(cs - l), kr = at(l - cs);
      f[kf] = make_double2(f[kf].x + w.real() / M, f[kf].y - w.imag() / M);
      r[kr] = make_double2(r[kr].x + w.real() / M, r[kr].y + w.imag() / M);
    }
    // the L-periodic kernel on M points: values at [0, L) and their copies at
    // M - L + k for k in [1, L) (offsets -(L-1)..-1)
    for (double2* row : {f, r})
      for (int k = 1; k < L; k++) row[M - L + k] = row[k];
  }
  void *A, *B, *spec;
  int rc;
  if ((rc = dev_buf(c, S_STK_A, h.size() * sizeof(double2), &A)) ||
      (rc = dev_buf(c, S_STK_B, h.size() * sizeof(double2), &B)) ||
      (rc = dev_buf(c, S_STK_SPEC, h.size() * sizeof(float2), &spec)))
    return rc;
  CK(cudaMemcpyAsync(A, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  double2* res = nullptr;
  if ((rc = passes64(c, (double2*)A, (double2*)B, M, 2 * S, -1, &res))) return rc;
  CK(launch_multi_convert<float2>(res, (float2*)spec, (int64_t)h.size(), c->stream));
  g_launches++;
  *out = (float2*)spec;
  return 0;
}

}  // namespace

extern "C" int fpcc_stack(fpcc_ctx* c, int mode, const float* d_y, int64_t ldg, int64_t ldj, int K, int L,
                          int ngroups, double nu, double pmin, double pmax, int V, int type, double op1,
                          float* d_out, int64_t ldo) {
  if (!c || !d_y || !d_out) return fail(FPCC_EARG, "null argument");
  if (K <= 0 || L < 2 || ngroups <= 0 || ldo < L || !(nu >= 0) || (K > 1 && ldj < L) ||
      (ngroups > 1 && ldg < L))
    return fail(FPCC_EARG, "stack: K >= 1, L >= 2, groups >= 1, nu >= 0 and strides of at least L are required");
  if (mode < FPCC_STACK_LINEAR || mode > FPCC_STACK_TSPWS) return fail(FPCC_EARG, "unknown stack mode %d", mode);
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int rc;
  if (mode == FPCC_STACK_LINEAR) {
    for (int g0 = 0; g0 < ngroups; g0 += 65535) {
      const int G = std::min(65535, ngroups - g0);
      CK(launch_stack_mean(d_y + (size_t)g0 * ldg, ldg, ldj, K, L, G, d_out + (size_t)g0 * ldo, ldo, c->stream));
      g_launches++;
    }
    return 0;
  }
  const int M = conv_class_len(L);
  if (mode == FPCC_STACK_PWS) {
    // analytic signals of the rows (packed stage of the phase methods, FP32), per chunk of groups
    const int Gc = (int)std::max<int64_t>(1, std::min<int64_t>(65535, ((int64_t)4096) / K));
    for (int g0 = 0; g0 < ngroups; g0 += Gc) {
      const int G = std::min(Gc, ngroups - g0);
      const int n = G * K;
      void* an;
      if ((rc = dev_buf(c, S_STK_AN, (size_t)n * L * sizeof(float2), &an))) return rc;
      std::vector<MultiRow> rows(n);
      for (int r = 0; r < n; r++) {
        rows[r] = MultiRow{};
        rows[r].x = d_y + (size_t)(g0 + r / K) * ldg + (size_t)(r % K) * ldj;
        rows[r].out = (float2*)an + (size_t)r * L;
        rows[r].N = L;
      }
      if ((rc = multi_group<float2>(c, rows, M))) return rc;
      CK(launch_stack_pws((const float2*)an, L, d_y + (size_t)g0 * ldg, ldg, ldj, K, L, G, nu,
                          d_out + (size_t)g0 * ldo, ldo, c->stream));
      g_launches++;
    }
    return 0;
  }
  WaveletFamily wf;
  double cpsi = 0;
  if (stack_family((unsigned)L, pmin, pmax, (unsigned)V, type, op1, &wf, &cpsi))
    return fail(FPCC_EARG, "stack: invalid wavelet parameters (pmin %g, pmax %g, V %d, type %d)", pmin, pmax, V, type);
  const int S = (int)wf.S;
  float2* spec = nullptr;
  if ((rc = stack_spectra(c, wf, L, M, &spec))) return rc;
  // groups per chunk: transform buffers of (G K + G) rows under 256 MB
  const int64_t per_group = (int64_t)(K + 1) * M * (int64_t)sizeof(float2);
  const int Gc = (int)std::max<int64_t>(1, std::min<int64_t>(65535 / (K + 1), ((int64_t)256 << 20) / per_group));
  if ((int64_t)(K + 1) > 65535) return fail(FPCC_EARG, "stack: at most 65534 traces per group");
  for (int g0 = 0; g0 < ngroups; g0 += Gc) {
    const int G = std::min(Gc, ngroups - g0);
    const int rows = G * K + G;
    void *X, *T, *T2, *Y, *Y2, *R;
    if ((rc = dev_buf(c, S_STK_X, (size_t)rows * M * sizeof(float2), &X)) ||
        (rc = dev_buf(c, S_STK_T, (size_t)rows * M * sizeof(float2), &T)) ||
        (rc = dev_buf(c, S_STK_T2, (size_t)rows * M * sizeof(float2), &T2)) ||
        (rc = dev_buf(c, S_STK_Y, (size_t)G * M * sizeof(float2), &Y)) ||
        (rc = dev_buf(c, S_STK_Y2, (size_t)G * M * sizeof(float2), &Y2)) ||
        (rc = dev_buf(c, S_STK_R, (size_t)G * M * sizeof(float2), &R)))
      return rc;
    // spectra of the traces, and of each group's linear stack in rows G K + g
    CK(launch_stack_load(d_y + (size_t)g0 * ldg, ldg, ldj, K, G, L, (float2*)X, M, c->stream));
    float2* xs = nullptr;
    if ((rc = passes(c, (float2*)X, (float2*)T, M, G * K, -1, &xs))) return rc;
    if (xs != (float2*)X) CK(cudaMemcpyAsync(X, xs, (size_t)G * K * M * sizeof(float2), cudaMemcpyDeviceToDevice,
                                             c->stream));
    CK(launch_stack_xlin((float2*)X, K, G, M, c->stream));
    g_launches += 2;
    const bool inblock = spec_supported(M);
    for (int s = 0; s < S; s++) {
      // CWT of every trace and of the linear stacks at scale s: in one block per
      // row when M is on the size menu (only the L outputs leave the block),
      // else a multiply and global radix passes
      float2* W = nullptr;
      int64_t ldw = M;
      if (inblock) {
        CwtRowArgs q{(const float2*)X, rows, M, spec + (size_t)s * M, L, (float2*)T, L};
        CK(launch_cwt_rows(q, c->stream));
        W = (float2*)T;
        ldw = L;
      } else {
        CK(launch_stack_mul((const float2*)X, rows, M, spec + (size_t)s * M, (float2*)T, c->stream));
        if ((rc = passes(c, (float2*)T, (float2*)T2, M, rows, +1, &W))) return rc;
      }
      // weighted linear-stack coefficients, back to the spectrum, times the reconstruction kernel
      CK(launch_stack_coherence(W, ldw, K, G, L, M, nu, (float2*)Y, c->stream));
      float2* Z = nullptr;
      if ((rc = passes(c, (float2*)Y, (float2*)Y2, M, G, -1, &Z))) return rc;
      const float a = (float)(std::log(2.0) / (2 * cpsi * V * wf.scale[s]));
      CK(launch_stack_acc(Z, G, M, spec + (size_t)(S + s) * M, a, s == 0, (float2*)R, c->stream));
      g_launches += 3;
    }
    float2* r = nullptr;
    if ((rc = passes(c, (float2*)R, (float2*)Y, M, G, +1, &r))) return rc;
    CK(launch_stack_real(r, G, L, M, d_out + (size_t)g0 * ldo, ldo, c->stream));
    g_launches++;
  }
  return 0;
}
