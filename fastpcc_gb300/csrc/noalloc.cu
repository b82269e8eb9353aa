// PCC2 entry point that allocates no memory.
//
// Some callers of this library cannot call cudaMalloc: a host that hands the
// whole of HBM to its own pool allocator up front (so a cudaMalloc from a plugin
// fails, or steals memory the pool has promised elsewhere), a plugin framework
// whose rules forbid device allocation by plugins, and latency-critical loops
// where cudaMalloc/cudaFree would synchronise the device and stall the other
// streams.  For them, fpcc_pcc2_noalloc runs the PCC2 station and pair stages on
// device buffers the caller owns, and keeps every intermediate (twiddle table,
// analytic signals, phase spectra, pair list) in one file-scope device array of
// kNoAllocScratchBytes.  Every GPU that loads the library holds that array until
// the process exits.
//
// The array's host-side name is only a stand-in for the symbol: every call asks
// the runtime for the device address in the current context with
// cudaGetSymbolAddress (which allocates nothing), so the address stays right
// after cudaDeviceReset or when another context is current.  The first call on a
// device loads the library's device code there, so it should come before any
// stream capture.  All calls share the array and it keeps the previous call's
// contents; this entry point writes every element it later reads, so nothing
// needs clearing, but two calls whose work overlaps on the GPU (on different
// streams, or from different host threads) race on the array and must be
// serialised by the caller.
#include <cmath>
#include <cstdio>

#include "../../include/fastpcc_gb300.h"
#include "engine.h"
#include "kernels.cuh"

namespace fpcc {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;   // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

thread_local char g_msg[256];

int fail_na(int code, const char* msg) {
  snprintf(g_msg, sizeof g_msg, "%s", msg);
  return code;
}

__global__ void k_twiddle_table(float2* tw, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    tw[t] = make_float2((float)c, (float)s);
  }
}

__global__ void k_pair_list(int2* pairs, int tr) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tr; t += gridDim.x * blockDim.x)
    pairs[t] = make_int2(t, tr + t);
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) return fail_na(FPCC_ECUDA, "cudaGetSymbolAddress of the scratch array failed");
  *out = p;
  return 0;
}

// Analytic signal of `rows` real rows into bufs[*cur] (generic passes), as the
// allocating path does, with the caller's twiddle table.
cudaError_t analytic(const float* x, int64_t ldx, int rows, int N, const FftPlan& p, const float2* tw, float2* A,
                     float2* B, float* st, cudaStream_t s, float2** result) {
  float2* bufs[2] = {A, B};
  int cur = 0;
  cudaError_t e;
  for (int dir = -1; dir <= 1; dir += 2) {
    int Ns = 1;
    for (int i = 0; i < p.npass; i++) {
      const bool first = (dir < 0 && i == 0);
      float2* dst = first ? bufs[0] : bufs[cur ^ 1];
      const void* src = first ? (const void*)x : (const void*)bufs[cur];
      if ((e = launch_gpass(p.rad[i], dir, src, first, ldx, dst, N, N, Ns, rows, tw, s)) != cudaSuccess) return e;
      cur = first ? 0 : (cur ^ 1);
      Ns *= p.rad[i];
    }
    if (dir < 0 && (e = launch_analytic_mask(bufs[cur], N, N, rows, s)) != cudaSuccess) return e;
  }
  if ((e = launch_rowstats(bufs[cur], N, N, rows, st, st + rows, s)) != cudaSuccess) return e;
  *result = bufs[cur];
  return cudaSuccess;
}

}  // namespace
}  // namespace fpcc

using namespace fpcc;

extern "C" size_t fpcc_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" const char* fpcc_noalloc_last_error(void) { return g_msg; }

extern "C" int fpcc_pcc2_noalloc(const float* d_x1, const float* d_x2, int64_t ldx, int N, int Tr, int Lag1,
                                 int Lag2, float* d_y, int64_t ldy, void* stream) {
  g_msg[0] = '\0';
  if (!d_x1 || !d_x2 || !d_y) return fail_na(FPCC_EARG, "null device pointer");
  if (N <= 0 || Tr <= 0 || ldx < N) return fail_na(FPCC_EARG, "N, Tr must be positive and ldx >= N");
  const int M = abs(Lag1) > abs(Lag2) ? abs(Lag1) : abs(Lag2);
  if (M >= N) return fail_na(FPCC_EARG, "|lag| must be below N");
  const int L = abs(Lag2 - Lag1) + 1;
  const int lag0 = Lag1 < Lag2 ? Lag1 : Lag2;
  if (ldy < L) return fail_na(FPCC_EARG, "ldy must be at least the number of lags");
  const int Nz = choose_nz(N, M, 1);
  if (Nz <= 0 || !spec_supported(Nz) || !pair_supported(Nz))
    return fail_na(FPCC_EUNSUP, "no in-block correlation length for this N and lag window");
  FftPlan p;
  if (!make_plan(N, &p)) return fail_na(FPCC_EUNSUP, "N must be 2,3,5-smooth");
  // scratch layout: twiddles | row stats | analytic A | analytic B | spectra | pairs
  const size_t b_tw = align256((size_t)N * sizeof(float2));
  const size_t b_st = align256((size_t)4 * Tr * sizeof(float));
  const size_t b_an = align256((size_t)Tr * N * sizeof(float2));
  const size_t b_sp = align256((size_t)2 * Tr * Nz * sizeof(float2));
  const size_t b_pr = align256((size_t)Tr * sizeof(int2));
  const size_t need = b_tw + b_st + 2 * b_an + b_sp + b_pr;
  if (need > kNoAllocScratchBytes) {
    snprintf(g_msg, sizeof g_msg,
             "fpcc_pcc2_noalloc: this call needs %zu bytes of scratch but the fixed array holds %zu; "
             "use fewer windows per call (Tr) or the allocating entry points",
             need, kNoAllocScratchBytes);
    return FPCC_EARG;
  }
  // An error left by the caller's earlier work stays with the caller (peek, do
  // not clear); this call then reports that it did not run.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    snprintf(g_msg, sizeof g_msg, "fpcc_pcc2_noalloc: not run, a CUDA error is pending from earlier work: %s",
             cudaGetErrorString(e));
    return FPCC_ECUDA;
  }
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  char* s = (char*)base;
  float2* tw = (float2*)s;
  float* st = (float*)(s + b_tw);
  float2* A = (float2*)(s + b_tw + b_st);
  float2* B = (float2*)(s + b_tw + b_st + b_an);
  float2* spec = (float2*)(s + b_tw + b_st + 2 * b_an);
  int2* pairs = (int2*)(s + b_tw + b_st + 2 * b_an + b_sp);
  cudaStream_t cs = (cudaStream_t)stream;
  k_twiddle_table<<<(N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024, 256, 0, cs>>>(tw, N);
  k_pair_list<<<(Tr + 255) / 256, 256, 0, cs>>>(pairs, Tr);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail_na(FPCC_ECUDA, cudaGetErrorString(e));
  // station stage for station 1 (rows 0..Tr-1) and station 2 (rows Tr..2Tr-1)
  for (int side = 0; side < 2; side++) {
    const float* x = side ? d_x2 : d_x1;
    float2* an = nullptr;
    float* rs = st + 2 * Tr * side;
    if ((e = analytic(x, ldx, Tr, N, p, tw, A, B, rs, cs, &an)) != cudaSuccess)
      return fail_na(FPCC_ECUDA, cudaGetErrorString(e));
    SpecArgs a{};
    a.in = an;
    a.ldin = N;
    a.nrows = Tr;
    a.N = N;
    a.Nz = Nz;
    a.mode = SPEC_PHASE;
    a.rule = AMP_F_REG;
    a.rowstat = rs;
    a.fmt = SPEC_F32;
    a.out = spec + (size_t)side * Tr * Nz;
    a.ldo = Nz;
    if ((e = launch_spec(a, cs)) != cudaSuccess) return fail_na(FPCC_ECUDA, cudaGetErrorString(e));
  }
  PairArgs q{};
  q.spec = spec;
  q.ldspec = Nz;
  q.fmt = SPEC_F32;
  q.pairs = pairs;
  q.npairs = Tr;
  q.Nz = Nz;
  q.lag0 = lag0;
  q.L = L;
  q.scale = 1.0f / ((float)Nz * (float)N);
  q.y = d_y;
  q.ldy = ldy;
  q.norm = 0;
  q.N = N;
  if ((e = launch_pairs(q, cs)) != cudaSuccess) return fail_na(FPCC_ECUDA, cudaGetErrorString(e));
  return 0;
}
