// Serving loop: continuous batching of correlation requests over station
// products kept resident in HBM.
//
// Requests (method, station pair, window, lag window) arrive from any host
// thread.  A worker thread repeatedly takes everything pending (up to max_batch
// requests), groups it — by (method, padded length, power) where the pair
// kernel takes per-correlation descriptors (window lengths and lag windows then
// differ freely inside one launch), else by (method, window length, padded
// length, lag window) — computes the station products the group lacks
// (uploading raw windows first) and launches one pair stage per group.  While a batch's kernels and
// output copy run, the worker is already forming the next batch: requests that
// arrive meanwhile join it.  Completion is detected from CUDA events; the
// worker copies each result into the caller's buffer and records its latency.
//
// Device memory: raw windows and station products live in slabs (one per
// product class) whose rows are recycled least-recently-used first; the total
// never exceeds the HBM budget given at creation.  Rows used by a batch in
// flight are never evicted.  Each result depends only on its own request (the
// same kernels and padded length whatever the batch holds), so a result is the
// same alone and in any mix.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/fastpcc_gb300.h"
#include "arena.h"
#include "engine.h"
#include "kernels.cuh"
#include "large.cuh"
#include "serve.h"
#include "wavelet.h"
#include "wpcc.h"

namespace fpcc {

struct Server;

// Makes a freshly created context allocate from `pool` (which it does not own).
int ctx_share_pool(fpcc_ctx* c, cudaMemPool_t pool);
void set_last_error(const char* msg);

namespace {
// A failed CUDA call of the server itself: status FPCC_ECUDA with a message.
// FPCC_ENOMEM with a message naming what could not be had.
int no_mem(const char* what) {
  set_last_error(what);
  return FPCC_ENOMEM;
}

int cuda_err(cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof buf, "server: %s: %s", what, cudaGetErrorString(e));
  set_last_error(buf);
  return FPCC_ECUDA;
}
}  // namespace

namespace {

using Clock = std::chrono::steady_clock;

__global__ void k_copy_rows(const char* __restrict__ src, int64_t lds, const int* __restrict__ sidx, char* __restrict__ dst,
                            int64_t ldd, const int* __restrict__ didx, int64_t row_bytes) {
  const int r = blockIdx.y;
  const char* s = src + (int64_t)(sidx ? sidx[r] : r) * lds;
  char* d = dst + (int64_t)(didx ? didx[r] : r) * ldd;
  const int64_t n16 = row_bytes / 16;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    reinterpret_cast<int4*>(d)[i] = reinterpret_cast<const int4*>(s)[i];
  const int64_t tail = row_bytes - n16 * 16;
  if (blockIdx.x == 0 && threadIdx.x < tail) d[n16 * 16 + threadIdx.x] = s[n16 * 16 + threadIdx.x];
}

// rows of row_bytes (multiple of 16 for the vector path; strides multiples of 16)
cudaError_t copy_rows(const void* src, int64_t lds, const int* sidx, void* dst, int64_t ldd, const int* didx, int n,
                      int64_t row_bytes, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int gx = (int)std::min<int64_t>((row_bytes / 16 + 255) / 256, 64);
  if (gx < 1) gx = 1;
  k_copy_rows<<<dim3(gx, n), 256, 0, st>>>((const char*)src, lds, sidx, (char*)dst, ldd, didx, row_bytes);
  return cudaGetLastError();
}

// Row copies with their own source, destination and length (16-byte aligned).
struct RowCopy {
  const char* src;
  char* dst;
  int64_t bytes;
};

__global__ void k_scatter_rows(const RowCopy* __restrict__ rc) {
  const RowCopy r = rc[blockIdx.y];
  const int64_t n16 = r.bytes / 16;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    reinterpret_cast<int4*>(r.dst)[i] = reinterpret_cast<const int4*>(r.src)[i];
}

// A slab of equal rows with least-recently-used recycling.
struct Slab {
  void* base = nullptr;
  int64_t row_bytes = 0;
  int cap = 0;
  std::vector<int64_t> key_of;     // row -> key (-1 free)
  std::vector<int> pin;            // in-flight references
  std::list<int> lru;              // front = most recent
  std::vector<std::list<int>::iterator> pos;
  std::unordered_map<int64_t, int> row_of;
  uint64_t last_use = 0;           // server tick of the last lookup or claim
};

struct Product {  // identifies a product class
  int kind;       // 0 raw window, 1 phase spectrum, 2 real half spectrum, 3 sign half spectrum (GE),
                  // 4 sign half spectrum (GT), 5 energies, 6 phase signal, 7 bits GE, 8 bits GT,
                  // 9 wavelet per-scale phase spectra (S x Nz)
  int N, Nz, fmt;
  int aux = 0;    // kind 9: the wavelet length cap of the family
  int S = 0;      // kind 9: scales
  bool operator<(const Product& o) const {
    return std::tie(kind, N, Nz, fmt, aux) < std::tie(o.kind, o.N, o.Nz, o.fmt, o.aux);
  }
};

struct Req {
  int64_t id;
  fpcc_request r;
  Clock::time_point t_submit;
  int N = 0, Nz = 0, lag0 = 0, L = 0;
  int aux = 0;    // WPCC: wavelet length cap
  int f64 = 0;    // bit 0 / bit 1: the station-1 / station-2 window has enough zero
                  // samples for an FP64 analytic signal (noted at submission)
};

struct InFlight {
  cudaEvent_t done = nullptr;
  std::vector<Req> reqs;
  std::vector<int64_t> out_off;    // offset of each request's output in the pinned buffer (floats or int64)
  void* h_out = nullptr;           // pinned result buffer
  void* d_out = nullptr;           // device results of the batch (group outputs at their offsets)
  size_t h_bytes = 0;
  char* h_up = nullptr;            // pinned upload staging (index arrays), bump-allocated
  size_t up_bytes = 0, up_used = 0;
  std::vector<std::pair<char*, size_t>> up_full;   // staging blocks this batch has filled
  Server* srv = nullptr;
  std::vector<std::pair<char*, size_t>> out_ranges;  // registered result ranges (snapshot at batch start)
  std::vector<char> direct;        // per request: result copied straight into the caller's buffer
  std::vector<std::pair<Slab*, int>> pinned_rows;
  int err = 0;
  std::string err_msg;             // the worker's message for err
};

void* pinned_get(Server* s, size_t bytes, size_t* got);

// Copy a small host array into the batch's pinned staging and queue its upload.
// A batch whose uploads outgrow its staging block (each upload starts on a
// 256-byte boundary, so many small groups can exceed the estimate) continues in
// another pinned block; all of them return to the pool with the batch.
cudaError_t upload(InFlight& fl, void* dst, const void* src, size_t bytes, cudaStream_t st) {
  size_t off = (fl.up_used + 255) & ~size_t(255);
  if (off + bytes > fl.up_bytes) {
    size_t got = 0;
    char* p = (char*)pinned_get(fl.srv, std::max(bytes, fl.up_bytes), &got);
    if (!p) return cudaErrorMemoryAllocation;
    if (fl.h_up) fl.up_full.push_back({fl.h_up, fl.up_bytes});
    fl.h_up = p;
    fl.up_bytes = got;
    off = 0;
  }
  memcpy(fl.h_up + off, src, bytes);
  fl.up_used = off + bytes;
  return cudaMemcpyAsync(dst, fl.h_up + off, bytes, cudaMemcpyHostToDevice, st);
}

}  // namespace

struct WaveletCfg {
  bool set = false;
  double pmin = 0, pmax = 0, op1 = 0;
  unsigned V = 0;
  int type = -1, rule = FPCC_AMP_D_REG, S = 0;
};

// A lane: a context of its own (stream, scratch, caches).  Station stages of
// independent product classes run on the lanes in turn, so that the many small
// per-length stages of a batch with uneven windows overlap on the GPU instead of
// following one another on one stream.
struct Lane {
  fpcc_ctx* ctx = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  bool dirty = false;                   // work queued since the last join
  void* d_tmp = nullptr; size_t n_tmp = 0;
  void* d_idx = nullptr; size_t n_idx = 0;
};
constexpr int kLanes = 4;

struct Server {
  int device = 0;
  size_t budget = 0, used = 0;
  int max_batch = 4096;
  int fmt = FPCC_F32;                  // storage of phase spectra and phase signals
  int nz_mode = FPCC_NZ_FAST;          // padded-length rule of FFT requests
  WaveletCfg wav;
  std::map<std::pair<int, int>, std::pair<int, int>> wsetup;   // (N, M) -> (Nz, length cap)   [mu]
  std::map<std::tuple<int, int, int>, fpcc_wpcc_plan*> wplans;  // (N, Nz, cap)   [worker]
  cudaStream_t st = nullptr;
  fpcc_ctx* ctx = nullptr;
  std::vector<Lane> lanes;
  Lane dlane;                           // pair stages of direct-sum groups, started early
  int next_lane = 0;
  cudaEvent_t main_ev = nullptr;        // marks the server's stream for the lanes
  // results go down on their own stream, so that one group's (and batch's)
  // download overlaps the next pair stages; out_ev mark finished pair stages
  cudaStream_t st_out = nullptr;
  std::vector<cudaEvent_t> out_ev;
  size_t out_used = 0;
  uint64_t lane_seq = 0;                // lane work items queued so far
  std::vector<int>* lane_rec = nullptr; // when set, lanes given work are noted here
  std::vector<cudaEvent_t> ev_pool;     // marks of lane progress for the pair stages
  size_t ev_used = 0;                   // of ev_pool, in the batch being formed
  const std::vector<cudaEvent_t>* pair_waits = nullptr;   // what the next pair stage waits for
  uint64_t pair_seq = 0;                // lane_seq when the group's pair phase began
  // device memory of slabs and scratch: a pool of the server's own whose freed
  // blocks stay mapped, allocated and freed in the order of the server's stream,
  // so growing a slab or releasing one needs no device synchronisation
  cudaMemPool_t pool = nullptr;
  // small slabs are carved from larger pool blocks (chunks), so that a batch
  // with many product classes (every window its own length) makes a few pool
  // allocations instead of one per class; see slab_alloc
  ChunkArena chunks{256};
  size_t chunk_bytes = 0;
  // host copies of registered windows
  std::mutex mu;
  std::condition_variable cv, cv_done;
  struct Window {
    float* x;      // pinned samples
    int N;
    int zeros;     // zero samples (such windows get FP64 analytic signals)
    int chunk;     // the pinned arena chunk holding x
  };
  std::map<std::pair<int, int>, Window> windows;
  std::vector<char*> arena;                                       // pinned chunks holding the windows
  size_t arena_left = 0;
  char* arena_ptr = nullptr;
  std::deque<Req> pending;
  std::vector<int> status;        // by request id (ids count up from 0): 0 pending, 1 done, <0 error
  int64_t next_id = 0;
  bool stop = false;
  std::thread worker;
  std::vector<std::thread> completers;
  std::mutex mu_c;
  std::condition_variable cv_c;
  std::deque<InFlight*> launched;     // worker -> completers
  std::deque<InFlight*> retired;      // completers -> worker
  int in_flight = 0;                  // launched, not yet retired by the worker
  // device state (worker thread only)
  std::map<Product, Slab> slabs;
  std::deque<InFlight> inflight;
  // scratch (worker only)
  void* d_tmp_x = nullptr; size_t n_tmp_x = 0;
  void* d_tmp_p = nullptr; size_t n_tmp_p = 0;
  void* d_idx = nullptr; size_t n_idx = 0;
  void* d_y = nullptr; size_t n_y = 0;
  void* d_pl = nullptr; size_t n_pl = 0;
  void* d_desc = nullptr; size_t n_desc = 0;
  std::vector<void*> pinned_pool;
  // host ranges that results may be copied into directly: (base, bytes, registered by the server)   [mu]
  std::vector<std::tuple<char*, size_t, bool>> out_ranges;
  // stats
  std::vector<double> lat_ms;
  int64_t completed = 0, batches = 0, station_rows = 0, pair_stages = 0;
  std::atomic<int64_t> worker_ns{0}, deliver_ns{0};   // host time forming batches / completing them
  double busy_s = 0;
  int last_error = 0;
  std::string err_msg;                // message of last_error   [mu]
};

namespace {

std::atomic<uint64_t> g_tick{0};   // recency clock of slab use

int64_t wkey(int sta, int win) { return ((int64_t)sta << 32) | (uint32_t)win; }

size_t product_row_bytes(const Product& p) {
  switch (p.kind) {
    case 0: return (size_t)p.N * 4;
    case 1: return p.fmt == FPCC_I16 ? 16 + (size_t)p.Nz * 4 : (size_t)p.Nz * (p.fmt ? 4 : 8);
    case 2: case 3: case 4: return (size_t)(p.Nz / 2 + 1) * 8;
    case 5: return (size_t)(p.N + 1) * 16;   // FP64 prefix sums + the normalisation tables
    case 6: return (size_t)p.N * (p.fmt ? 4 : 8);
    case 9: return (size_t)p.S * p.Nz * (p.fmt ? 4 : 8);
    default: return (size_t)((p.N + 31) / 32) * 4;
  }
}

int64_t round16(int64_t b) { return (b + 15) & ~int64_t(15); }

void* dalloc(Server* s, size_t bytes) {
  void* p = nullptr;
  if (cudaMallocFromPoolAsync(&p, bytes, s->pool, s->st) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void dfree(Server* s, void* p) {
  if (p) cudaFreeAsync(p, s->st);
}

// Lane work starts after everything queued on the server's stream so far (raw
// window uploads, slab copies and frees), and the server's stream waits for all
// lane work queued so far before it touches slab memory again (lanes_join):
// before a pair stage, and before a slab is copied or freed.
Lane& lane_at(Server* s, int k) {
  Lane& l = s->lanes[(size_t)k];
  cudaEventRecord(s->main_ev, s->st);
  cudaStreamWaitEvent(l.st, s->main_ev, 0);
  l.dirty = true;
  s->lane_seq++;
  if (s->lane_rec) s->lane_rec->push_back(k);
  return l;
}

// Per-length stages go round the lanes.
Lane& lane_begin(Server* s) { return lane_at(s, s->next_lane++ % (int)s->lanes.size()); }

// Events marking, on each lane in `used`, the work queued so far (appended to out).
void lane_marks(Server* s, std::vector<int>& used, std::vector<cudaEvent_t>& out) {
  std::sort(used.begin(), used.end());
  used.erase(std::unique(used.begin(), used.end()), used.end());
  for (int k : used) {
    if (s->ev_used == s->ev_pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        out.clear();   // no event: the pair stage waits for every lane instead
        out.push_back(nullptr);
        used.clear();
        return;
      }
      s->ev_pool.push_back(e);
    }
    cudaEvent_t e = s->ev_pool[s->ev_used++];
    cudaEventRecord(e, s->lanes[(size_t)k].st);
    out.push_back(e);
  }
  used.clear();
}

void lanes_join(Server* s) {
  for (auto& l : s->lanes)
    if (l.dirty) {
      cudaEventRecord(l.ev, l.st);
      cudaStreamWaitEvent(s->st, l.ev, 0);
      l.dirty = false;
    }
  if (s->dlane.dirty) {
    cudaEventRecord(s->dlane.ev, s->dlane.st);
    cudaStreamWaitEvent(s->st, s->dlane.ev, 0);
    s->dlane.dirty = false;
  }
}

// Before a pair stage: the server's stream waits for the lane work that made the
// group's products (all lane work when the marks are missing, or when the pair
// phase itself queued lane work).
void pair_join(Server* s) {
  const std::vector<cudaEvent_t>* w = s->pair_waits;
  if (!w || s->lane_seq != s->pair_seq || std::find(w->begin(), w->end(), nullptr) != w->end()) {
    lanes_join(s);
    return;
  }
  for (cudaEvent_t e : *w) cudaStreamWaitEvent(s->st, e, 0);
}

// Scratch of a lane, allocated and freed in its own stream's order.
void* lane_buf(Server* s, Lane& l, void** p, size_t* n, size_t need) {
  if (*n < need) {
    if (*p) cudaFreeAsync(*p, l.st);
    *p = nullptr;
    *n = 0;
    const size_t nn = need + need / 2;
    if (cudaMallocFromPoolAsync(p, nn, s->pool, l.st) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return nullptr;
    }
    *n = nn;
  }
  return *p;
}

// Slab memory.  Blocks up to a quarter of a chunk come first-fit from the
// chunks (256-byte granules, `ChunkArena`); larger ones straight from the pool.
// Every kernel and copy that touches slab memory runs on the server's stream or
// on a lane joined to it before the free, so a range freed here may be handed
// out again at once: its next user is queued after every earlier reader, the
// ordering cudaFreeAsync gives on one stream.
void* slab_alloc(Server* s, size_t bytes) {
  if (s->chunks.round(bytes) > s->chunk_bytes / 4) return dalloc(s, bytes);
  if (void* p = s->chunks.take(bytes)) return p;
  void* base = dalloc(s, s->chunk_bytes);
  if (!base) return nullptr;
  return s->chunks.add_chunk(base, s->chunk_bytes, bytes);
}

void slab_free(Server* s, void* p, size_t bytes) {
  if (!p) return;
  lanes_join(s);
  bool found = false;
  void* empty = s->chunks.give(p, bytes, &found);
  if (!found) dfree(s, p);
  else if (empty) dfree(s, empty);
}

// Frees the least recently used slab (other than `keep`) none of whose rows a
// batch in flight holds; its products are recomputed when next needed.
bool release_idle_slab(Server* s, const Slab* keep) {
  Slab* victim = nullptr;
  for (auto& kv : s->slabs) {
    Slab& c = kv.second;
    if (&c == keep || !c.base) continue;
    bool busy = false;
    for (int r = 0; r < c.cap && !busy; r++) busy = c.pin[r] != 0;
    if (busy) continue;
    if (!victim || c.last_use < victim->last_use) victim = &c;
  }
  if (!victim) return false;
  slab_free(s, victim->base, (size_t)victim->cap * victim->row_bytes);
  s->used -= (size_t)victim->cap * victim->row_bytes;
  victim->base = nullptr;
  victim->cap = 0;
  victim->key_of.clear();
  victim->pin.clear();
  victim->lru.clear();
  victim->pos.clear();
  victim->row_of.clear();
  return true;
}

bool grow(Server* s, Slab& sl, int need_rows) {
  if (sl.cap >= need_rows) return true;
  // start at what is needed (at least 1 MB of rows, at most 64 rows), then double
  const int64_t init = std::max<int64_t>(1, std::min<int64_t>(64, ((int64_t)1 << 20) / sl.row_bytes));
  int ncap = std::max(need_rows, sl.cap ? sl.cap * 2 : (int)init);
  // over budget: grow only to what is needed now, then release idle slabs
  while (s->used + (size_t)(ncap - sl.cap) * sl.row_bytes > s->budget) {
    if (ncap > need_rows) { ncap = need_rows; continue; }
    if (!release_idle_slab(s, &sl)) return false;
  }
  const size_t add = (size_t)(ncap - sl.cap) * sl.row_bytes;
  void* nb = slab_alloc(s, (size_t)ncap * sl.row_bytes);
  if (!nb) return false;
  if (sl.base) {
    // queued kernels that read the old rows run before the copy and the free
    lanes_join(s);
    cudaMemcpyAsync(nb, sl.base, (size_t)sl.cap * sl.row_bytes, cudaMemcpyDeviceToDevice, s->st);
    slab_free(s, sl.base, (size_t)sl.cap * sl.row_bytes);
  }
  sl.base = nb;
  sl.key_of.resize(ncap, -1);
  sl.pin.resize(ncap, 0);
  sl.pos.resize(ncap);
  // new rows at the least-recently-used end, the lowest last, so that claims
  // (taken from that end) come out ascending and a batch's new products are
  // usually one contiguous run of rows
  for (int r = ncap - 1; r >= sl.cap; r--) {
    sl.lru.push_back(r);
    sl.pos[r] = std::prev(sl.lru.end());
  }
  sl.cap = ncap;
  s->used += add;
  return true;
}

Slab& slab_of(Server* s, const Product& p) {
  Slab& sl = s->slabs[p];
  if (!sl.row_bytes) sl.row_bytes = round16((int64_t)product_row_bytes(p));
  return sl;
}

void touch(Slab& sl, int r) {
  sl.lru.splice(sl.lru.begin(), sl.lru, sl.pos[r]);   // moves the node: no allocation, iterator stays valid
}

// Row holding `key`, or -1.
int find_row(Slab& sl, int64_t key) {
  if (sl.base) sl.last_use = ++g_tick;
  auto it = sl.row_of.find(key);
  if (it == sl.row_of.end()) return -1;
  touch(sl, it->second);
  return it->second;
}

void wait_one_retired(Server* s);

// A free or least-recently-used unpinned row for `key` (grows the slab first).
// When every row is held by batches in flight, waits for them to finish
// (admission by memory): only rows of the batch being built can then remain.
int claim_row(Server* s, Slab& sl, int64_t key, int rows_needed_now) {
  sl.last_use = ++g_tick;
  for (;;) {
    // room first (growing may release idle product classes), then the least recently used free row
    if ((int)sl.row_of.size() + rows_needed_now > sl.cap)
      grow(s, sl, std::max(sl.cap * 2, (int)sl.row_of.size() + rows_needed_now));
    for (auto it = sl.lru.rbegin(); it != sl.lru.rend(); ++it) {
      const int r = *it;
      if (sl.pin[r]) continue;
      if (sl.key_of[r] >= 0) sl.row_of.erase(sl.key_of[r]);
      sl.key_of[r] = key;
      sl.row_of[key] = r;
      touch(sl, r);
      return r;
    }
    if (s->in_flight == 0) return -1;
    wait_one_retired(s);
  }
}

// Scratch buffer of at least `need` bytes, grown by half again at least when
// it grows; the old buffer is freed in stream order after the work queued on it.
void* dbuf(Server* s, void** p, size_t* n, size_t need) {
  if (*n < need) {
    const size_t nn = std::max(need, *n + *n / 2);
    if (*p) dfree(s, *p);
    *n = 0;
    if (!(*p = dalloc(s, nn))) return nullptr;
    *n = nn;
  }
  return *p;
}

}  // namespace

// ---------------------------------------------------------------- batch execution
namespace {

// Product rows of a group's requests, found by its products pass and kept
// (pinned) for its pair pass, so that each request's rows are looked up once.
struct GroupRows {
  bool ok = false;
  std::vector<int> r1, r2, e1, e2;
};

struct GroupKey {
  int method, N, Nz, lag0, L, fmt;
  float v;
  int aux;      // WPCC: wavelet length cap
  bool operator<(const GroupKey& o) const {
    return std::tie(method, N, Nz, lag0, L, fmt, v, aux) <
           std::tie(o.method, o.N, o.Nz, o.lag0, o.L, o.fmt, o.v, o.aux);
  }
};

// Pair kernels that take per-correlation descriptors: every request of the
// method (and padded length class) shares one launch.
bool packable(int method, int Nz) {
  if (method == FPCC_PCC1 || method == FPCC_PCCV || method == FPCC_CC1B_POPCOUNT) return true;
  int n1, n2;
  if (method == FPCC_PCC2 || method == FPCC_GNCC || method == FPCC_CC1B)
    return pair_supported(Nz) || large_supported(Nz / 2, &n1, &n2);
  return false;
}

int product_fmt(const Server* s, int method) {
  if (method == FPCC_WPCC) return s->fmt == FPCC_I16 ? FPCC_F32 : s->fmt;   // wavelet spectra: F32 or F16
  return (method == FPCC_PCC2 || method == FPCC_PCC1 || method == FPCC_PCCV) ? s->fmt : FPCC_F32;
}

void method_kinds(int m, int* kind1, int* kind2) {
  switch (m) {
    case FPCC_PCC2: *kind1 = *kind2 = 1; break;
    case FPCC_GNCC: *kind1 = *kind2 = 2; break;
    case FPCC_CC1B: *kind1 = 3; *kind2 = 4; break;
    case FPCC_CC1B_POPCOUNT: *kind1 = 7; *kind2 = 8; break;
    case FPCC_WPCC: *kind1 = *kind2 = 9; break;
    default: *kind1 = *kind2 = 6; break;
  }
}

// Ensure raw windows of the listed (sta, win) are on the device; returns rows.
int ensure_raw(Server* s, int N, const std::vector<int64_t>& keys, std::vector<int>& rows, InFlight& fl) {
  Slab& sl = slab_of(s, Product{0, N, 0, 0});
  rows.resize(keys.size());
  std::vector<int> miss;
  for (size_t i = 0; i < keys.size(); i++) {
    int r = find_row(sl, keys[i]);
    if (r < 0) {
      r = claim_row(s, sl, keys[i], 1);
      if (r < 0) return no_mem("server: no free row for a raw window (every row held by this batch, budget reached)");
      miss.push_back((int)i);
    }
    rows[i] = r;
    sl.pin[r]++;
    fl.pinned_rows.push_back({&sl, r});
  }
  std::vector<const char*> src(miss.size());
  std::vector<int> chunk(miss.size());
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t k = 0; k < miss.size(); k++) {
      const int64_t key = keys[miss[k]];
      auto it = s->windows.find({(int)(key >> 32), (int)(uint32_t)key});
      if (it == s->windows.end()) return FPCC_EARG;
      src[k] = (const char*)it->second.x;
      chunk[k] = it->second.chunk;
    }
  }
  // one copy per run of windows that sit at a constant pitch in one pinned
  // arena chunk (registered one after the other) and go to consecutive rows; a
  // copy never spans two host allocations
  const int64_t w = (int64_t)N * 4;
  for (size_t k = 0; k < miss.size();) {
    const int r0 = rows[miss[k]];
    size_t k1 = k + 1;
    int64_t pitch = 0;
    for (; k1 < miss.size(); k1++) {
      const int64_t d = src[k1] - src[k];
      if (chunk[k1] != chunk[k] || rows[miss[k1]] != r0 + (int)(k1 - k)) break;
      if (k1 == k + 1) {
        if (d < w || d > ((int64_t)1 << 30)) break;
        pitch = d;
      } else if (d != pitch * (int64_t)(k1 - k)) {
        break;
      }
    }
    char* dst = (char*)sl.base + (int64_t)r0 * sl.row_bytes;
    const cudaError_t e = (k1 - k == 1)
        ? cudaMemcpyAsync(dst, src[k], (size_t)w, cudaMemcpyHostToDevice, s->st)
        : cudaMemcpy2DAsync(dst, (size_t)sl.row_bytes, src[k], (size_t)pitch, (size_t)w, k1 - k,
                            cudaMemcpyHostToDevice, s->st);
    if (e != cudaSuccess) return cuda_err(e, "window upload");
    k = k1;
  }
  return 0;
}

// Ensure products of `kind` for the keys; computes the missing ones from raw rows.
int ensure_products(Server* s, const Product& pk, const std::vector<int64_t>& keys, std::vector<int>& rows,
                    InFlight& fl) {
  Slab& sl = slab_of(s, pk);
  rows.resize(keys.size());
  std::vector<int64_t> miss_keys;
  std::vector<int> miss_rows;
  // resident products first (pinned as found), then the claims for the rest:
  // room for every distinct missing key is asked for at the first claim (one
  // growth of the slab), and one row fewer at each claim after it; the keys
  // repeat (both stations of many pairs), so counting them would ask for more
  // rows than the windows need and fail under a tight budget
  std::vector<size_t> absent;
  for (size_t i = 0; i < keys.size(); i++) {
    const int r = find_row(sl, keys[i]);
    if (r < 0) {
      absent.push_back(i);
      continue;
    }
    rows[i] = r;
    sl.pin[r]++;
    fl.pinned_rows.push_back({&sl, r});
  }
  if (absent.empty()) return 0;
  int left;
  {
    std::vector<int64_t> ak;
    ak.reserve(absent.size());
    for (size_t i : absent) ak.push_back(keys[i]);
    std::sort(ak.begin(), ak.end());
    left = (int)(std::unique(ak.begin(), ak.end()) - ak.begin());
  }
  for (size_t i : absent) {
    int r = find_row(sl, keys[i]);   // claimed already for an earlier repeat of the key
    if (r < 0) {
      r = claim_row(s, sl, keys[i], std::max(1, left--));
      if (r < 0) return no_mem("server: no free product row (every row held by this batch, budget reached)");
      miss_keys.push_back(keys[i]);
      miss_rows.push_back(r);
    }
    rows[i] = r;
    sl.pin[r]++;
    fl.pinned_rows.push_back({&sl, r});
  }
  const int n = (int)miss_keys.size();
  std::vector<int> raw_rows;
  int rc = ensure_raw(s, pk.N, miss_keys, raw_rows, fl);
  if (rc) return rc;
  Slab& raw = slab_of(s, Product{0, pk.N, 0, 0});
  // the station stage reads the raw rows and writes the slab rows in place when
  // each set is one ascending run of rows (the usual case: fresh rows are claimed
  // in order); otherwise it gathers / scatters through scratch rows
  auto ascending = [](const std::vector<int>& r) {
    for (size_t i = 1; i < r.size(); i++)
      if (r[i] != r[0] + (int)i) return false;
    return true;
  };
  const bool in_place_x = ascending(raw_rows), in_place_p = ascending(miss_rows);
  const int64_t N = pk.N;
  void* dx = in_place_x ? (char*)raw.base + (int64_t)raw_rows[0] * raw.row_bytes
                        : dbuf(s, &s->d_tmp_x, &s->n_tmp_x, (size_t)n * round16(N * 4));
  void* dp = in_place_p ? (char*)sl.base + (int64_t)miss_rows[0] * sl.row_bytes
                        : dbuf(s, &s->d_tmp_p, &s->n_tmp_p, (size_t)n * sl.row_bytes);
  void* di = dbuf(s, &s->d_idx, &s->n_idx, (size_t)2 * n * sizeof(int) + 64);
  if (!dx || !dp || !di) return no_mem("server: device scratch of a station stage");
  if (!in_place_x || !in_place_p) {
    std::vector<int> idx(2 * n);
    for (int i = 0; i < n; i++) { idx[i] = raw_rows[i]; idx[n + i] = miss_rows[i]; }
    if (cudaError_t ue = upload(fl, di, idx.data(), idx.size() * sizeof(int), s->st)) return cuda_err(ue, "upload");
  }
  const int64_t ldx = round16(N * 4) / 4;   // = raw.row_bytes / 4
  if (!in_place_x &&
      copy_rows(raw.base, raw.row_bytes, (const int*)di, dx, ldx * 4, nullptr, n, N * 4, s->st) != cudaSuccess)
    return cuda_err(cudaGetLastError(), "row copy");
  int method = FPCC_PCC2, rule = FPCC_AMP_F_REG;
  int64_t ldo = sl.row_bytes / (pk.fmt ? 4 : 8);
  switch (pk.kind) {
    case 1: method = FPCC_PCC2; break;
    case 2: method = FPCC_GNCC; break;
    case 3: method = FPCC_CC1B; rule = FPCC_SIGN_GE; break;
    case 4: method = FPCC_CC1B; rule = FPCC_SIGN_GT; break;
    case 6: method = FPCC_PCC1; break;
    case 7: method = FPCC_CC1B_POPCOUNT; rule = FPCC_SIGN_GE; ldo = sl.row_bytes / 4; break;
    case 8: method = FPCC_CC1B_POPCOUNT; rule = FPCC_SIGN_GT; ldo = sl.row_bytes / 4; break;
    default: break;
  }
  // in place, the stage touches only slab rows (no server scratch): it runs on a lane
  fpcc_ctx* cx = (in_place_x && in_place_p && !s->lanes.empty()) ? lane_begin(s).ctx : s->ctx;
  if (pk.kind == 5) {
    rc = fpcc_energy_stage(cx, (const float*)dx, ldx, n, pk.N, (double*)dp, sl.row_bytes / 8);
  } else {
    // FP64 analytic signals for windows with zero runs (known from the host copies)
    std::vector<int32_t> f64;
    if (method == FPCC_PCC2 || method == FPCC_PCC1) {
      std::lock_guard<std::mutex> lk(s->mu);
      for (int i = 0; i < n; i++) {
        auto it = s->windows.find({(int)(miss_keys[i] >> 32), (int)(uint32_t)miss_keys[i]});
        if (it != s->windows.end() && it->second.zeros >= FPCC_F64_ZERO_SAMPLES) f64.push_back(i);
      }
    }
    rc = fpcc_station_stage_ex(cx, method, (const float*)dx, ldx, n, pk.N, pk.Nz, pk.fmt, rule, dp, ldo,
                               f64.data(), (int)f64.size());
  }
  if (rc) return rc;
  if (!in_place_p &&
      copy_rows(dp, sl.row_bytes, nullptr, sl.base, sl.row_bytes, (const int*)di + n, n, sl.row_bytes, s->st) !=
          cudaSuccess)
    return cuda_err(cudaGetLastError(), "row copy");
  s->station_rows += n;
  return 0;
}

// Results of a group from the device block dy (requests `reqs` in output order,
// batch indices first.., the same layout as the batch's result block at
// out_base) to where they go.  A request whose output lies in a range the caller
// registered (page-locked host memory) is copied straight into it, and runs of
// such rows at one stride as a single strided copy; the others go to the batch's
// pinned block, from which the completer threads copy them out.
cudaError_t d2h_results(InFlight& fl, const std::vector<Req*>& reqs, size_t first, size_t out_base, const char* dy,
                        cudaStream_t st) {
  const size_t n = reqs.size();
  auto dst_of = [&](size_t i) -> char* {
    const Req& q = *reqs[i];
    return q.r.method == FPCC_CC1B_POPCOUNT ? (char*)q.r.num : (char*)q.r.y;
  };
  auto bytes_of = [&](size_t i) -> size_t {
    return (size_t)reqs[i]->L * (reqs[i]->r.method == FPCC_CC1B_POPCOUNT ? 8 : 4);
  };
  auto registered = [&](size_t i) {
    const char* d = dst_of(i);
    if (!d || fl.out_ranges.empty()) return false;
    const size_t b = bytes_of(i);
    for (auto& r : fl.out_ranges)
      if (d >= r.first && d + b <= r.first + r.second) return true;
    return false;
  };
  size_t off = 0;
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < n && e == cudaSuccess;) {
    const size_t b = bytes_of(i);
    size_t j = i + 1, run_bytes = b;
    if (registered(i)) {
      // rows of equal length at a constant stride: one strided copy
      const ptrdiff_t stride = (j < n) ? dst_of(j) - dst_of(i) : (ptrdiff_t)b;
      if (stride >= (ptrdiff_t)b && stride <= ((ptrdiff_t)1 << 30))
        while (j < n && bytes_of(j) == b && registered(j) && dst_of(j) - dst_of(j - 1) == stride) j++;
      for (size_t k = i; k < j; k++) fl.direct[first + k] = 1;
      if (j - i == 1)
        e = cudaMemcpyAsync(dst_of(i), dy + off, b, cudaMemcpyDeviceToHost, st);
      else
        e = cudaMemcpy2DAsync(dst_of(i), (size_t)stride, dy + off, b, b, j - i, cudaMemcpyDeviceToHost, st);
      off += b * (j - i);
    } else {
      while (j < n && !registered(j)) run_bytes += bytes_of(j++);
      e = cudaMemcpyAsync((char*)fl.h_out + out_base + off, dy + off, run_bytes, cudaMemcpyDeviceToHost, st);
      off += run_bytes;
    }
    i = j;
  }
  return e;
}

// Device output of a group: its place in the batch's result buffer, or the
// shared scratch buffer when the batch has none.
char* group_out(Server* s, InFlight& fl, size_t out_base, size_t bytes) {
  if (fl.d_out) return (char*)fl.d_out + out_base;
  return (char*)dbuf(s, &s->d_y, &s->n_y, bytes);
}

// Results of a group whose pair stage was queued on `st`: downloaded on the
// results stream after that pair stage (the batch's own result buffer is not
// reused before the batch completes), else on `st` itself.
cudaError_t results_down(Server* s, InFlight& fl, const std::vector<Req*>& reqs, size_t first, size_t out_base,
                         const char* dy, cudaStream_t st) {
  if (!fl.d_out || !s->st_out) return d2h_results(fl, reqs, first, out_base, dy, st);
  if (s->out_used == s->out_ev.size()) {
    cudaEvent_t e;
    if (cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming)) return ce;
    s->out_ev.push_back(e);
  }
  cudaEvent_t e = s->out_ev[s->out_used++];
  if (cudaError_t ce = cudaEventRecord(e, st)) return ce;
  if (cudaError_t ce = cudaStreamWaitEvent(s->st_out, e, 0)) return ce;
  return d2h_results(fl, reqs, first, out_base, dy, s->st_out);
}

int run_group(Server* s, const GroupKey& g, std::vector<Req*>& reqs, InFlight& fl, size_t out_base,
              bool products_only, size_t first = 0, GroupRows* gr = nullptr) {
  const int n = (int)reqs.size();
  const int m = g.method;
  int kind1, kind2;
  method_kinds(m, &kind1, &kind2);
  const int Nz = (m == FPCC_PCC1 || m == FPCC_PCCV || m == FPCC_CC1B_POPCOUNT) ? 0 : g.Nz;
  Product p1{kind1, g.N, Nz, g.fmt}, p2{kind2, g.N, Nz, g.fmt};
  std::vector<int> r1, r2, e1, e2;
  int rc;
  if (gr && gr->ok) {
    r1.swap(gr->r1);
    r2.swap(gr->r2);
    e1.swap(gr->e1);
    e2.swap(gr->e2);
    gr->ok = false;
  } else {
    std::vector<int64_t> k1(n), k2(n);
    for (int i = 0; i < n; i++) {
      k1[i] = wkey(reqs[i]->r.sta1, reqs[i]->r.window);
      k2[i] = wkey(reqs[i]->r.sta2, reqs[i]->r.window);
    }
    if (kind1 == kind2) {
      std::vector<int64_t> all(k1);
      all.insert(all.end(), k2.begin(), k2.end());
      std::vector<int> rr;
      if ((rc = ensure_products(s, p1, all, rr, fl))) return rc;
      r1.assign(rr.begin(), rr.begin() + n);
      r2.assign(rr.begin() + n, rr.end());
    } else {
      if ((rc = ensure_products(s, p1, k1, r1, fl)) || (rc = ensure_products(s, p2, k2, r2, fl))) return rc;
    }
    if (m == FPCC_GNCC) {
      std::vector<int64_t> all(k1);
      all.insert(all.end(), k2.begin(), k2.end());
      std::vector<int> rr;
      if ((rc = ensure_products(s, Product{5, g.N, 0, 0}, all, rr, fl))) return rc;
      e1.assign(rr.begin(), rr.begin() + n);
      e2.assign(rr.begin() + n, rr.end());
    }
  }
  if (products_only) {
    if (gr) {
      gr->r1.swap(r1);
      gr->r2.swap(r2);
      gr->e1.swap(e1);
      gr->e2.swap(e2);
      gr->ok = true;
    }
    return 0;
  }
  pair_join(s);
  // pair list: rows in one slab (both roles share a slab except the 1-bit methods,
  // whose station-2 rows are offset by the station-1 slab capacity after a merge)
  Slab& s1 = slab_of(s, p1);
  Slab& s2 = slab_of(s, p2);
  const void* base = s1.base;
  std::vector<int32_t> pairs(2 * n);
  if (&s1 != &s2) {
    // stage the station-2 rows behind the station-1 rows in the temporary buffer
    const int64_t rb = s1.row_bytes;
    void* merged = dbuf(s, &s->d_tmp_p, &s->n_tmp_p, (size_t)2 * n * rb);
    void* di = dbuf(s, &s->d_idx, &s->n_idx, (size_t)2 * n * sizeof(int) + 64);
    if (!merged || !di) return no_mem("server: device scratch of a pair stage");
    std::vector<int> idx(2 * n);
    for (int i = 0; i < n; i++) { idx[i] = r1[i]; idx[n + i] = r2[i]; }
    if (cudaError_t ue = upload(fl, di, idx.data(), idx.size() * sizeof(int), s->st)) return cuda_err(ue, "upload");
    if (copy_rows(s1.base, rb, (const int*)di, merged, rb, nullptr, n, rb, s->st) != cudaSuccess ||
        copy_rows(s2.base, rb, (const int*)di + n, (char*)merged + (size_t)n * rb, rb, nullptr, n, rb, s->st) !=
            cudaSuccess)
      return cuda_err(cudaGetLastError(), "row copy");
    base = merged;
    for (int i = 0; i < n; i++) { pairs[2 * i] = i; pairs[2 * i + 1] = n + i; }
  } else {
    for (int i = 0; i < n; i++) { pairs[2 * i] = r1[i]; pairs[2 * i + 1] = r2[i]; }
  }
  const double* E = nullptr;
  int64_t ldE = 0;
  std::vector<int32_t> epairs;
  if (m == FPCC_GNCC) {
    // energies are indexed by the same pair entries: rewrite both lists onto one index space
    Slab& se = slab_of(s, Product{5, g.N, 0, 0});
    // the pair kernel reads energy rows by the pair's station rows, so stage both
    // spectra and energies in pair order
    const int64_t rb = s1.row_bytes, eb = se.row_bytes;
    void* tmp = dbuf(s, &s->d_tmp_p, &s->n_tmp_p, (size_t)2 * n * (rb + eb));
    void* di = dbuf(s, &s->d_idx, &s->n_idx, (size_t)4 * n * sizeof(int) + 64);
    if (!tmp || !di) return no_mem("server: device scratch of a GNCC pair stage");
    std::vector<int> idx(4 * n);
    for (int i = 0; i < n; i++) { idx[i] = r1[i]; idx[n + i] = r2[i]; idx[2 * n + i] = e1[i]; idx[3 * n + i] = e2[i]; }
    if (cudaError_t ue = upload(fl, di, idx.data(), idx.size() * sizeof(int), s->st)) return cuda_err(ue, "upload");
    char* spec = (char*)tmp;
    char* en = spec + (size_t)2 * n * rb;
    if (copy_rows(s1.base, rb, (const int*)di, spec, rb, nullptr, 2 * n, rb, s->st) != cudaSuccess ||
        copy_rows(se.base, eb, (const int*)di + 2 * n, en, eb, nullptr, 2 * n, eb, s->st) != cudaSuccess)
      return cuda_err(cudaGetLastError(), "row copy");
    base = spec;
    E = (const double*)en;
    ldE = eb / 8;
    for (int i = 0; i < n; i++) { pairs[2 * i] = i; pairs[2 * i + 1] = n + i; }
  }
  // device pair list (its own buffer: the index buffer may still feed queued copies) and output
  const size_t ybytes = (size_t)n * g.L * (m == FPCC_CC1B_POPCOUNT ? 8 : 4);
  void* dpl = dbuf(s, &s->d_pl, &s->n_pl, (size_t)2 * n * sizeof(int32_t));
  void* dy = group_out(s, fl, out_base, ybytes);
  if (!dpl || !dy) return no_mem("server: device pair list or output of a pair stage");
  if (cudaError_t ue = upload(fl, dpl, pairs.data(), pairs.size() * sizeof(int32_t), s->st)) return cuda_err(ue, "upload");
  const int64_t lds = slab_of(s, p1).row_bytes / ((m == FPCC_CC1B_POPCOUNT) ? 4 : (g.fmt ? 4 : 8));
  if (m == FPCC_CC1B_POPCOUNT) {
    rc = fpcc_pair_stage(s->ctx, m, base, lds, 0, (const int32_t*)dpl, n, g.N, 0, g.lag0, g.lag0 + g.L - 1, 0.f,
                         nullptr, 0, nullptr, g.L, (int64_t*)dy);
  } else {
    rc = fpcc_pair_stage(s->ctx, m, base, lds, g.fmt, (const int32_t*)dpl, n, g.N, Nz ? Nz : g.N, g.lag0,
                         g.lag0 + g.L - 1, g.v, E, ldE, (float*)dy, g.L, nullptr);
  }
  if (rc) return rc;
  if (cudaError_t ce = results_down(s, fl, reqs, first, out_base, (const char*)dy, s->st))
    return cuda_err(ce, "results");
  return 0;
}

// Station products of the phase methods for windows of different lengths, in
// shared launches (fpcc_station_stage_multi): every missing product of the group
// whose window length is not 2,3,5-smooth, or whose window has zero samples
// (FP64 analytic signal), is made here; the per-length path makes the rest.
// Which path makes a product depends only on its window, so a result is the
// same alone and in any mix.
// All the batch's groups of one kind (1: PCC2 phase spectra, Nz per group;
// 6: phase signals of PCC1 / PCC_v) go through one call, so that windows of
// every length and padded length share the packed stage's launches.
int prefetch_phase(Server* s, int kind, int fmt, const std::vector<std::pair<int, std::vector<Req*>*>>& sets,
                   InFlight& fl) {
  struct Miss {
    int N, Nz;
    int64_t key;
    Slab* sl;
    int row;
    int f64;
  };
  std::vector<Miss> miss;
  std::set<std::tuple<int, int, int64_t>> seen;
  int lastN = -1;
  bool smooth = false;
  for (const auto& set : sets)
  for (Req* q : *set.second) {
    const int Nz = set.first;
    if (q->N != lastN) {
      int a2, b3, c5;
      lastN = q->N;
      smooth = factor235(q->N, &a2, &b3, &c5);
    }
    for (int side = 0; side < 2; side++) {
      // the per-length path makes products of smooth lengths without gaps
      const int f64 = (q->f64 >> side) & 1;
      if (smooth && !f64) continue;
      const int64_t key = wkey(side ? q->r.sta2 : q->r.sta1, q->r.window);
      if (!seen.insert(std::make_tuple(q->N, Nz, key)).second) continue;
      Slab& sl = slab_of(s, Product{kind, q->N, Nz, fmt});
      if (const int r = find_row(sl, key); r >= 0) {
        // resident: pinned for the batch, so that the claims below (which may
        // release idle product classes to stay in budget) cannot take it away
        // before the batch's pair stages read it
        sl.pin[r]++;
        fl.pinned_rows.push_back({&sl, r});
        continue;
      }
      miss.push_back({q->N, Nz, key, &sl, -1, f64});
    }
  }
  if (miss.empty()) return 0;
  // rows for the missing products, each slab growing once to what it needs
  {
    std::map<Slab*, int> left;
    for (const Miss& m : miss) left[m.sl]++;
    for (Miss& m : miss) {
      const int r = claim_row(s, *m.sl, m.key, left[m.sl]--);
      if (r < 0) return no_mem("server: no free product row (every row held by this batch, budget reached)");
      m.sl->pin[r]++;
      fl.pinned_rows.push_back({m.sl, r});
      m.row = r;
    }
  }
  std::stable_sort(miss.begin(), miss.end(),
                   [](const Miss& a, const Miss& b) { return std::tie(a.N, a.Nz) < std::tie(b.N, b.Nz); });
  const int n = (int)miss.size();
  std::vector<int> rawrow(n);
  int rc;
  for (int i0 = 0; i0 < n;) {
    int i1 = i0;
    std::vector<int64_t> keys;
    while (i1 < n && miss[i1].N == miss[i0].N) keys.push_back(miss[i1++].key);
    std::vector<int> rr;
    if ((rc = ensure_raw(s, miss[i0].N, keys, rr, fl))) return rc;
    for (int i = i0; i < i1; i++) rawrow[i] = rr[i - i0];
    i0 = i1;
  }
  // all rows claimed: addresses are stable from here on
  const int64_t esz = fmt == FPCC_F32 ? 8 : 4;
  int64_t ldo = 0;
  for (auto& m : miss) ldo = std::max<int64_t>(ldo, m.sl->row_bytes / esz);
  std::vector<fpcc_station_row> rows(n);
  for (int i = 0; i < n; i++) {
    Slab& raw = slab_of(s, Product{0, miss[i].N, 0, 0});
    rows[i].d_x = (const float*)((const char*)raw.base + (int64_t)rawrow[i] * raw.row_bytes);
    rows[i].N = miss[i].N;
    rows[i].Nz = miss[i].Nz;
    rows[i].f64 = miss[i].f64;
    rows[i].pad = 0;
  }
  // whole conversion classes (rows sharing M-point transforms) go to the lanes,
  // longest work first onto the least loaded lane; one packed stage per lane
  std::map<int, std::vector<int>> byM;
  for (int i = 0; i < n; i++) byM[conv_class_len(miss[i].N)].push_back(i);
  std::vector<std::pair<double, int>> work;
  for (auto& kv : byM) work.push_back({(double)kv.second.size() * (double)kv.first, kv.first});
  std::sort(work.rbegin(), work.rend());
  const int K = std::max(1, (int)s->lanes.size());
  std::vector<double> load(K, 0.0);
  std::vector<std::vector<int>> part(K);
  for (auto& w : work) {
    const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[l] += w.first;
    const std::vector<int>& v = byM[w.second];
    part[l].insert(part[l].end(), v.begin(), v.end());
  }
  const int method = (kind == 1) ? FPCC_PCC2 : FPCC_PCC1;
  for (int l = 0; l < K; l++) {
    std::vector<int>& ix = part[l];
    if (ix.empty()) continue;
    std::sort(ix.begin(), ix.end());   // (N, Nz) order, as the packed stage requires
    const int m = (int)ix.size();
    std::vector<fpcc_station_row> sub(m);
    for (int i = 0; i < m; i++) sub[i] = rows[ix[i]];
    // without lanes: the server's own context, stream and scratch
    const bool lane = !s->lanes.empty();
    Lane* ln = lane ? &lane_at(s, l) : nullptr;
    fpcc_ctx* cx = lane ? ln->ctx : s->ctx;
    cudaStream_t st = lane ? ln->st : s->st;
    void* tmp = lane ? lane_buf(s, *ln, &ln->d_tmp, &ln->n_tmp, (size_t)m * ldo * esz)
                     : dbuf(s, &s->d_tmp_p, &s->n_tmp_p, (size_t)m * ldo * esz);
    void* dc = lane ? lane_buf(s, *ln, &ln->d_idx, &ln->n_idx, (size_t)m * sizeof(RowCopy) + 64)
                    : dbuf(s, &s->d_idx, &s->n_idx, (size_t)m * sizeof(RowCopy) + 64);
    if (!tmp || !dc) return no_mem("server: device scratch of a packed station stage");
    if ((rc = fpcc_station_stage_multi(cx, method, sub.data(), m, fmt, FPCC_AMP_F_REG, tmp, ldo))) return rc;
    std::vector<RowCopy> cp(m);
    for (int i = 0; i < m; i++) {
      const Miss& q = miss[ix[i]];
      cp[i] = RowCopy{(const char*)tmp + (size_t)i * ldo * esz, (char*)q.sl->base + (int64_t)q.row * q.sl->row_bytes,
                      q.sl->row_bytes};
    }
    if (cudaError_t ue = upload(fl, dc, cp.data(), cp.size() * sizeof(RowCopy), st)) return cuda_err(ue, "upload");
    for (int i0 = 0; i0 < m; i0 += 65535) {
      const int k = std::min(65535, m - i0);
      int64_t mx = 0;
      for (int i = i0; i < i0 + k; i++) mx = std::max(mx, cp[i].bytes);
      const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(64, (mx / 16 + 255) / 256));
      k_scatter_rows<<<dim3(gx, k), 256, 0, st>>>((const RowCopy*)dc + i0);
      if (cudaError_t ke = cudaGetLastError()) return cuda_err(ke, "row scatter");
    }
  }
  s->station_rows += n;
  return 0;
}

// A group whose pair kernel takes descriptors: window lengths and lag windows
// vary per request; products are ensured per window length, then every
// correlation of the group runs in one launch reading its rows in place.
int run_group_packed(Server* s, const GroupKey& g, std::vector<Req*>& reqs, InFlight& fl, size_t out_base,
                     bool products_only, Lane* on = nullptr, size_t first = 0, GroupRows* gr = nullptr) {
  const int n = (int)reqs.size();
  const int m = g.method;
  int kind1, kind2;
  method_kinds(m, &kind1, &kind2);
  const bool fft = (m == FPCC_PCC2 || m == FPCC_GNCC || m == FPCC_CC1B);
  const int Nz = fft ? g.Nz : 0;
  std::vector<int> r1(n), r2(n), e1(n), e2(n);
  int rc;
  std::map<int, std::vector<int>> byN;
  if (gr && gr->ok) {
    r1.swap(gr->r1);
    r2.swap(gr->r2);
    e1.swap(gr->e1);
    e2.swap(gr->e2);
    gr->ok = false;
  } else {
    for (int i = 0; i < n; i++) byN[reqs[i]->N].push_back(i);
  }
  for (auto& kv : byN) {
    const int N = kv.first;
    const std::vector<int>& ix = kv.second;
    const int k = (int)ix.size();
    std::vector<int64_t> all(2 * k);
    for (int j = 0; j < k; j++) {
      all[j] = wkey(reqs[ix[j]]->r.sta1, reqs[ix[j]]->r.window);
      all[k + j] = wkey(reqs[ix[j]]->r.sta2, reqs[ix[j]]->r.window);
    }
    std::vector<int> rr;
    if (kind1 == kind2) {
      if ((rc = ensure_products(s, Product{kind1, N, Nz, g.fmt}, all, rr, fl))) return rc;
      for (int j = 0; j < k; j++) { r1[ix[j]] = rr[j]; r2[ix[j]] = rr[k + j]; }
    } else {
      std::vector<int64_t> k1(all.begin(), all.begin() + k), k2(all.begin() + k, all.end());
      std::vector<int> rb;
      if ((rc = ensure_products(s, Product{kind1, N, Nz, g.fmt}, k1, rr, fl)) ||
          (rc = ensure_products(s, Product{kind2, N, Nz, g.fmt}, k2, rb, fl)))
        return rc;
      for (int j = 0; j < k; j++) { r1[ix[j]] = rr[j]; r2[ix[j]] = rb[j]; }
    }
    if (m == FPCC_GNCC) {
      if ((rc = ensure_products(s, Product{5, N, 0, 0}, all, rr, fl))) return rc;
      for (int j = 0; j < k; j++) { e1[ix[j]] = rr[j]; e2[ix[j]] = rr[k + j]; }
    }
  }
  if (products_only) {
    if (gr) {
      gr->r1.swap(r1);
      gr->r2.swap(r2);
      gr->e1.swap(e1);
      gr->e2.swap(e2);
      gr->ok = true;
    }
    return 0;
  }
  // the pair stage runs on the server's stream, or on the lane `on` (its own
  // context, stream and output buffers), which first waits for the server's
  // stream and for the lane work that made the group's products
  fpcc_ctx* cx = s->ctx;
  cudaStream_t st = s->st;
  if (on) {
    cx = on->ctx;
    st = on->st;
    cudaEventRecord(s->main_ev, s->st);
    cudaStreamWaitEvent(st, s->main_ev, 0);
    const std::vector<cudaEvent_t>* w = s->pair_waits;
    const bool all = !w || s->lane_seq != s->pair_seq || std::find(w->begin(), w->end(), nullptr) != w->end();
    if (all) {
      for (auto& l : s->lanes)
        if (l.dirty) {
          cudaEventRecord(l.ev, l.st);
          cudaStreamWaitEvent(st, l.ev, 0);
        }
    } else {
      for (cudaEvent_t e : *w) cudaStreamWaitEvent(st, e, 0);
    }
    on->dirty = true;
  } else {
    pair_join(s);
  }
  // every product is in place (slabs no longer move): descriptors with row addresses
  const size_t osz = (m == FPCC_CC1B_POPCOUNT) ? 8 : 4;
  size_t total = 0;
  for (int i = 0; i < n; i++) total += (size_t)reqs[i]->L * osz;
  char* dy = on ? (char*)lane_buf(s, *on, &on->d_tmp, &on->n_tmp, total) : group_out(s, fl, out_base, total);
  void* dd = on ? lane_buf(s, *on, &on->d_idx, &on->n_idx, (size_t)n * sizeof(fpcc_pair_desc))
                : dbuf(s, &s->d_desc, &s->n_desc, (size_t)n * sizeof(fpcc_pair_desc));
  if (!dy || !dd) return no_mem("server: device output or descriptors of a packed pair stage");
  std::vector<fpcc_pair_desc> d(n);
  size_t off = 0;
  int maxL = 0;
  // the slabs of the group's window lengths, looked up once per length
  int lastN = -1;
  Slab *sa = nullptr, *sb = nullptr, *se = nullptr;
  for (int i = 0; i < n; i++) {
    const Req& q = *reqs[i];
    if (q.N != lastN) {
      lastN = q.N;
      sa = &slab_of(s, Product{kind1, q.N, Nz, g.fmt});
      sb = &slab_of(s, Product{kind2, q.N, Nz, g.fmt});
      if (m == FPCC_GNCC) se = &slab_of(s, Product{5, q.N, 0, 0});
    }
    fpcc_pair_desc& e = d[i];
    memset(&e, 0, sizeof(e));
    e.a = (const char*)sa->base + (int64_t)r1[i] * sa->row_bytes;
    e.b = (const char*)sb->base + (int64_t)r2[i] * sb->row_bytes;
    if (m == FPCC_GNCC) {
      e.ea = (const double*)((const char*)se->base + (int64_t)e1[i] * se->row_bytes);
      e.eb = (const double*)((const char*)se->base + (int64_t)e2[i] * se->row_bytes);
    }
    e.y = dy + off;
    off += (size_t)q.L * osz;
    e.N = q.N;
    e.lag0 = q.lag0;
    e.L = q.L;
    // the scales of the per-group pair stage (src/FFTapps.c:832, :340, :357)
    e.scale = (m == FPCC_PCC2) ? 1.0f / ((float)Nz * (float)q.N) : (fft ? (float)(1.0 / (double)Nz) : 0.0f);
    maxL = std::max(maxL, q.L);
  }
  // direct sums: a block's work grows with its window length, and blocks are
  // issued descriptor by descriptor, so the longest windows go first (each
  // descriptor names its own output row: the order changes no result)
  if (m == FPCC_PCC1 || m == FPCC_PCCV || m == FPCC_CC1B_POPCOUNT)
    std::stable_sort(d.begin(), d.end(), [](const fpcc_pair_desc& a, const fpcc_pair_desc& b) { return a.N > b.N; });
  if (cudaError_t ue = upload(fl, dd, d.data(), d.size() * sizeof(fpcc_pair_desc), st)) return cuda_err(ue, "upload");
  rc = fpcc_pair_stage_packed(cx, m, g.fmt, Nz, (const fpcc_pair_desc*)dd, n, maxL, g.v, m == FPCC_CC1B_POPCOUNT);
  if (rc) return rc;
  // a lane's output buffer is its own: its results go down on the lane
  const cudaError_t ce = on ? d2h_results(fl, reqs, first, out_base, dy, st)
                            : results_down(s, fl, reqs, first, out_base, dy, st);
  if (ce) return cuda_err(ce, "results");
  return 0;
}

// Wavelet PCC plan of a window length, padded length and family cap (built once).
fpcc_wpcc_plan* wpcc_plan_for(Server* s, int N, int Nz, int cap, int Lag1, int Lag2) {
  auto key = std::make_tuple(N, Nz, cap);
  auto it = s->wplans.find(key);
  if (it != s->wplans.end()) return it->second;
  fpcc_wpcc_plan* p = nullptr;
  if (fpcc_wpcc_plan_create(s->ctx, &p, (unsigned)N, Lag1, Lag2, s->wav.pmin, s->wav.pmax, s->wav.V, s->wav.type,
                            s->wav.op1, s->wav.rule, FPCC_NZ_FAST) != 0)
    return nullptr;
  int nz = 0;
  fpcc_wpcc_plan_info(p, &nz, nullptr, nullptr);
  if (nz != Nz) {   // the request's length came from the same rule; a mismatch is a bug
    fpcc_wpcc_plan_destroy(p);
    return nullptr;
  }
  s->wplans[key] = p;
  return p;
}

// A WPCC group (one window length, padded length and lag window): per-scale
// phase spectra of each station window are computed into their slab rows
// directly, then one pair stage runs over the group.
int run_group_wpcc(Server* s, const GroupKey& g, std::vector<Req*>& reqs, InFlight& fl, size_t out_base,
                   size_t first) {
  const int n = (int)reqs.size();
  const int lag1 = reqs[0]->r.Lag1, lag2 = reqs[0]->r.Lag2;
  fpcc_wpcc_plan* p = wpcc_plan_for(s, g.N, g.Nz, g.aux, lag1, lag2);
  if (!p) return FPCC_EUNSUP;
  int rc;
  if ((rc = fpcc_wpcc_plan_set_lags(p, g.lag0, g.lag0 + g.L - 1))) return rc;
  const Product pk{9, g.N, g.Nz, g.fmt, g.aux, s->wav.S};
  Slab& sl = slab_of(s, pk);
  std::vector<int64_t> keys(2 * n);
  for (int i = 0; i < n; i++) {
    keys[i] = wkey(reqs[i]->r.sta1, reqs[i]->r.window);
    keys[n + i] = wkey(reqs[i]->r.sta2, reqs[i]->r.window);
  }
  std::vector<int> rows(2 * n);
  std::vector<int64_t> miss_keys;
  std::vector<int> miss_rows;
  int left = 0;   // distinct missing keys (room asked for at the first claim, as ensure_products)
  {
    std::vector<int64_t> absent;
    for (int64_t k : keys)
      if (sl.row_of.find(k) == sl.row_of.end()) absent.push_back(k);
    std::sort(absent.begin(), absent.end());
    left = (int)(std::unique(absent.begin(), absent.end()) - absent.begin());
  }
  for (int i = 0; i < 2 * n; i++) {
    int r = find_row(sl, keys[i]);
    if (r < 0) {
      r = claim_row(s, sl, keys[i], std::max(1, left--));
      if (r < 0) return no_mem("server: no free product row (every row held by this batch, budget reached)");
      miss_keys.push_back(keys[i]);
      miss_rows.push_back(r);
    }
    rows[i] = r;
    sl.pin[r]++;
    fl.pinned_rows.push_back({&sl, r});
  }
  if (!miss_keys.empty()) {
    std::vector<int> raw_rows;
    if ((rc = ensure_raw(s, g.N, miss_keys, raw_rows, fl))) return rc;
    Slab& raw = slab_of(s, Product{0, g.N, 0, 0});
    for (size_t i = 0; i < miss_keys.size(); i++) {
      const float* x = (const float*)((const char*)raw.base + (int64_t)raw_rows[i] * raw.row_bytes);
      void* dst = (char*)sl.base + (int64_t)miss_rows[i] * sl.row_bytes;
      if ((rc = fpcc_wpcc_station_stage(s->ctx, p, x, g.N, 1, dst, g.fmt))) return rc;
    }
    s->station_rows += (int64_t)miss_keys.size();
  }
  lanes_join(s);
  std::vector<int32_t> pairs(2 * n);
  for (int i = 0; i < n; i++) { pairs[2 * i] = rows[i]; pairs[2 * i + 1] = rows[n + i]; }
  const size_t ybytes = (size_t)n * g.L * 4;
  void* dpl = dbuf(s, &s->d_pl, &s->n_pl, (size_t)2 * n * sizeof(int32_t));
  void* dy = group_out(s, fl, out_base, ybytes);
  if (!dpl || !dy) return no_mem("server: device pair list or output of a pair stage");
  if (cudaError_t ue = upload(fl, dpl, pairs.data(), pairs.size() * sizeof(int32_t), s->st)) return cuda_err(ue, "upload");
  if ((rc = fpcc_wpcc_pair_stage(s->ctx, p, sl.base, g.fmt, (const int32_t*)dpl, n, (float*)dy, g.L))) return rc;
  if (cudaError_t ce = results_down(s, fl, reqs, first, out_base, (const char*)dy, s->st))
    return cuda_err(ce, "results");
  return 0;
}

void* pinned_get(Server* s, size_t bytes, size_t* got) {
  for (size_t i = 0; i < s->pinned_pool.size(); i += 2) {
    if ((size_t)s->pinned_pool[i + 1] >= bytes) {
      void* p = s->pinned_pool[i];
      *got = (size_t)s->pinned_pool[i + 1];
      s->pinned_pool.erase(s->pinned_pool.begin() + i, s->pinned_pool.begin() + i + 2);
      return p;
    }
  }
  void* p = nullptr;
  const size_t b = std::max(bytes, (size_t)1 << 20);
  if (cudaMallocHost(&p, b) != cudaSuccess) return nullptr;
  *got = b;
  return p;
}

constexpr int kDeliverThreads = 8;                   // threads copying out one large batch
constexpr size_t kDeliverChunk = (size_t)16 << 20;   // bytes per delivering thread, at least

void pinned_put(Server* s, void* p, size_t bytes) {
  s->pinned_pool.push_back(p);
  s->pinned_pool.push_back((void*)bytes);
}

// Copies results [i0, i1) of a batch into the callers' buffers.
void deliver_range(InFlight* fl, size_t i0, size_t i1) {
  for (size_t i = i0; i < i1; i++) {
    Req& q = fl->reqs[i];
    if (fl->direct[i]) continue;
    if (q.r.method == FPCC_CC1B_POPCOUNT) {
      if (q.r.num) memcpy(q.r.num, (char*)fl->h_out + fl->out_off[i], (size_t)q.L * 8);
    } else if (q.r.y) {
      memcpy(q.r.y, (char*)fl->h_out + fl->out_off[i], (size_t)q.L * 4);
    }
  }
}

// Deliver a batch's results and record its latencies (completer threads).  A
// large batch is copied out by several threads: one thread's memcpy into the
// callers' (pageable) buffers is slower than the GPU makes the results.
void deliver(Server* s, InFlight& fl) {
  const int err = fl.err;
  const auto now = Clock::now();
  if (!err) {
    size_t bytes = 0;
    for (size_t i = 0; i < fl.reqs.size(); i++)
      if (!fl.direct[i]) bytes += (size_t)fl.reqs[i].L * (fl.reqs[i].r.method == FPCC_CC1B_POPCOUNT ? 8 : 4);
    const size_t n = fl.reqs.size();
    const int k = (int)std::min<size_t>(kDeliverThreads, std::max<size_t>(1, bytes / kDeliverChunk));
    if (k <= 1 || n < (size_t)k) {
      deliver_range(&fl, 0, n);
    } else {
      std::vector<std::thread> th;
      for (int t = 1; t < k; t++) th.emplace_back(deliver_range, &fl, n * t / k, n * (t + 1) / k);
      deliver_range(&fl, 0, n / k);
      for (auto& t : th) t.join();
    }
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& q : fl.reqs) {
      s->status[(size_t)q.id] = err ? err : 1;
      s->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - q.t_submit).count());
    }
    s->completed += (int64_t)fl.reqs.size();
    if (err) {
      s->last_error = err;
      s->err_msg = fl.err_msg;
    }
  }
  s->cv_done.notify_all();
}

void completer_main(Server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    InFlight* fl = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu_c);
      s->cv_c.wait(lk, [&] { return !s->launched.empty() || s->stop; });
      if (s->launched.empty()) return;
      fl = s->launched.front();
      s->launched.pop_front();
    }
    const auto t_done = Clock::now();
    if (fl->done) {
      const cudaError_t e = cudaEventSynchronize(fl->done);
      if (e != cudaSuccess) {
        fl->err = FPCC_ECUDA;
        fl->err_msg = std::string("server: batch completion: ") + cudaGetErrorString(e);
      }
    }
    deliver(s, *fl);
    s->deliver_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t_done).count();
    {
      std::lock_guard<std::mutex> lk(s->mu_c);
      s->retired.push_back(fl);
    }
    s->cv_c.notify_all();
    s->cv.notify_all();
  }
}

// Worker side: release pins and pinned buffers of retired batches.
void release_retired(Server* s) {
  std::deque<InFlight*> done;
  {
    std::lock_guard<std::mutex> lk(s->mu_c);
    done.swap(s->retired);
  }
  for (InFlight* fl : done) {
    for (auto& pr : fl->pinned_rows) pr.first->pin[pr.second]--;
    if (fl->d_out) dfree(s, fl->d_out);   // the batch is complete: its downloads have ended
    if (fl->h_out) pinned_put(s, fl->h_out, fl->h_bytes);
    if (fl->h_up) pinned_put(s, fl->h_up, fl->up_bytes);
    for (auto& b : fl->up_full) pinned_put(s, b.first, b.second);
    if (fl->done) cudaEventDestroy(fl->done);
    delete fl;
    s->in_flight--;
  }
}

void wait_one_retired(Server* s) {
  {
    std::unique_lock<std::mutex> lk(s->mu_c);
    s->cv_c.wait_for(lk, std::chrono::milliseconds(1), [&] { return !s->retired.empty(); });
  }
  release_retired(s);
}

constexpr int kMaxInFlight = 3;
constexpr auto kLingerStep = std::chrono::microseconds(25);
constexpr auto kLingerMax = std::chrono::microseconds(400);

void worker_main(Server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    release_retired(s);
    std::vector<Req> batch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->pending.empty()) {
        s->cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return s->stop || !s->pending.empty(); });
        if (s->pending.empty()) {
          if (s->stop) {
            lk.unlock();
            // wait for the completers to drain what is in flight
            for (;;) {
              release_retired(s);
              if (s->in_flight == 0) return;
              std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
          }
          continue;
        }
      }
      // While earlier batches keep the GPU busy and requests keep arriving,
      // let this batch grow (continuous batching); an idle GPU starts at once.
      const auto t0 = Clock::now();
      while (s->in_flight > 0 && (int)s->pending.size() < s->max_batch && Clock::now() - t0 < kLingerMax) {
        const size_t before = s->pending.size();
        s->cv.wait_for(lk, kLingerStep);
        if (s->pending.size() == before) break;
      }
      while (!s->pending.empty() && (int)batch.size() < s->max_batch) {
        batch.push_back(std::move(s->pending.front()));
        s->pending.pop_front();
      }
    }
    // bound the number of batches in flight
    while (s->in_flight >= kMaxInFlight) wait_one_retired(s);
    const auto t_form = Clock::now();
    InFlight* fl = new InFlight();
    fl->srv = s;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (auto& r : s->out_ranges) fl->out_ranges.push_back({std::get<0>(r), std::get<1>(r)});
    }
    std::map<GroupKey, std::vector<Req*>> groups;
    {
      std::vector<Req*>* last = nullptr;   // requests in a row usually share their group
      GroupKey last_key{};
      for (auto& q : batch) {
        const int m = q.r.method;
        const float v = m == FPCC_PCCV ? q.r.v : 0.f;
        const int f = product_fmt(s, m);
        // packed groups carry N = -1 (lengths and lags per request)
        GroupKey g = packable(m, q.Nz) ? GroupKey{m, -1, q.Nz, 0, 0, f, v, 0}
                                       : GroupKey{m, q.N, q.Nz, q.lag0, q.L, f, v, q.aux};
        if (!last || g < last_key || last_key < g) {
          last = &groups[g];
          last_key = g;
        }
        last->push_back(&q);
      }
    }
    size_t total = 0;
    for (auto& q : batch) total += (size_t)q.L * (q.r.method == FPCC_CC1B_POPCOUNT ? 8 : 4);
    fl->h_out = (char*)pinned_get(s, total, &fl->h_bytes);
    // the batch's device results (freed when the batch retires); without it the
    // groups share one scratch buffer and download on the server's stream
    fl->d_out = s->st_out ? dalloc(s, std::max<size_t>(total, 256)) : nullptr;
    s->out_used = 0;
    fl->h_up = (char*)pinned_get(s, (size_t)(16 * 4 + sizeof(fpcc_pair_desc)) * batch.size() +
                                     1024 * (groups.size() + 4 + 2 * s->lanes.size()),
                                 &fl->up_bytes);
    int err = (fl->h_out && fl->h_up) ? 0 : no_mem("server: pinned result or upload buffer of a batch");
    fl->reqs.reserve(batch.size());
    // Station products first, all on the lanes: the phase products of the
    // packed groups in packed stages (one kind at a time, the direct sums'
    // phase signals first), then every other group's products.  A packed
    // direct-sum group starts its pair stage on the direct-sum lane as soon as
    // its products are queued; the other pair stages follow on the server's
    // stream, each after the lane work that made its own products.  Groups go
    // direct-sum methods first: theirs are the longest pair stages, and they
    // overlap the later groups' station stages.
    std::vector<std::pair<const GroupKey, std::vector<Req*>>*> order;
    for (auto& kv : groups) order.push_back(&kv);
    std::stable_partition(order.begin(), order.end(), [](const std::pair<const GroupKey, std::vector<Req*>>* kv) {
      const int m = kv->first.method;
      return m == FPCC_PCC1 || m == FPCC_PCCV || m == FPCC_CC1B_POPCOUNT;
    });
    s->ev_used = 0;
    std::vector<std::vector<cudaEvent_t>> waits(order.size());
    std::vector<cudaEvent_t> marks6, marks1;
    std::vector<int> used;
    if (!err) {
      std::vector<std::pair<int, std::vector<Req*>*>> ph[2];
      for (auto* kv : order) {
        const GroupKey& g = kv->first;
        if (g.N >= 0) continue;
        if (g.method == FPCC_PCC2) ph[0].push_back({g.Nz, &kv->second});
        else if (g.method == FPCC_PCC1 || g.method == FPCC_PCCV) ph[1].push_back({0, &kv->second});
      }
      const int f = product_fmt(s, FPCC_PCC2);
      s->lane_rec = &used;
      if (!ph[1].empty()) err = prefetch_phase(s, 6, f, ph[1], *fl);
      lane_marks(s, used, marks6);
      if (!err && !ph[0].empty()) err = prefetch_phase(s, 1, f, ph[0], *fl);
      lane_marks(s, used, marks1);
      s->lane_rec = nullptr;
    }
    // output offsets of every group, in group order
    std::vector<size_t> base(order.size()), first(order.size());
    {
      size_t off = 0;
      for (size_t i = 0; i < order.size(); i++) {
        base[i] = off;
        first[i] = fl->reqs.size();
        for (Req* q : order[i]->second) {
          fl->reqs.push_back(*q);
          fl->out_off.push_back((int64_t)off);
          off += (size_t)q->L * (q->r.method == FPCC_CC1B_POPCOUNT ? 8 : 4);
        }
      }
      fl->direct.assign(fl->reqs.size(), 0);
    }
    // a packed direct-sum group starts its pair stage on the direct lane as
    // soon as its own products are queued, overlapping the later station stages
    std::vector<char> early(order.size(), 0);
    std::vector<GroupRows> grows(order.size());
    for (size_t i = 0; i < order.size(); i++) {
      if (err) break;
      const GroupKey& g = order[i]->first;
      if (g.method == FPCC_WPCC) continue;
      s->lane_rec = &used;
      err = (g.N < 0) ? run_group_packed(s, g, order[i]->second, *fl, 0, true, nullptr, 0, &grows[i])
                      : run_group(s, g, order[i]->second, *fl, 0, true, 0, &grows[i]);
      s->lane_rec = nullptr;
      lane_marks(s, used, waits[i]);
      if (g.N < 0 && g.method == FPCC_PCC2) waits[i].insert(waits[i].end(), marks1.begin(), marks1.end());
      if (g.N < 0 && (g.method == FPCC_PCC1 || g.method == FPCC_PCCV))
        waits[i].insert(waits[i].end(), marks6.begin(), marks6.end());
      const bool direct = g.method == FPCC_PCC1 || g.method == FPCC_PCCV || g.method == FPCC_CC1B_POPCOUNT;
      if (!err && direct && g.N < 0 && s->dlane.ctx) {
        s->pair_waits = &waits[i];
        s->pair_seq = s->lane_seq;
        err = run_group_packed(s, g, order[i]->second, *fl, base[i], false, &s->dlane, first[i], &grows[i]);
        s->pair_waits = nullptr;
        early[i] = 1;
        s->pair_stages++;
      }
    }
    for (size_t i = 0; i < order.size(); i++) {
      if (err) break;
      if (early[i]) continue;
      auto& kv = *order[i];
      const size_t base_i = base[i];
      const GroupKey& g = kv.first;
      s->pair_waits = &waits[i];
      s->pair_seq = s->lane_seq;
      if (g.method == FPCC_WPCC) err = run_group_wpcc(s, g, kv.second, *fl, base_i, first[i]);
      else if (g.N < 0) err = run_group_packed(s, g, kv.second, *fl, base_i, false, nullptr, first[i], &grows[i]);
      else err = run_group(s, g, kv.second, *fl, base_i, false, first[i], &grows[i]);
      s->pair_waits = nullptr;
      s->pair_stages++;
    }
    // later batches' lane work and slab frees follow everything of this one
    lanes_join(s);
    if (err) {
      lanes_join(s);
      cudaStreamSynchronize(s->st);
      if (s->st_out) cudaStreamSynchronize(s->st_out);
      fl->reqs.clear();
      for (auto& q : batch) fl->reqs.push_back(q);
      fl->direct.assign(fl->reqs.size(), 0);
      fl->err = err;
      fl->err_msg = fpcc_last_error();
    } else {
      cudaEventCreateWithFlags(&fl->done, cudaEventDisableTiming);
      if (fl->d_out) {
        // done = the server's stream and the results stream both past this batch
        cudaEventRecord(s->main_ev, s->st);
        cudaStreamWaitEvent(s->st_out, s->main_ev, 0);
        cudaEventRecord(fl->done, s->st_out);
      } else {
        cudaEventRecord(fl->done, s->st);
      }
      s->batches++;
    }
    s->in_flight++;
    s->worker_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t_form).count();
    {
      std::lock_guard<std::mutex> lk(s->mu_c);
      s->launched.push_back(fl);
    }
    s->cv_c.notify_one();
  }
}

}  // namespace
}  // namespace fpcc

using namespace fpcc;

extern "C" int fpcc_server_create(fpcc_server** out, int device, size_t hbm_budget_bytes, int max_batch) {
  if (!out) return FPCC_EARG;
  Server* s = new Server();
  s->device = device;
  s->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)150 << 30;
  s->max_batch = max_batch > 0 ? max_batch : 4096;
  s->chunk_bytes = std::min<size_t>((size_t)64 << 20, std::max<size_t>((size_t)1 << 20, s->budget / 8)) &
                   ~(size_t)255;
  // one pool for the slabs and for the scratch of every context of the server
  // (the main one and the lanes): freed blocks stay mapped up to the budget and a
  // quarter again, and memory one lane frees serves the others
  cudaMemPoolProps pp = {};
  pp.allocType = cudaMemAllocationTypePinned;
  pp.location.type = cudaMemLocationTypeDevice;
  pp.location.id = device;
  uint64_t keep = (uint64_t)s->budget + (uint64_t)s->budget / 4;
  if (cudaSetDevice(device) != cudaSuccess || cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess ||
      cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return cuda_err(cudaGetLastError(), "row copy");
  }
  auto undo = [s]() {
    for (auto& l : s->lanes) {
      fpcc_destroy(l.ctx);
      if (l.ev) cudaEventDestroy(l.ev);
    }
    if (s->dlane.ctx) fpcc_destroy(s->dlane.ctx);
    if (s->dlane.ev) cudaEventDestroy(s->dlane.ev);
    if (s->main_ev) cudaEventDestroy(s->main_ev);
    if (s->st_out) cudaStreamDestroy(s->st_out);
    if (s->ctx) fpcc_destroy(s->ctx);
    cudaMemPoolDestroy(s->pool);
    delete s;
    return cuda_err(cudaGetLastError(), "row copy");
  };
  if (fpcc_create(&s->ctx, device)) {
    s->ctx = nullptr;
    return undo();
  }
  ctx_share_pool(s->ctx, s->pool);
  s->st = (cudaStream_t)fpcc_get_stream(s->ctx);
  if (cudaEventCreateWithFlags(&s->main_ev, cudaEventDisableTiming) != cudaSuccess) {
    s->main_ev = nullptr;
    return undo();
  }
  if (cudaStreamCreateWithFlags(&s->st_out, cudaStreamNonBlocking) != cudaSuccess) {
    s->st_out = nullptr;
    return undo();
  }
  // FPCC_SERVER_LANES sets the number of lanes (0: everything on the server's stream)
  int nlanes = kLanes;
  if (const char* e = getenv("FPCC_SERVER_LANES")) nlanes = std::max(0, std::min(16, atoi(e)));
  for (int i = 0; i < nlanes; i++) {
    Lane l;
    if (fpcc_create(&l.ctx, device)) return undo();
    ctx_share_pool(l.ctx, s->pool);
    l.st = (cudaStream_t)fpcc_get_stream(l.ctx);
    s->lanes.push_back(l);
    if (cudaEventCreateWithFlags(&s->lanes.back().ev, cudaEventDisableTiming) != cudaSuccess) {
      s->lanes.back().ev = nullptr;
      return undo();
    }
  }
  if (nlanes > 0) {
    if (fpcc_create(&s->dlane.ctx, device)) {
      s->dlane.ctx = nullptr;
      return undo();
    }
    ctx_share_pool(s->dlane.ctx, s->pool);
    s->dlane.st = (cudaStream_t)fpcc_get_stream(s->dlane.ctx);
    if (cudaEventCreateWithFlags(&s->dlane.ev, cudaEventDisableTiming) != cudaSuccess) {
      s->dlane.ev = nullptr;
      return undo();
    }
  }
  // map a first reserve of the pool now, at start-up, rather than block by
  // block under the first batches
  void* warm = nullptr;
  const size_t reserve = std::min<size_t>((size_t)2 << 30, s->budget / 4);
  if (reserve && cudaMallocFromPoolAsync(&warm, reserve, s->pool, s->st) == cudaSuccess) {
    cudaFreeAsync(warm, s->st);
    cudaStreamSynchronize(s->st);
  } else {
    cudaGetLastError();
  }
  s->worker = std::thread(worker_main, s);
  for (int i = 0; i < 4; i++) s->completers.emplace_back(completer_main, s);
  *out = reinterpret_cast<fpcc_server*>(s);
  return 0;
}

extern "C" int fpcc_server_register_output(fpcc_server* h, void* p, size_t bytes) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !p || !bytes) return FPCC_EARG;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(s->device);
  bool owned = false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterPortable);
    if (e != cudaSuccess) {
      cudaSetDevice(prev);
      return cuda_err(e, "registering a result buffer");
    }
    owned = true;
  }
  cudaSetDevice(prev);
  std::lock_guard<std::mutex> lk(s->mu);
  s->out_ranges.emplace_back((char*)p, bytes, owned);
  return 0;
}

extern "C" int fpcc_server_unregister_output(fpcc_server* h, void* p) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !p) return FPCC_EARG;
  bool owned = false, found = false;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t i = 0; i < s->out_ranges.size(); i++)
      if (std::get<0>(s->out_ranges[i]) == (char*)p) {
        owned = std::get<2>(s->out_ranges[i]);
        s->out_ranges.erase(s->out_ranges.begin() + (ptrdiff_t)i);
        found = true;
        break;
      }
  }
  if (!found) return FPCC_EARG;
  if (owned) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    const cudaError_t e = cudaHostUnregister(p);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_err(e, "unregistering a result buffer");
  }
  return 0;
}

extern "C" int fpcc_server_destroy(fpcc_server* h) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->mu_c);
  }
  s->cv_c.notify_all();
  for (auto& t : s->completers) t.join();
  cudaSetDevice(s->device);
  for (auto& kv : s->slabs) slab_free(s, kv.second.base, (size_t)kv.second.cap * kv.second.row_bytes);
  for (auto& c : s->chunks.chunks()) dfree(s, c.base);
  for (void** p : {&s->d_tmp_x, &s->d_tmp_p, &s->d_idx, &s->d_y, &s->d_pl, &s->d_desc}) dfree(s, *p);
  for (auto& kv : s->wplans) fpcc_wpcc_plan_destroy(kv.second);
  for (auto& r : s->out_ranges)
    if (std::get<2>(r)) cudaHostUnregister(std::get<0>(r));
  s->out_ranges.clear();
  // the contexts share the server's pool: they go first, the pool last
  for (auto& l : s->lanes) {
    if (l.d_tmp) cudaFreeAsync(l.d_tmp, l.st);
    if (l.d_idx) cudaFreeAsync(l.d_idx, l.st);
    fpcc_destroy(l.ctx);   // frees its buffers and waits for its stream
    cudaEventDestroy(l.ev);
  }
  if (s->dlane.ctx) {
    if (s->dlane.d_tmp) cudaFreeAsync(s->dlane.d_tmp, s->dlane.st);
    if (s->dlane.d_idx) cudaFreeAsync(s->dlane.d_idx, s->dlane.st);
    fpcc_destroy(s->dlane.ctx);
    cudaEventDestroy(s->dlane.ev);
  }
  cudaStreamSynchronize(s->st);
  if (s->st_out) {
    cudaStreamSynchronize(s->st_out);
    cudaStreamDestroy(s->st_out);
  }
  fpcc_destroy(s->ctx);
  cudaMemPoolDestroy(s->pool);
  for (size_t i = 0; i < s->pinned_pool.size(); i += 2) cudaFreeHost(s->pinned_pool[i]);
  for (char* a : s->arena) cudaFreeHost(a);
  if (s->main_ev) cudaEventDestroy(s->main_ev);
  for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : s->out_ev) cudaEventDestroy(e);
  delete s;
  return 0;
}

extern "C" int fpcc_server_set_format(fpcc_server* h, int fmt) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || (fmt != FPCC_F32 && fmt != FPCC_F16 && fmt != FPCC_I16)) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->next_id) return FPCC_EARG;   // before the first request
  s->fmt = fmt;
  return 0;
}

extern "C" int fpcc_server_set_nz_mode(fpcc_server* h, int mode) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || mode < FPCC_NZ_TUNED || mode > FPCC_NZ_FAST) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->next_id) return FPCC_EARG;
  s->nz_mode = mode;
  return 0;
}

extern "C" int fpcc_server_set_wavelet(fpcc_server* h, double pmin, double pmax, unsigned V, int type, double op1,
                                       int rule) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return FPCC_EARG;
  // the scale count is fixed by pmin, pmax, V and type; probe it on a long window
  WpccSetup su;
  if (wpcc_setup(1u << 20, 0, 0, pmin, pmax, V, type, op1, &su) != 0) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->next_id) return FPCC_EARG;
  s->wav.set = true;
  s->wav.pmin = pmin;
  s->wav.pmax = pmax;
  s->wav.V = V;
  s->wav.type = type;
  s->wav.op1 = op1;
  s->wav.rule = rule;
  s->wav.S = (int)su.wf.S;
  s->wsetup.clear();
  return 0;
}

extern "C" int fpcc_put_station_window(fpcc_server* h, int32_t sta, int32_t window, const float* x, int N) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !x || N <= 0) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  const size_t bytes = ((size_t)N * 4 + 255) & ~size_t(255);
  if (bytes > s->arena_left) {
    const size_t chunk = std::max(bytes, (size_t)64 << 20);
    char* p = nullptr;
    if (cudaMallocHost(&p, chunk) != cudaSuccess) return FPCC_ENOMEM;
    s->arena.push_back(p);
    s->arena_ptr = p;
    s->arena_left = chunk;
  }
  float* dst = (float*)s->arena_ptr;
  s->arena_ptr += bytes;
  s->arena_left -= bytes;
  memcpy(dst, x, (size_t)N * 4);
  int zeros = 0;
  for (int n = 0; n < N; n++) zeros += (x[n] == 0.0f);
  s->windows[{sta, window}] = Server::Window{dst, N, zeros, (int)s->arena.size() - 1};
  return 0;
}

namespace fpcc {
namespace {

// Validates a request and fills its planning fields (window length, padded
// length, lags).  `mu` is taken for the window and wavelet-setup lookups only.
// Window length of a request's two windows (FPCC_EARG if either is missing or
// they differ); the caller holds `mu`.
// *f64 (when given) receives the windows' FP64 flags (Req::f64).
int request_window_len(Server* s, const fpcc_request* req, int* f64 = nullptr) {
  auto a = s->windows.find({req->sta1, req->window});
  auto b = s->windows.find({req->sta2, req->window});
  if (a == s->windows.end() || b == s->windows.end()) return FPCC_EARG;
  if (b->second.N != a->second.N) return FPCC_EARG;
  if (f64)
    *f64 = (a->second.zeros >= FPCC_F64_ZERO_SAMPLES ? 1 : 0) | (b->second.zeros >= FPCC_F64_ZERO_SAMPLES ? 2 : 0);
  return a->second.N;
}

// As prepare_request, for a window length already looked up.
int prepare_request_n(Server* s, const fpcc_request* req, Req& q, int N);

int prepare_request(Server* s, const fpcc_request* req, Req& q) {
  int N = 0, f64 = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    N = request_window_len(s, req, &f64);
  }
  if (N < 0) return N;
  q.f64 = f64;
  return prepare_request_n(s, req, q, N);
}

int prepare_request_n(Server* s, const fpcc_request* req, Req& q, int N) {
  q.r = *req;
  const int M = std::max(std::abs(req->Lag1), std::abs(req->Lag2));
  if (M >= N) return FPCC_EARG;
  q.N = N;
  q.lag0 = std::min(req->Lag1, req->Lag2);
  q.L = std::abs(req->Lag2 - req->Lag1) + 1;
  const int m = req->method;
  if (m == FPCC_PCC2 || m == FPCC_GNCC || m == FPCC_CC1B) {
    q.Nz = choose_nz(N, M, s->nz_mode);
    if (q.Nz <= 0) return FPCC_EUNSUP;
  } else if (m == FPCC_PCC1 || m == FPCC_PCCV || m == FPCC_CC1B_POPCOUNT) {
    q.Nz = 0;
    if ((m == FPCC_PCC1 || m == FPCC_PCCV) && req->Lag1 > req->Lag2) return FPCC_EARG;
  } else if (m == FPCC_WPCC) {
    std::pair<int, int> nz{0, 0};
    bool known = false;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (!s->wav.set) return FPCC_EARG;
      auto it = s->wsetup.find({N, M});
      if (it != s->wsetup.end()) { nz = it->second; known = true; }
    }
    if (!known) {
      WpccSetup su;
      if (wpcc_setup((unsigned)N, req->Lag1, req->Lag2, s->wav.pmin, s->wav.pmax, s->wav.V, s->wav.type,
                     s->wav.op1, &su) != 0)
        return FPCC_EARG;
      nz.first = wpcc_choose_nz(su, (unsigned)N, FPCC_NZ_FAST);
      bool capped = false;
      for (unsigned k = 0; k < su.wf.S; k++) capped |= (su.wf.Ls[k] >= su.Nz0);
      nz.second = capped ? (int)su.Nz0 : 0;   // the family depends on the cap only when a length hit it
      if (nz.first <= 0) return FPCC_EUNSUP;
      std::lock_guard<std::mutex> lk(s->mu);
      s->wsetup[{N, M}] = nz;
    }
    q.Nz = nz.first;
    q.aux = nz.second;
  } else {
    return FPCC_EUNSUP;
  }
  return 0;
}

}  // namespace
}  // namespace fpcc

extern "C" int64_t fpcc_submit(fpcc_server* h, const fpcc_request* req) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !req) return FPCC_EARG;
  Req q;
  if (int rc = prepare_request(s, req, q)) return rc;
  q.t_submit = Clock::now();
  bool wake;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    q.id = s->next_id++;
    s->status.push_back(0);
    // the worker sleeps only on an empty queue (a batch it lingers over is
    // re-checked on a short timeout), so only the first request wakes it
    wake = s->pending.empty();
    s->pending.push_back(q);
  }
  if (wake) s->cv.notify_one();
  return q.id;
}

extern "C" int fpcc_poll(fpcc_server* h, int64_t id) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->status.size()) return FPCC_EARG;
  const int st = s->status[(size_t)id];
  if (st < 0) set_last_error(s->err_msg.c_str());
  return st;
}

extern "C" int fpcc_wait(fpcc_server* h, int64_t id, double timeout_s) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return FPCC_EARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->status.size()) return FPCC_EARG;
  auto pred = [&] { return s->status[(size_t)id] != 0; };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return 0;
  } else {
    s->cv_done.wait(lk, pred);
  }
  const int st = s->status[(size_t)id];
  if (st < 0) set_last_error(s->err_msg.c_str());
  return st;
}

extern "C" int fpcc_server_drain(fpcc_server* h) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return FPCC_EARG;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->pending.empty() && s->completed >= s->next_id; });
  if (s->last_error) set_last_error(s->err_msg.c_str());
  return s->last_error;
}

extern "C" int fpcc_server_get_stats(fpcc_server* h, fpcc_server_stats* o) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !o) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> v = s->lat_ms;
  std::sort(v.begin(), v.end());
  auto pct = [&](double p) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
  o->completed = s->completed;
  o->batches = s->batches;
  o->station_rows = s->station_rows;
  o->hbm_used = (int64_t)s->used;
  o->p50_ms = pct(0.50);
  o->p99_ms = pct(0.99);
  o->max_ms = v.empty() ? 0.0 : v.back();
  o->pair_stages = s->pair_stages;
  o->worker_ms = (double)s->worker_ns.load() * 1e-6;
  o->deliver_ms = (double)s->deliver_ns.load() * 1e-6;
  return 0;
}

extern "C" int fpcc_server_reset_stats(fpcc_server* h) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s) return FPCC_EARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat_ms.clear();
  s->batches = 0;
  s->station_rows = 0;
  s->pair_stages = 0;
  s->worker_ns = 0;
  s->deliver_ns = 0;
  return 0;
}

extern "C" int fpcc_submit_many(fpcc_server* h, const fpcc_request* reqs, int n, int64_t* ids) {
  Server* s = reinterpret_cast<Server*>(h);
  if (!s || !reqs || n < 0) return FPCC_EARG;
  // chunks of requests enter the queue under one lock and one wake-up each, so
  // that the worker can start on the first chunk while the rest are prepared
  constexpr int kChunk = 1024;
  std::vector<Req> qs;
  std::vector<int> lens, f64s;
  qs.reserve(std::min(n, kChunk));
  for (int i0 = 0; i0 < n; i0 += kChunk) {
    const int i1 = std::min(n, i0 + kChunk);
    qs.clear();
    int rc = 0, bad = i1;
    lens.resize((size_t)(i1 - i0));
    f64s.resize((size_t)(i1 - i0));
    {
      std::lock_guard<std::mutex> lk(s->mu);   // the chunk's window lookups under one lock
      for (int i = i0; i < i1; i++)
        lens[(size_t)(i - i0)] = request_window_len(s, reqs + i, &f64s[(size_t)(i - i0)]);
    }
    for (int i = i0; i < i1; i++) {
      Req q;
      q.f64 = f64s[(size_t)(i - i0)];
      const int N = lens[(size_t)(i - i0)];
      if ((rc = (N < 0) ? N : prepare_request_n(s, reqs + i, q, N))) {
        bad = i;
        break;
      }
      qs.push_back(q);
    }
    const auto now = Clock::now();
    bool wake;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      wake = s->pending.empty();
      for (size_t k = 0; k < qs.size(); k++) {
        Req& q = qs[k];
        q.t_submit = now;
        q.id = s->next_id++;
        s->status.push_back(0);
        if (ids) ids[i0 + (int)k] = q.id;
        s->pending.push_back(std::move(q));
      }
    }
    if (wake) s->cv.notify_one();
    if (rc) {
      if (ids) ids[bad] = rc;
      return rc;
    }
  }
  return 0;
}

// Offer the requests at Poisson arrival times of the given rate (requests/s)
// from the calling thread; returns when the last one has been submitted.
extern "C" int fpcc_server_offer_poisson(fpcc_server* h, const fpcc_request* reqs, int n, double rate,
                                         uint64_t seed, int64_t* ids) {
  if (!h || !reqs || n < 0 || !(rate > 0)) return FPCC_EARG;
  uint64_t x = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto next = [&]() {   // xorshift64* uniform in (0,1)
    x ^= x >> 12; x ^= x << 25; x ^= x >> 27;
    return ((x * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0) + 1e-18;
  };
  const auto t0 = Clock::now();
  double t = 0;
  for (int i = 0; i < n; i++) {
    t += -std::log(next()) / rate;
    const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t));
    while (Clock::now() < due) {
      const auto left = due - Clock::now();
      if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
    }
    const int64_t id = fpcc_submit(h, reqs + i);
    if (ids) ids[i] = id;
    if (id < 0) return (int)id;
  }
  return 0;
}
