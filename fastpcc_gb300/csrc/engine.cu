// Host-side planning: radix schedules and padded correlation lengths.
#include <math.h>

#include <algorithm>
#include <map>
#include <atomic>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.h"
#include "menu.cuh"
#include "large.cuh"

namespace fpcc {

bool factor235(int n, int* a, int* b, int* c) {
  if (n < 1) return false;
  *a = *b = *c = 0;
  while (n % 2 == 0) { n /= 2; (*a)++; }
  while (n % 3 == 0) { n /= 3; (*b)++; }
  while (n % 5 == 0) { n /= 5; (*c)++; }
  return n == 1;
}

std::vector<int> smooth235_in(int lo, int hi) {
  std::vector<int> v;
  if (lo < 1) lo = 1;
  if (hi < lo) return v;
  for (int64_t p5 = 1; p5 <= hi; p5 *= 5)
    for (int64_t p3 = p5; p3 <= hi; p3 *= 3)
      for (int64_t p2 = p3; p2 <= hi; p2 *= 2)
        if (p2 >= lo) v.push_back((int)p2);
  std::sort(v.begin(), v.end());
  return v;
}

static void encode(FftPlan* p) {
  p->code = 0;
  for (int i = p->npass - 1; i >= 0; i--) p->code = (p->code << 5) | (uint64_t)p->rad[i];
}

bool make_plan(int n, FftPlan* p, const int* forced, int nforced) {
  const bool ok = make_plan_raw(n, p, forced, nforced);
  encode(p);
  return ok;
}

bool make_plan_raw(int n, FftPlan* p, const int* forced, int nforced) {
  p->n = n;
  p->npass = 0;
  if (forced) {
    long prod = 1;
    for (int i = 0; i < nforced && i < kMaxPass; i++) {
      p->rad[p->npass++] = forced[i];
      prod *= forced[i];
    }
    return prod == n;
  }
  int a, b, c;
  if (!factor235(n, &a, &b, &c)) return false;
  if (n == 1) return true;
  const int np2 = (a + 3) / 4;
  for (int i = 0; i < np2; i++) {
    // spread the exponent a over np2 passes as evenly as possible
    const int e = a / np2 + (i < a % np2 ? 1 : 0);
    p->rad[p->npass++] = 1 << e;
  }
  for (int i = 0; i < c; i++) p->rad[p->npass++] = 5;
  for (int i = 0; i < b; i++) p->rad[p->npass++] = 3;
  return p->npass <= kMaxPass;
}

double plan_cost(int n) {
  FftPlan p;
  if (!make_plan(n, &p)) return 1e30;
  double c = 0;
  for (int i = 0; i < p.npass; i++) {
    // one shared-memory round trip per pass plus the butterfly work per point
    const int R = p.rad[i];
    c += 1.0 + 0.35 * log2((double)R) + (R == 3 || R == 5 ? 0.6 : 0.0);
  }
  return c * (double)n;
}

// A transform length is usable when it runs in one block (menu) or as a
// four-step transform; the cost model charges the four-step form its two extra
// global-memory passes.
static bool usable(int n) {
  int n1, n2;
  return on_menu(n) || large_supported(n, &n1, &n2);
}

static double length_cost(int n) {
  if (on_menu(n)) return plan_cost(n);
  int n1, n2;
  if (!large_supported(n, &n1, &n2)) return 1e30;
  return plan_cost(n1) * (double)(n / n1) + plan_cost(n2) * (double)(n / n2) + 4.0 * (double)n;
}

bool nz_usable(int nz) { return nz > 0 && (nz % 2) == 0 && usable(nz) && usable(nz / 2); }

static int choose_nz_uncached(int N, int M, int mode);

// Memoised: the serving loop asks once per request.
static std::mutex g_memo_mu;
static std::map<std::tuple<int, int, int>, int> g_memo;
// generation of g_memo (bumped whenever it is cleared), so that a thread's
// copy of its last answer is used only while the memo it came from stands
static std::atomic<uint64_t> g_memo_gen{1};

// Measured costs per padded length (autotuner): pair stage per correlation and
// station stage per window, in ns; a length's cost is pair + station / reuse.
static std::mutex g_tune_mu;
static std::map<int, std::pair<double, double>> g_tuned;
static double g_reuse = 8.0;

void tuned_set(int nz, double pair_ns, double station_ns) {
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[nz] = {pair_ns, station_ns};
  }
  std::lock_guard<std::mutex> lk(g_memo_mu);
  g_memo.clear();
  g_memo_gen.fetch_add(1);
}

void tuned_set_reuse(double reuse) {
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_reuse = reuse > 0 ? reuse : 8.0;
  }
  std::lock_guard<std::mutex> lk(g_memo_mu);
  g_memo.clear();
  g_memo_gen.fetch_add(1);
}

std::vector<std::tuple<int, double, double>> tuned_table(double* reuse) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::vector<std::tuple<int, double, double>> v;
  for (auto& kv : g_tuned) v.emplace_back(kv.first, kv.second.first, kv.second.second);
  if (reuse) *reuse = g_reuse;
  return v;
}


std::vector<int> usable_lengths(int lo, int hi) {
  std::vector<int> v;
  for (int nz : smooth235_in(lo, hi))
    if (!(nz & 1) && nz_usable(nz)) v.push_back(nz);
  return v;
}

int choose_nz(int N, int M, int mode) {
  const auto key = std::make_tuple(N, M, mode);
  // requests in a row usually ask the same question (one per request when serving)
  thread_local std::tuple<int, int, int> last_key{-1, -1, -1};
  thread_local int last_nz = 0;
  thread_local uint64_t last_gen = 0;
  const uint64_t gen = g_memo_gen.load(std::memory_order_acquire);
  if (gen == last_gen && key == last_key) return last_nz;
  {
    std::lock_guard<std::mutex> lk(g_memo_mu);
    auto it = g_memo.find(key);
    if (it != g_memo.end()) {
      last_key = key;
      last_nz = it->second;
      last_gen = gen;
      return it->second;
    }
  }
  int nz = choose_nz_uncached(N, M, mode);
  if (nz <= 0 && mode == FPCC_NZ_TUNED_MODE) nz = choose_nz_uncached(N, M, 1);
  std::lock_guard<std::mutex> lk(g_memo_mu);
  g_memo[key] = nz;
  return nz;
}

static int choose_nz_uncached(int N, int M, int mode) {
  const int need = N + M;
  if (mode == FPCC_NZ_TUNED_MODE) {
    // the measured cheapest length among those the autotuner timed
    int best = -1;
    double bc = 1e300;
    const int hi = std::min(2 * need + 64, 1 << 21);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto it = g_tuned.lower_bound(need + (need & 1)); it != g_tuned.end() && it->first <= hi; ++it) {
      if (it->first & 1) continue;
      const double c = it->second.first + it->second.second / g_reuse;
      if (c < bc) { bc = c; best = it->first; }
    }
    return best;
  }
  if (mode >= 2) {
    // explicit padded length
    return (mode >= need && nz_usable(mode)) ? mode : -1;
  }
  if (mode == 0) {
    const int nz = 1 << (int)ceil(log2((double)need));
    return nz_usable(nz) ? nz : -1;
  }
  // candidates: menu lengths and four-step lengths 2^a 3^b 5^c up to 2^20
  int best = -1;
  double bc = 1e300;
  for (int nz : smooth235_in(need, std::min(2 * need + 64, 1 << 21))) {
    if ((nz & 1) || !nz_usable(nz)) continue;
    // the pair transform (Nz/2) dominates a batch of correlations
    const double cost = length_cost(nz / 2) + 0.1 * length_cost(nz);
    if (cost < bc) { bc = cost; best = nz; }
  }
  return best;
}

int conv_class_len(int N) {
  const int need = 2 * N - 1;
  int best = -1;
  for (int base : {1, 3, 5})
    for (long long m = base; m <= (1LL << 26); m *= 2)
      if (m >= need) {
        if (best < 0 || m < best) best = (int)m;
        break;
      }
  return best;
}

}  // namespace fpcc
