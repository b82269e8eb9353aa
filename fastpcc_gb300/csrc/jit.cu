// Run-time specialisation of the fused station kernel (see fused.cuh).
//
// The window length of a workload is data (18000 here, 36000 there, any length
// in a serving stream), so the fused kernel's radix schedule for N cannot be
// fixed when the library is built.  On first use of an (N, Nz) the host picks a
// schedule for each length (fewest passes over the in-register radices whose
// staging stays within 24 complex values per thread), instantiates k_station_fused with it through
// NVRTC for sm_103a, and caches the cubin in memory and under the disk cache
// directory (FPCC_JIT_CACHE, default ~/.cache/fastpcc_gb300).  FPCC_JIT=0
// disables the path.  For even N the real window's DFT_N runs as an N/2-point
// complex transform (k_station_fused_real).
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <tuple>
#include <vector>

#include "engine.h"
#include "fused.cuh"
#include "jit.h"
#include "jit_source.inc"

#ifndef FPCC_CUDA_INCLUDE
#define FPCC_CUDA_INCLUDE "/usr/local/cuda/include"
#endif

namespace fpcc {
namespace {

constexpr int kStageCap = 24;        // complex values staged per thread per pass
constexpr long long kMaxSmem = 227 * 1024;

struct Entry {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t fn = nullptr;
  int T = 0;
  long long smem = 0;
  bool failed = false;
};

std::mutex g_mu;
std::map<std::tuple<int, int, int>, Entry> g_cache;   // (device, N, Nz)

int ceil_div(int a, int b) { return (a + b - 1) / b; }

bool stage_ok(int n, int R, int T) { return ceil_div(n / R, T) * R <= kStageCap; }

// Radix schedule for n with T threads, or empty when none fits: the fewest
// passes (each pass is a round trip through shared memory between two block
// barriers) over the radices of the in-register DFTs (2, 3, 4, 5, 8, 16 and the
// composites 6, 9, 10, 12, 15, 20, 24), each within the staging cap; among
// equally short schedules, the one with the fewest radices that are not powers
// of two (their butterflies cost more per point) and no radix-2 pass (a whole
// pass for one butterfly stage).  Larger radices go first.
std::vector<int> schedule(int n, int T) {
  int a, b, c;
  if (!factor235(n, &a, &b, &c)) return {};
  if (n == 1) return {1};
  struct Rad { int r, x, y, z; };   // r = 2^x 3^y 5^z
  const Rad rads[] = {{24, 3, 1, 0}, {20, 2, 0, 1}, {16, 4, 0, 0}, {15, 0, 1, 1}, {12, 2, 1, 0}, {10, 1, 0, 1},
                      {9, 0, 2, 0},  {8, 3, 0, 0},  {6, 1, 1, 0},  {5, 0, 0, 1},  {4, 2, 0, 0},  {3, 0, 1, 0},
                      {2, 1, 0, 0}};
  // cost[(x, y, z)] of the exponents still to cover: passes * 64 + non-power-of-two radices
  const int A = a + 1, B = b + 1, C = c + 1;
  const int kInf = 1 << 29;
  std::vector<int> cost((size_t)A * B * C, kInf), pick((size_t)A * B * C, -1);
  auto id = [&](int x, int y, int z) { return ((size_t)x * B + y) * C + z; };
  cost[id(0, 0, 0)] = 0;
  for (int x = 0; x <= a; x++)
    for (int y = 0; y <= b; y++)
      for (int z = 0; z <= c; z++) {
        if (!x && !y && !z) continue;
        for (int i = 0; i < (int)(sizeof(rads) / sizeof(rads[0])); i++) {
          const Rad& q = rads[i];
          if (q.x > x || q.y > y || q.z > z || !stage_ok(n, q.r, T)) continue;
          const int prev = cost[id(x - q.x, y - q.y, z - q.z)];
          if (prev >= kInf) continue;
          const int cst = prev + 64 + ((q.r & (q.r - 1)) ? 1 : 0) + (q.r == 2 ? 2 : 0);
          if (cst < cost[id(x, y, z)]) {
            cost[id(x, y, z)] = cst;
            pick[id(x, y, z)] = i;
          }
        }
      }
  if (cost[id(a, b, c)] >= kInf) return {};
  std::vector<int> r;
  for (int x = a, y = b, z = c; x || y || z;) {
    const Rad& q = rads[pick[id(x, y, z)]];
    r.push_back(q.r);
    x -= q.x;
    y -= q.y;
    z -= q.z;
  }
  std::sort(r.rbegin(), r.rend());
  return r;
}

std::string list(const std::vector<int>& v) {
  std::ostringstream o;
  for (size_t i = 0; i < v.size(); i++) o << (i ? "," : "") << v[i];
  return o.str();
}

std::string cache_dir() {
  const char* e = getenv("FPCC_JIT_CACHE");
  if (e && *e) return e;
  const char* h = getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.cache/fastpcc_gb300";
}

void mkdirs(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i < d.size(); i++) {
    cur += d[i];
    if (d[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(d.c_str(), 0755);
}

bool compile(const std::string& name, std::vector<char>* cubin, std::string* lowered) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, kJitSource, "fpcc_fused.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) return false;
  nvrtcAddNameExpression(prog, name.c_str());
  const std::string inc = std::string("--include-path=") + FPCC_CUDA_INCLUDE;
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device", "-lineinfo",
                        "--extra-device-vectorization", inc.c_str()};
  const nvrtcResult rc = nvrtcCompileProgram(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
  if (rc != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    fprintf(stderr, "fastpcc_gb300: run-time compilation of %s failed:\n%s\n", name.c_str(), log.c_str());
    nvrtcDestroyProgram(&prog);
    return false;
  }
  const char* low = nullptr;
  nvrtcGetLoweredName(prog, name.c_str(), &low);
  *lowered = low ? low : "";
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin->resize(n);
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  return !lowered->empty() && n > 0;
}

Entry build(int dev, int N, int Nz) {
  Entry e;
  const int nmax = N > Nz ? N : Nz;
  int T = ((ceil_div(nmax, 16) + 31) / 32) * 32;
  if (T < 128) T = 128;
  if (T > 1024) T = 1024;
  std::vector<int> rn, rz;
  for (; T <= 1024; T += 32) {
    rn = schedule(N, T);
    rz = schedule(Nz, T);
    if (!rn.empty() && !rz.empty()) break;
  }
  e.smem = fused_smem_bytes(N, Nz);
  if (rn.empty() || rz.empty() || T > 1024 || e.smem > kMaxSmem) {
    e.failed = true;
    return e;
  }
  e.T = T;
  // even N: the real window's DFT_N as an N/2-point complex transform
  // (k_station_fused_real); FPCC_STATION_REAL=0 keeps the N-point one
  std::vector<int> rh;
  const char* re = getenv("FPCC_STATION_REAL");
  if (N % 2 == 0 && !(re && re[0] == '0') && fused_smem_bytes(N, Nz, N / 2) <= kMaxSmem) rh = schedule(N / 2, T);
  std::string name;
  if (!rh.empty()) {
    e.smem = fused_smem_bytes(N, Nz, N / 2);
    name = "fpcc::k_station_fused_real<" + std::to_string(T) + ", fpcc::Radices<" + list(rh) + ">, fpcc::Radices<" +
           list(rn) + ">, fpcc::Radices<" + list(rz) + ">>";
  } else {
    name = "fpcc::k_station_fused<" + std::to_string(T) + ", fpcc::Radices<" + list(rn) + ">, fpcc::Radices<" +
           list(rz) + ">>";
  }
  // disk cache keyed by the kernel name and the source text
  const size_t h = std::hash<std::string>()(name + "|" + kJitSource);
  char file[128];
  snprintf(file, sizeof file, "/fused_%016zx_sm103a", h);
  const std::string dir = cache_dir();
  std::vector<char> cubin;
  std::string lowered;
  {
    std::ifstream f(dir + file + ".cubin", std::ios::binary);
    std::ifstream g(dir + file + ".name");
    if (f && g) {
      cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
      std::getline(g, lowered);
    }
  }
  if (cubin.empty() || lowered.empty()) {
    if (!compile(name, &cubin, &lowered)) {
      e.failed = true;
      return e;
    }
    mkdirs(dir);
    const std::string tmp = dir + file + ".tmp" + std::to_string((long)getpid());
    std::ofstream(tmp + "c", std::ios::binary).write(cubin.data(), (std::streamsize)cubin.size());
    std::ofstream(tmp + "n") << lowered << "\n";
    std::rename((tmp + "c").c_str(), (dir + file + ".cubin").c_str());
    std::rename((tmp + "n").c_str(), (dir + file + ".name").c_str());
  }
  (void)dev;
  if (cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
      cudaLibraryGetKernel(&e.fn, e.lib, lowered.c_str()) != cudaSuccess ||
      cudaFuncSetAttribute((const void*)e.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem) !=
          cudaSuccess) {
    cudaGetLastError();
    e.failed = true;
  }
  return e;
}

bool jit_enabled() {
  const char* e = getenv("FPCC_JIT");
  return !(e && e[0] == '0');
}

}  // namespace

bool fused_fits(int N, int Nz) { return fused_smem_bytes(N, Nz) <= kMaxSmem && N <= Nz; }

cudaError_t launch_station_fused(const float* x, long long ldx, int nrows, int N, int Nz, int rule, int fmt,
                                 void* out, long long ldo, cudaStream_t st) {
  if (!jit_enabled() || !fused_fits(N, Nz) || nrows <= 0) return cudaErrorNotSupported;
  int dev = 0;
  cudaGetDevice(&dev);
  Entry* e = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_tuple(dev, N, Nz);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) it = g_cache.emplace(key, build(dev, N, Nz)).first;
    e = &it->second;
  }
  if (e->failed) return cudaErrorNotSupported;
  FusedArgs a{x, ldx, nrows, rule, fmt, out, ldo};
  void* args[] = {&a};
  return cudaLaunchKernel((const void*)e->fn, dim3((unsigned)nrows), dim3((unsigned)e->T), args, (size_t)e->smem, st);
}

}  // namespace fpcc
