// Autotuner: measured cost of every usable padded length, and the pair kernel
// of each length that two kernels can run.
//
// Every padded length Nz >= N + max|lag| gives the same correlation; which one
// is fastest depends on its radix schedule, on whether Nz/2 runs in one block
// or as a four-step transform, and on the GPU.  The autotuner times, on the
// context's GPU, the pair stage (per correlation) and the station stage (per
// window) of each usable length and keeps the table for FPCC_NZ_TUNED; a
// length's cost is pair + station / reuse, reuse being the correlations each
// station window takes part in.  Where both the one-block-per-correlation
// kernel and the tiled kernel run a length, both are timed and the faster one
// is selected for that length (fpcc_pair_form).  The radix schedules, block
// sizes and tile shapes inside each kernel are compile-time choices (the
// register and shared-memory budgets of each shape are fixed by them), so the
// tuned dimensions are the padded length and the kernel form.  The table is
// saved and loaded as JSON:
//   {"reuse": R, "lengths": {"Nz": [pair_ns, station_ns, form], ...}}
// form: 1 block kernel, 2 tiled kernel, 0 only one kernel runs the length.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fastpcc_gb300.h"
#include "engine.h"
#include "kernels.cuh"

using namespace fpcc;

namespace {

int save_table(const char* path) {
  double reuse = 0;
  const auto t = tuned_table(&reuse);
  FILE* f = fopen(path, "w");
  if (!f) return FPCC_EARG;
  fprintf(f, "{\"reuse\": %.6g, \"lengths\": {\n", reuse);
  for (size_t i = 0; i < t.size(); i++) {
    const int nz = std::get<0>(t[i]);
    const int form = (pair_tiled_supported(nz) && pair_supported(nz)) ? pair_form_get(nz) : 0;
    fprintf(f, "  \"%d\": [%.6g, %.6g, %d]%s\n", nz, std::get<1>(t[i]), std::get<2>(t[i]), form,
            i + 1 < t.size() ? "," : "");
  }
  fprintf(f, "}}\n");
  return fclose(f) == 0 ? 0 : FPCC_EARG;
}

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  Timer() { cudaEventCreate(&a); cudaEventCreate(&b); }
  ~Timer() { cudaEventDestroy(a); cudaEventDestroy(b); }
};

}  // namespace

extern "C" int fpcc_autotune(fpcc_ctx* ctx, int min_nz, int max_nz, double reuse, const char* json_path) {
  if (!ctx || min_nz < 2 || max_nz < min_nz || max_nz > (1 << 21)) return FPCC_EARG;
  tuned_set_reuse(reuse);
  cudaStream_t st = (cudaStream_t)fpcc_get_stream(ctx);
  const std::vector<int> lengths = usable_lengths(min_nz, max_nz);
  if (lengths.empty()) return FPCC_EUNSUP;
  const int R = 32, P = 256, reps = 3;
  const int nz_max = lengths.back();
  const int Lmax = 2 * (nz_max / 10) + 1;
  void *d_x = nullptr, *d_spec = nullptr, *d_half = nullptr, *d_y = nullptr, *d_pairs = nullptr;
  int rc = 0;
  auto fail = [&](int code) { rc = code; };
  if (cudaMalloc(&d_x, (size_t)R * (nz_max / 2) * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_spec, (size_t)R * nz_max * 8) != cudaSuccess ||
      cudaMalloc(&d_half, (size_t)R * (nz_max / 2 + 1) * 8) != cudaSuccess ||
      cudaMalloc(&d_y, (size_t)P * Lmax * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_pairs, (size_t)2 * P * sizeof(int32_t)) != cudaSuccess) {
    fail(FPCC_ENOMEM);
  }
  if (!rc) {
    // finite, non-denormal contents (0x3c3c3c3c ~ 0.0115)
    cudaMemsetAsync(d_x, 0x3c, (size_t)R * (nz_max / 2) * sizeof(float), st);
    cudaMemsetAsync(d_spec, 0x3c, (size_t)R * nz_max * 8, st);
    std::vector<int32_t> pr(2 * P);
    for (int p = 0; p < P; p++) { pr[2 * p] = p % R; pr[2 * p + 1] = (7 * p + 1) % R; }
    cudaMemcpyAsync(d_pairs, pr.data(), pr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  Timer tm;
  for (size_t i = 0; i < lengths.size() && !rc; i++) {
    const int nz = lengths[i];
    const int N = nz / 2, M = nz / 10;
    const int np = std::max(16, std::min(P, (1 << 23) / nz));   // fewer pairs for long transforms
    // station stage: DFT_Nz of R real windows (the part of every station stage that depends on Nz)
    float t_st = 0, t_pr = 0;
    for (int k = 0; k <= reps && !rc; k++) {
      if (k == 1) cudaEventRecord(tm.a, st);
      rc = fpcc_station_stage(ctx, FPCC_GNCC, (const float*)d_x, N, R, N, nz, FPCC_F32, 0, d_half, nz / 2 + 1);
    }
    if (rc) break;
    cudaEventRecord(tm.b, st);
    cudaEventSynchronize(tm.b);
    cudaEventElapsedTime(&t_st, tm.a, tm.b);
    // pair stage: P PCC2 correlations of full F32 spectra, lags +-nz/10; each
    // kernel form that runs this length, the faster one kept
    const bool two = pair_tiled_supported(nz) && pair_supported(nz);
    float best = -1.f;
    int best_form = 0;
    for (int form : {PAIR_FORM_BLOCK, PAIR_FORM_TILED}) {
      if (two) pair_form_set(nz, form);
      else if (form == PAIR_FORM_TILED) break;
      for (int k = 0; k <= reps && !rc; k++) {
        if (k == 1) cudaEventRecord(tm.a, st);
        rc = fpcc_pair_stage(ctx, FPCC_PCC2, d_spec, nz, FPCC_F32, (const int32_t*)d_pairs, np, N, nz, -M, M, 0.f,
                             nullptr, 0, (float*)d_y, 2 * M + 1, nullptr);
      }
      if (rc) break;
      cudaEventRecord(tm.b, st);
      cudaEventSynchronize(tm.b);
      cudaEventElapsedTime(&t_pr, tm.a, tm.b);
      if (best < 0.f || t_pr < best) { best = t_pr; best_form = form; }
    }
    if (rc) break;
    if (two) pair_form_set(nz, best_form);
    tuned_set(nz, 1e6 * best / (reps * np), 1e6 * t_st / (reps * R));
  }
  cudaFree(d_x);
  cudaFree(d_spec);
  cudaFree(d_half);
  cudaFree(d_y);
  cudaFree(d_pairs);
  if (!rc && json_path && *json_path) rc = save_table(json_path);
  return rc;
}

extern "C" int fpcc_autotune_load(const char* json_path) {
  if (!json_path) return FPCC_EARG;
  FILE* f = fopen(json_path, "r");
  if (!f) return FPCC_EARG;
  char line[512];
  int n = 0;
  while (fgets(line, sizeof line, f)) {
    double reuse;
    int nz;
    double a, b;
    int form = 0;
    if (sscanf(line, " {\"reuse\": %lf", &reuse) == 1) {
      tuned_set_reuse(reuse);
    } else {
      const int got = sscanf(line, " \"%d\": [%lf, %lf, %d]", &nz, &a, &b, &form);
      if (got >= 3 && nz_usable(nz)) {
        tuned_set(nz, a, b);
        if (got == 4 && form > 0) pair_form_set(nz, form);   // ignored where the form does not run nz
        n++;
      }
    }
  }
  fclose(f);
  return n > 0 ? 0 : FPCC_EARG;
}
