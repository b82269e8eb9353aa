// Host-side planning: radix schedules and padded correlation lengths.
#pragma once

#include <stdint.h>

#include <tuple>
#include <vector>

#include "fft_core.cuh"

namespace fpcc {

// Largest length one thread block transforms in shared memory.
constexpr int kMaxCtaLen = 21120;

// Factor n into 2^a 3^b 5^c; false for any other prime factor.
bool factor235(int n, int* a, int* b, int* c);

// Every 2^a 3^b 5^c in [lo, hi], ascending (about a hundred per octave near 1e5,
// against tens of thousands of integers: length searches walk this list).
std::vector<int> smooth235_in(int lo, int hi);

// Transform length class of a window length in the packed analytic-signal
// stage: the smallest 2^a, 3 2^a or 5 2^a >= 2N - 1 (about three classes per
// octave, so windows of nearby lengths share their transforms).
int conv_class_len(int N);

// Radix schedule for an in-block transform of length n (2,3,5-smooth):
// ceil(a/4) power-of-two passes with the exponent spread evenly, then the 5s
// and 3s.  When `forced` is non-null it lists the radices to use instead.
bool make_plan(int n, FftPlan* p, const int* forced = nullptr, int nforced = 0);
bool make_plan_raw(int n, FftPlan* p, const int* forced, int nforced);

// Padded correlation length for a window of N samples and max |lag| M.
//   mode 0: the reference rule 2^ceil(log2(N+M))   (src/FFTapps.c:805)
//   mode 1: the cheapest even 2,3,5-smooth length >= N+M whose half length fits
//           one block, by a per-pass cost model (results are identical for any
//           length >= N+M: the correlation is linear).
//   mode >= 2: that explicit length, if usable and >= N+M.
//   mode FPCC_NZ_TUNED_MODE (-1): the measured cheapest length from the autotuner's
//           table (mode 1 when the table holds no length >= N+M).
constexpr int FPCC_NZ_TUNED_MODE = -1;
int choose_nz(int N, int M, int mode);

// Autotuner table: measured pair-stage ns per correlation and station-stage ns
// per window for a padded length; reuse = correlations per station window
// assumed when weighing the two.
void tuned_set(int nz, double pair_ns, double station_ns);
void tuned_set_reuse(double reuse);
std::vector<std::tuple<int, double, double>> tuned_table(double* reuse);
// Even 2,3,5-smooth lengths in [lo, hi] usable as padded lengths.
std::vector<int> usable_lengths(int lo, int hi);
// Nz and Nz/2 both run in one block or as four-step transforms.
bool nz_usable(int nz);

// Estimated relative cost of an in-block transform of length n.
double plan_cost(int n);

}  // namespace fpcc
