/*
 * oracle64 — FP64 CPU restatement of FastPCC's interstation-correlation methods.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/, the smoke check and the CPU-baseline
 * leg of bench.py as the checker; the product library never links it.
 *
 * Conventions (reference src/FFTapps.c):
 *   - A lag window [Lag1, Lag2] (either order) gives L = |Lag2-Lag1|+1 outputs,
 *     y[l] <-> lag = min(Lag1,Lag2) + l, with out[lag] = sum_n conj(a1[n]) a2[n+lag]
 *     (src/FFTapps.c:792-798, 851-856).
 *   - Batched entry points take Tr windows stored contiguously (Tr x N floats)
 *     and write Tr x L doubles; windows run in parallel with OpenMP.
 */
#ifndef FASTPCC_ORACLE64_H
#define FASTPCC_ORACLE64_H

#include <complex.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Amplitude-normalisation rules found in the reference. */
enum {
    ORC_AMP_F_REG = 0,   /* AmpNormf  src/FFTapps.c:178-205: x/(|x| + 1e-6*max|x|)         */
    ORC_AMP_D_REG = 1,   /* AmpNorm   src/FFTapps.c:147-175: x/sqrt(|x|^2 + 1e-6*max|x|^2) */
    ORC_AMP_PURE = 2,    /* GPU_AmpNormf, mabs=0  src/ccs_cuda.cu:212-232: x/|x| if |x|>0  */
    ORC_AMP_THRESH = 3,  /* GPU_AmpNormf2 + max   src/ccs_cuda.cu:190-210,513-531:
                            x/|x| if |x|^2 > 1e-6*max|x|^2, else 0                        */
    ORC_AMP_SUMTHR = 4   /* GPU_AmpNormf2 + sum   src/ccs_cuda.cu:107-146,493-511:
                            x/|x| if |x|^2 > 1e-6*sum|x|^2, else 0                        */
};

/* Reference padding rule Nz = 2^ceil(log2(N+M)) (src/FFTapps.c:805). */
unsigned orc_nz_rule(unsigned N, int Lag1, int Lag2);

int orc_analytic(double complex *y, const float *x, unsigned N);
void orc_ampnorm(double complex *y, unsigned N, int rule);
/* phase signal = ampnorm(analytic(x)) */
int orc_phase(double complex *y, const float *x, unsigned N, int rule);

/* PCC2 (src/FFTapps.c:785-881).  Nz = 0 selects the reference rule. */
int orc_pcc2_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2, unsigned Nz, int rule);

/* PCC at power v by direct lag sums (src/FFTapps.c:223-336, GPU twins
 * src/ccs_cuda.cu:260-321,388-453).  norm_gpu = 0 divides by 2^(v/2)*(N-|lag|)
 * (CPU pccf_lowlevel) — for v = 1 the CPU pcc1 path divides by 2*(N-|lag|),
 * which callers select with norm_gpu = 1, the GPU rule 2*(N-|lag|). */
int orc_pccv_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 double v, int Lag1, int Lag2, int rule, int norm_gpu);
/* Same on caller-supplied phase signals (complex, Tr x N, already normalised). */
int orc_pccv_phase(double *y, const double complex *p1, const double complex *p2, unsigned N,
                   double v, int Lag1, int Lag2, int norm_gpu);

/* GNCC (src/FFTapps.c:883-978 with cc_lowlevel :338-353 and gn_lowlevel :372-399). */
int orc_gncc_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2);

/* 1-bit GNCC (src/FFTapps.c:980-1073): s1 = x1>=0 ? 1 : -1, s2 = x2>0 ? 1 : -1. */
int orc_cc1b_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2);
/* Exact integer numerators sum_n s1[n] s2[n+lag] over the overlap. */
int orc_cc1b_num(int64_t *num, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2);

/* Wavelet family (src/FWTa/wavelet_def_v7.c:204-322).  Writes S = J*V scales,
 * lengths, centres; taps (concatenated, sum of Ls) when taps != NULL.  Returns
 * the total tap count. */
unsigned orc_wavelet_family(int type, unsigned J, unsigned V, unsigned Nz, double s0,
                            double op1, double *scale, unsigned *Ls, int *center,
                            double complex *taps);

/* WPCC set-up of src/FFTapps.c:1084-1115: returns S, and writes Nz (after the
 * doubling rule), s0, op1, K0 through the pointers.  Returns 0 on error. */
unsigned orc_wpcc_setup(unsigned N, int Lag1, int Lag2, double pmin, double pmax,
                        unsigned V, int type, double op1_in, unsigned *Nz_out,
                        double *s0_out, double *op1_out, unsigned *J_out);

/* WPCC (src/FFTapps.c:1076-1255, CPU path).  rule = ORC_AMP_D_REG for the
 * reference CPU path, ORC_AMP_THRESH for the GPU path's normalisation
 * (src/ccs_cuda.cu:1004,1009). */
int orc_wpcc_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type,
                 double op1, int rule);

/* The same restricted to scales s_lo <= s < s_hi (per-band diagnostics; the
 * output scale C still uses all scales). */
int orc_wpcc_band(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                  int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type,
                  double op1, int rule, unsigned s_lo, unsigned s_hi);

#ifdef __cplusplus
}
#endif

/* Stacks of K correlation traces of L samples (row-major y): mode 0 linear,
 * 1 phase-weighted (time domain), 2 time-scale phase-weighted; nu the
 * coherence power; pmin/pmax (samples), V, type, op1 select the wavelet
 * family of mode 2.  out: L values.  Returns 0, -1 or -3. */
int orc_stack(double *out, const float *y, unsigned K, unsigned L, int mode, double nu, double pmin,
              double pmax, unsigned V, int type, double op1);
unsigned orc_stack_family(unsigned L, double pmin, double pmax, unsigned V, int type, double op1_in,
                          double *s0_out, double *op1_out, unsigned *J_out);
double orc_cpsi(int type, double w0);
void orc_cwt(double complex *W, const double *x, unsigned L, unsigned S, const unsigned *Ls,
             const int *center, const double complex *taps);
void orc_icwt(double *x, const double complex *W, unsigned L, unsigned S, unsigned V, double cpsi,
              const double *scale, const unsigned *Ls, const int *center, const double complex *taps);

#endif
