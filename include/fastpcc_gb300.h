/*
 * fastpcc_gb300 — GB300-native interstation correlations (C ABI).
 *
 * Methods (reference: FastPCC src/FFTapps.c):
 *   FPCC_PCC2   phase cross-correlation at power 2 via DFTs of unit-modulus
 *               analytic phase signals                     (pcc2_set  :785-881)
 *   FPCC_GNCC   geometrically normalised cross-correlation  (ccgn_set  :883-978)
 *   FPCC_CC1B   1-bit GNCC, DFT path                        (cc1b_set  :980-1073)
 *   FPCC_CC1B_POPCOUNT  1-bit GNCC with exact integer numerators from
 *               popcounts of packed sign bits (same outputs as cc1b_set)
 *   FPCC_PCC1   PCC at power 1 by direct lag sums           (pcc1_set  :611-783)
 *   FPCC_PCCV   PCC at power v by direct lag sums           (pcc_set   :475-608)
 *   FPCC_WPCC   wavelet PCC                                 (tspcc2_set :1076-1255)
 *
 * Lag conventions follow the reference: a window [Lag1, Lag2] (either order)
 * yields L = |Lag2-Lag1|+1 outputs, output l <-> lag min(Lag1,Lag2)+l, with
 * out[lag] = sum_n conj(a1[n]) a2[n+lag]; |Lag1|,|Lag2| < N.
 *
 * All calls return 0 on success and a negative FPCC_E* code on failure (the
 * message is available from fpcc_last_error()).  No call resets the device.
 *
 * The reference's own GPU entry points (src/ccs_cuda.h) are declared, with
 * identical signatures, in ccs_cuda.h beside this header.
 */
#ifndef FASTPCC_GB300_H
#define FASTPCC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPCC_OK 0
#define FPCC_ECUDA (-1)    /* CUDA runtime failure (the reference's -1)          */
#define FPCC_ENOMEM (-2)   /* allocation failure                                  */
#define FPCC_EARG (-3)     /* invalid argument, e.g. |lag| >= N (reference's -3)  */
#define FPCC_EUNSUP (-4)   /* size or option not supported by this library        */

enum fpcc_method {
  FPCC_PCC2 = 0,
  FPCC_GNCC = 1,
  FPCC_CC1B = 2,
  FPCC_CC1B_POPCOUNT = 3,
  FPCC_PCC1 = 4,
  FPCC_PCCV = 5,
  FPCC_WPCC = 6
};

/* Amplitude-normalisation rules of the reference (phase signals). */
enum fpcc_amp_rule {
  FPCC_AMP_F_REG = 0,  /* AmpNormf, src/FFTapps.c:178-205 (CPU PCC paths, default) */
  FPCC_AMP_D_REG = 1,  /* AmpNorm,  src/FFTapps.c:147-175 (CPU WPCC)               */
  FPCC_AMP_PURE = 2,   /* x/|x|, src/ccs_cuda.cu:212-232 with mabs = 0 (GPU PCC)   */
  FPCC_AMP_THRESH = 3, /* x/|x| above 1e-6 max|x|^2, src/ccs_cuda.cu:190-210 (GPU WPCC) */
  FPCC_AMP_SUMTHR = 4  /* x/|x| above 1e-6 sum|x|^2, src/ccs_cuda.cu:493-511        */
};

/* Storage formats of cached station products (phase spectra, phase signals).
 * FPCC_I16: block-scaled int16 — phase-spectrum rows start with a 16-byte
 * header holding the row's float scale (value = q * scale, the largest
 * component at 32767), then Nz short2 bins, so a row spans Nz + 4 four-byte
 * elements; phase-signal rows hold N short2 values of scale 1/32767 (|phase| <= 1)
 * and no header.  4 bytes per complex value like F16, with about 8 times less
 * rounding error on the correlations. */
enum fpcc_format { FPCC_F32 = 0, FPCC_F16 = 1, FPCC_I16 = 2 };

/* 1-bit sign rules: the reference maps x1 >= 0 -> +1 but x2 > 0 -> +1
 * (src/FFTapps.c:1037,1042). */
enum fpcc_sign_rule { FPCC_SIGN_GE = 0, FPCC_SIGN_GT = 1 };

/* Precision of the analytic signals of the phase methods (PCC2, PCC1, PCCV).
 * FP32 transforms leave an absolute error of about 1e-7 x rms on every sample,
 * which loses the phase where the analytic signal is small — inside runs of
 * zero samples (data gaps, zero padding).  AUTO (the default) computes the
 * analytic signals of windows with at least FPCC_F64_ZERO_SAMPLES zero samples
 * in FP64. */
enum fpcc_analytic_precision { FPCC_ANALYTIC_F32 = 0, FPCC_ANALYTIC_AUTO = 1, FPCC_ANALYTIC_F64 = 2 };
#define FPCC_F64_ZERO_SAMPLES 4

/* Padded correlation length rules. */
enum fpcc_nz_mode { FPCC_NZ_TUNED = -1, FPCC_NZ_REFERENCE = 0, FPCC_NZ_FAST = 1 };

typedef struct fpcc_ctx fpcc_ctx;

/* ---- context ------------------------------------------------------------ */
int fpcc_create(fpcc_ctx **out, int device);
int fpcc_destroy(fpcc_ctx *ctx);
/* fpcc_analytic_precision mode of the context's station stages (default AUTO). */
int fpcc_set_analytic_precision(fpcc_ctx *ctx, int mode);
/* Run subsequent work on this CUDA stream (cudaStream_t; NULL = the context's own). */
int fpcc_set_stream(fpcc_ctx *ctx, void *stream);
void *fpcc_get_stream(fpcc_ctx *ctx);
int fpcc_sync(fpcc_ctx *ctx);
const char *fpcc_last_error(void);
const char *fpcc_version(void);
/* Kernel launches issued by this process so far (all contexts). */
int64_t fpcc_launch_count(void);

/* ---- planning ----------------------------------------------------------- */
/* Padded correlation length for N samples and the lag window (mode: fpcc_nz_mode). */
int fpcc_choose_nz(int N, int Lag1, int Lag2, int mode);
/* Autotuner: times the pair stage (per correlation) and the station stage (per
 * window) of every usable padded length in [min_nz, max_nz] on the context's
 * GPU and keeps the table that FPCC_NZ_TUNED chooses from (cost = pair +
 * station / reuse, reuse = correlations per station window); writes it as JSON
 * to json_path when given.  FPCC_NZ_TUNED falls back to FPCC_NZ_FAST for
 * lengths the table does not cover. */
int fpcc_autotune(fpcc_ctx *ctx, int min_nz, int max_nz, double reuse, const char *json_path);
int fpcc_autotune_load(const char *json_path);
/* Largest length an in-block transform of this library supports. */
int fpcc_max_block_len(void);
/* Pair kernel that runs the FFT methods' pair stage at padded length Nz:
 * FPCC_PAIR_BLOCK (one block per correlation, Stockham passes through shared
 * memory) or FPCC_PAIR_TILED (Nz/2 = R1 x 256, R1 in {32, 40}: stage 1 in
 * registers, warp-private second stage).  form > 0 selects it (the autotuner
 * does this per length), form = 0 only queries.  Returns the form in use, or
 * FPCC_EUNSUP if the requested form does not run Nz. */
enum fpcc_pair_form { FPCC_PAIR_BLOCK = 1, FPCC_PAIR_TILED = 2 };
int fpcc_pair_form(int Nz, int form);
/* Elements per row of the station product of a method (for sizing buffers). */
int64_t fpcc_station_row_elems(int method, int N, int Nz);
/* Bytes per row of the station product of a method in a storage format. */
int64_t fpcc_station_row_bytes(int method, int N, int Nz, int fmt);

/* ---- device-resident stages (all pointers are device memory) -------------
 * Station stage: one output row per input row.
 *   PCC2:            DFT_Nz of the zero-padded phase signal, Nz complex (fmt F32/F16), rule = fpcc_amp_rule
 *   PCC1, PCCV:      phase signal, N complex (fmt F32 float2 / F16 half2), rule = fpcc_amp_rule
 *   GNCC:            DFT_Nz of the zero-padded trace, bins 0..Nz/2 (F32)
 *   CC1B:            DFT_Nz of the zero-padded 1-bit signs, bins 0..Nz/2 (F32), rule = fpcc_sign_rule
 *   CC1B_POPCOUNT:   packed sign bits, ceil(N/32) uint32 words, rule = fpcc_sign_rule
 */
int fpcc_station_stage(fpcc_ctx *ctx, int method, const float *d_x, int64_t ldx, int nrows, int N,
                       int Nz, int fmt, int rule, void *d_out, int64_t ldo);
/* As fpcc_station_stage, with the rows whose analytic signals are computed in
 * FP64 named by the caller (host array of n_f64_rows row indices); n_f64_rows < 0
 * applies the context's fpcc_analytic_precision mode instead. */
int fpcc_station_stage_ex(fpcc_ctx *ctx, int method, const float *d_x, int64_t ldx, int nrows, int N,
                          int Nz, int fmt, int rule, void *d_out, int64_t ldo, const int32_t *h_f64_rows,
                          int n_f64_rows);
/* Station stage of the phase methods (PCC2, PCC1, PCCV) for windows of
 * different lengths: row r reads h_rows[r].d_x (N samples) and writes d_out +
 * r * ldo (ldo in elements of the format: 8 bytes for F32, 4 otherwise).  The
 * analytic signal of each row is its circular convolution with the kernel
 * IDFT_N(mask), computed with M-point transforms shared by every row of the same
 * length class (M = 2^a, 3 2^a or 5 2^a >= 2N - 1; FP64 for rows with f64 set),
 * two rows per forward transform, so the windows share their launches; rows
 * must be ordered by (N, Nz). */
typedef struct {
  const float *d_x;   /* the window's samples (device)                */
  int32_t N, Nz;      /* window length, padded length (PCC2)          */
  int32_t f64;        /* 1: FP64 analytic signal (windows with gaps)  */
  int32_t pad;
} fpcc_station_row;
int fpcc_station_stage_multi(fpcc_ctx *ctx, int method, const fpcc_station_row *h_rows, int nrows, int fmt,
                             int rule, void *d_out, int64_t ldo);
/* FP64 prefix sums E[n] = sum_{m<n} x[m]^2, N+1 per row (GNCC normalisation).
 * Rows with ldE >= 2 (N+1) also receive, after the sums, 2 (N+1) floats of
 * normalisation tables (reciprocal square roots of the prefix and suffix
 * energies), and E[0] is written as -0.0 to flag them; the pair stage then reads
 * two floats per lag instead of two FP64 sums, with identical results. */
int fpcc_energy_stage(fpcc_ctx *ctx, const float *d_x, int64_t ldx, int nrows, int N, double *d_E,
                      int64_t ldE);
/* Pair stage: output row p correlates station rows pairs[2p] (station 1) and
 * pairs[2p+1] (station 2).  v is the power for PCCV; d_E/ldE the energies for
 * GNCC; d_num (optional, CC1B_POPCOUNT) receives exact int64 numerators. */
int fpcc_pair_stage(fpcc_ctx *ctx, int method, const void *d_station, int64_t lds, int fmt,
                    const int32_t *d_pairs, int npairs, int N, int Nz, int Lag1, int Lag2, float v,
                    const double *d_E, int64_t ldE, float *d_y, int64_t ldy, int64_t *d_num);

/* Packed pair stage: correlations of different window lengths and lag windows
 * in one launch.  Each descriptor names its own product rows (anywhere in device
 * memory), window length, lags and output row; only the padded length Nz (FFT
 * methods; must satisfy Nz >= N + max|lag| for every entry; lengths above
 * 2 * fpcc_max_block_len() run as four-step transforms), the storage format and
 * the power v are shared.
 * d_desc is a device array of npairs descriptors; maxL >= every entry's L.
 * scale: 0 selects the method's own (PCC2 1/(Nz N), GNCC and 1-bit 1/Nz). */
typedef struct {
  const void *a, *b;          /* station-1 / station-2 product rows                    */
  const double *ea, *eb;      /* GNCC: energy prefix sums of the two windows (N+1)     */
  void *y;                    /* output row: L floats (L int64 for popcount numerators) */
  int32_t N, lag0, L;         /* window length, first lag, number of lags              */
  float scale;
} fpcc_pair_desc;
int fpcc_pair_stage_packed(fpcc_ctx *ctx, int method, int fmt, int Nz, const fpcc_pair_desc *d_desc,
                           int npairs, int maxL, float v, int numerators);

/* ---- preprocessing of station windows (device memory, in place) -----------
 * The reference CLI's optional steps before correlating (src/PCC_fullpair_1b.c).
 * fpcc_clip_rows: clip each of nrows rows (N samples, stride ldx) at
 *   4 median(|x|) / 0.6745 (clipping :881-891 with qabsmedian :1179-1214).
 * fpcc_whiten_rows: smooth spectral whitening of a station's windows between
 *   f1 and f2 Hz at sampling interval dt (AveWhite :1065-1177): FP64 transforms
 *   of length 2^ceil(log2 N), the amplitude spectrum averaged over the nrows
 *   windows, the band-limited inverse filter (gain capped at 1000x its minimum,
 *   11-tap smoothing), applied to every window.  Messages: fpcc_prep_last_error(). */
int fpcc_clip_rows(fpcc_ctx *ctx, float *d_x, int64_t ldx, int nrows, int N);
int fpcc_whiten_rows(fpcc_ctx *ctx, float *d_x, int64_t ldx, int nrows, int N, double f1, double f2,
                     double dt);
const char *fpcc_prep_last_error(void);

/* ---- stacks of correlation traces over windows (device memory) -------------
 * The obin output is written for an external stacking code (ts-PWS,
 * src/PCC_fullpair_1b.c:568-569) whose source is not part of the reference;
 * stacking on the device instead keeps the per-window correlations in HBM.
 * ngroups groups of K traces of L samples: trace j of group g starts at
 * d_y + g*ldg + j*ldj (groups of adjacent rows: ldj = row stride, ldg = K*ldj;
 * the window-major rows of an all-pairs pair stage: ldj = pairs per window *
 * row stride, ldg = row stride); group g's stack goes to row g of d_out
 * (stride ldo).
 *   FPCC_STACK_LINEAR  the mean of the group's traces
 *   FPCC_STACK_PWS     the mean times |mean_j a_j / |a_j||^nu, a_j the analytic
 *                      signal of trace j (the rule of src/FFTapps.c:45-80);
 *                      phase-weighted stack of Schimmel and Paulssen (1997)
 *   FPCC_STACK_TSPWS   the inverse CWT of |mean_j W_j / |W_j||^nu * CWT(mean),
 *                      W_j the CWT of trace j; time-scale phase-weighted stack
 *                      of Ventosa, Schimmel and Stutzmann (2017), with the CWT
 *                      and the inverse of the reference's wavelet library
 *                      (complex_1D_wavelet_dec, Re_complex_1D_wavelet_rec,
 *                      src/FWTa/wavelet_v7.c:43-150: circular over the trace)
 *                      and its family (type -1/-2 Morlet, -3 Mexican hat; V
 *                      voices; s0 from pmin, the octaves from pmax/pmin, both in
 *                      samples, as src/FFTapps.c:1097-1107; op1 = w0, 0 for the
 *                      default).  pmin, pmax, V, type, op1 are unused otherwise.
 * Phasors of zero modulus count as zero.  Returns 0, FPCC_EARG or a CUDA error. */
enum fpcc_stack_mode { FPCC_STACK_LINEAR = 0, FPCC_STACK_PWS = 1, FPCC_STACK_TSPWS = 2 };
int fpcc_stack(fpcc_ctx *ctx, int mode, const float *d_y, int64_t ldg, int64_t ldj, int K, int L, int ngroups,
               double nu, double pmin, double pmax, int V, int type, double op1, float *d_out, int64_t ldo);

/* ---- host-buffer entry points (row-pointer arrays like the reference's *_set)
 * x1, x2: Tr rows of N floats (station 1 / station 2 windows); y: Tr rows of L.
 * The "batched" calls run each stage once over all windows; the plain drop-ins
 * below run one launch sequence per window. */
int fpcc_host_batched(int method, float **y, float **x1, float **x2, unsigned N, unsigned Tr,
                      int Lag1, int Lag2, float v, int nz_mode, int fmt);
int fpcc_host_plain(int method, float **y, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1,
                    int Lag2, float v, int nz_mode, int fmt);

/* Contiguous host arrays (pinned or pageable): x is nsta x N, pairs 2*npairs
 * (row indices in [0, nsta), else FPCC_EARG before any work), y npairs x L.
 * Host<->device copies happen inside the call: the rows go up in chunks that
 * the station stage consumes as they arrive, and the results come down in
 * chunks while later pair chunks compute. */
int fpcc_allpairs_host(fpcc_ctx *ctx, int method, const float *h_x, int nsta, int N,
                       const int32_t *h_pairs, int npairs, int Lag1, int Lag2, float v, int nz_mode,
                       int fmt, float *h_y);

/* Drop-in siblings of the reference's GPU calls for the methods it runs on the
 * CPU (raw float traces in, y rows out; semantics of pcc2_set, ccgn_set,
 * cc1b_set).  Plain form: one launch sequence per pair and window. */
int pcc2_highlevel(float **y, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1, int Lag2);
int ccgn_highlevel(float **y, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1, int Lag2);
int cc1b_highlevel(float **y, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1, int Lag2);
/* Exact integer numerators of 1-bit GNCC (num rows of L int64). */
int cc1b_popcount_highlevel(int64_t **num, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1,
                            int Lag2);

/* ---- wavelet PCC (reference tspcc2_set, src/FFTapps.c:1076-1255) ---------
 * A plan holds the complex wavelet family (type -1 Morlet, -2 complete Morlet,
 * -3 complex Mexican hat; scales from pmin/pmax in samples, V voices), its
 * spectra on the device and the padded length (nz_mode as fpcc_nz_mode or an
 * explicit length).  rule: FPCC_AMP_D_REG (the reference CPU path) or
 * FPCC_AMP_THRESH (the reference GPU path).  Station products are S x Nz complex
 * per station window (the per-scale phase spectra). */
typedef struct fpcc_wpcc_plan fpcc_wpcc_plan;
int fpcc_wpcc_plan_create(fpcc_ctx *ctx, fpcc_wpcc_plan **out, unsigned N, int Lag1, int Lag2, double pmin,
                          double pmax, unsigned V, int type, double op1, int rule, int nz_mode);
int fpcc_wpcc_plan_info(const fpcc_wpcc_plan *p, int *Nz, int *S, int *L);
/* Accumulate only scales s_lo <= s < s_hi (per-band diagnostics; the output
 * scale keeps all scales).  fpcc_wpcc_plan_set_band(p, 0, S) restores the plan. */
int fpcc_wpcc_plan_set_band(fpcc_wpcc_plan *p, int s_lo, int s_hi);
/* Change the plan's lag window (station products stay valid); lags must fit the
 * plan's padded length. */
int fpcc_wpcc_plan_set_lags(fpcc_wpcc_plan *p, int Lag1, int Lag2);
int fpcc_wpcc_plan_destroy(fpcc_wpcc_plan *p);
int fpcc_wpcc_station_stage(fpcc_ctx *ctx, const fpcc_wpcc_plan *p, const float *d_x, int64_t ldx, int nrows,
                            void *d_P, int fmt);
int fpcc_wpcc_pair_stage(fpcc_ctx *ctx, const fpcc_wpcc_plan *p, const void *d_P, int fmt, const int32_t *d_pairs,
                         int npairs, float *d_y, int64_t ldy);
/* Host rows in and out, arguments of tspcc2_set plus rule and nz_mode. */
int fpcc_wpcc_host(float **y, float **x1, float **x2, unsigned N, unsigned Tr, int Lag1, int Lag2, double pmin,
                   double pmax, unsigned V, int type, double op1, int rule, int nz_mode);

/* ---- serving loop -----------------------------------------------------------
 * A server keeps station products (phase spectra, real/sign spectra, energies,
 * phase signals, sign bits) resident in HBM under a byte budget and runs a
 * worker thread that batches requests continuously: everything pending when the
 * worker is free forms the next batch, grouped by method and lengths; requests
 * that arrive while a batch is on the GPU join the following one.  Each result
 * depends only on its request, so it is the same alone and in any mix.
 * Station windows are registered once (host samples, copied); products are
 * computed on first use and recycled least-recently-used.  Station stages run
 * concurrently on lanes of the server (contexts with their own streams; the
 * environment variable FPCC_SERVER_LANES at creation sets their number, 0 for
 * one stream).  A failed request's status is a negative FPCC_E* code, and
 * fpcc_last_error() on the thread that collected it (fpcc_poll, fpcc_wait,
 * fpcc_server_drain) describes it. */
typedef struct fpcc_server fpcc_server;
typedef struct {
  int method;            /* FPCC_PCC2, GNCC, CC1B, CC1B_POPCOUNT, PCC1, PCCV, WPCC    */
  int32_t sta1, sta2;    /* station ids (station 1 = virtual source)                  */
  int32_t window;        /* window id, registered for both stations                   */
  int Lag1, Lag2;
  float v;               /* power for FPCC_PCCV                                       */
  float *y;              /* host output, L floats (written before completion)         */
  int64_t *num;          /* host output for FPCC_CC1B_POPCOUNT, L int64               */
} fpcc_request;
typedef struct {
  int64_t completed, batches, station_rows, hbm_used;
  double p50_ms, p99_ms, max_ms;   /* submit -> result latency of completed requests */
  int64_t pair_stages;             /* pair-stage launches (one per group of a batch)  */
  double worker_ms;                /* host time the worker spent forming and queueing
                                      batches (taken off the pending queue -> launched) */
  double deliver_ms;               /* host time of completion (wait for the batch, copy-out
                                      into unregistered outputs, status), summed         */
} fpcc_server_stats;
int fpcc_server_create(fpcc_server **out, int device, size_t hbm_budget_bytes, int max_batch);
/* Storage format (FPCC_F32 / FPCC_F16 / FPCC_I16) of the phase spectra and phase signals
 * the server caches (PCC2, PCC1, PCCV, WPCC); before the first request. */
int fpcc_server_set_format(fpcc_server *s, int fmt);
/* Padded-length rule of FFT requests (fpcc_nz_mode; default FPCC_NZ_FAST);
 * before the first request. */
int fpcc_server_set_nz_mode(fpcc_server *s, int mode);
/* Wavelet family of FPCC_WPCC requests (arguments of fpcc_wpcc_plan_create);
 * before the first request.  WPCC requests fail with FPCC_EARG without it. */
int fpcc_server_set_wavelet(fpcc_server *s, double pmin, double pmax, unsigned V, int type, double op1,
                            int rule);
/* A host range [p, p + bytes) that results may be written into straight from
 * the device: requests whose output rows lie inside it get their results by
 * device-to-host copies into those rows (rows at one stride as one strided
 * copy) instead of through the server's pinned buffer and a host copy.  The
 * range is page-locked here unless it already is (then it is only recorded).
 * Unregister it (or destroy the server) only when no request writing into it
 * is pending.  No counterpart in the reference (its calls return results in
 * the caller's arrays synchronously). */
int fpcc_server_register_output(fpcc_server *s, void *p, size_t bytes);
int fpcc_server_unregister_output(fpcc_server *s, void *p);
int fpcc_server_destroy(fpcc_server *s);
int fpcc_put_station_window(fpcc_server *s, int32_t sta, int32_t window, const float *x, int N);
/* Returns a request id (>= 0) or a negative FPCC_E* code. */
int64_t fpcc_submit(fpcc_server *s, const fpcc_request *req);
/* n requests at once; ids[i] receives each id (or a negative code, which stops the call). */
int fpcc_submit_many(fpcc_server *s, const fpcc_request *reqs, int n, int64_t *ids);
/* Submits the requests at Poisson arrival times of `rate` per second (load generator). */
int fpcc_server_offer_poisson(fpcc_server *s, const fpcc_request *reqs, int n, double rate, uint64_t seed,
                              int64_t *ids);
/* 1 done, 0 pending, < 0 failed. */
int fpcc_poll(fpcc_server *s, int64_t id);
/* Blocks until done (timeout_s <= 0: no limit); returns as fpcc_poll. */
int fpcc_wait(fpcc_server *s, int64_t id, double timeout_s);
/* Blocks until every submitted request has completed. */
int fpcc_server_drain(fpcc_server *s);
int fpcc_server_get_stats(fpcc_server *s, fpcc_server_stats *out);
int fpcc_server_reset_stats(fpcc_server *s);

/* ---- allocation-free PCC2 ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host whose pool allocator owns all device memory, plugin frameworks that
 * forbid device allocation, latency-critical loops that must not synchronise
 * the device): PCC2 of the same-index windows of d_x1 and d_x2 (Tr rows of N
 * floats, row stride ldx, device memory) into d_y (Tr rows, stride ldy >= L),
 * on `stream` (a cudaStream_t; NULL = legacy default stream).  Every
 * intermediate lives in one fixed device array of fpcc_noalloc_scratch_bytes()
 * (64 MiB) that each GPU loading the library holds until exit; calls needing
 * more are rejected with FPCC_EARG and a message.  Each call looks up that
 * array's address in the current context (cudaGetSymbolAddress allocates
 * nothing); the first call on a device loads the library's device code, so make
 * it before any stream capture.  Calls share the array: calls whose work
 * overlaps on the GPU race and must be serialised by the caller.  A CUDA error
 * pending from the caller's earlier work is left in place and the call returns
 * FPCC_ECUDA without running.  Errors: fpcc_noalloc_last_error() (empty after a
 * successful call). */
int fpcc_pcc2_noalloc(const float *d_x1, const float *d_x2, int64_t ldx, int N, int Tr, int Lag1, int Lag2,
                      float *d_y, int64_t ldy, void *stream);
size_t fpcc_noalloc_scratch_bytes(void);
const char *fpcc_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
