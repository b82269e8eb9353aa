/*
 * oracle64 — FP64 CPU restatement of FastPCC's interstation-correlation methods.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle64.h).  Every function follows the
 * reference lines cited beside it; all arithmetic is FP64 and every transform
 * comes from oracle/fft64.c.
 */
#include "oracle64.h"
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

static void lag_window(int Lag1, int Lag2, int *lag0, unsigned *L) {
    /* src/FFTapps.c:792-798 */
    if (Lag2 >= Lag1) { *L = (unsigned)(Lag2 - Lag1 + 1); *lag0 = Lag1; }
    else              { *L = (unsigned)(Lag1 - Lag2 + 1); *lag0 = Lag2; }
}

unsigned orc_nz_rule(unsigned N, int Lag1, int Lag2) {
    /* src/FFTapps.c:801-805 */
    unsigned ua1 = (unsigned)abs(Lag1), ua2 = (unsigned)abs(Lag2);
    unsigned M = ua1 > ua2 ? ua1 : ua2;
    return 1u << (unsigned)ceil(log2((double)(N + M)));
}

/* Analytic signal, src/FFTapps.c:45-80 (FP64 twin of AnalyticSignal_plan_float
 * :104-124): X = DFT_N(x); X[0]/=N; X[1..ceil(N/2)-1] *= 2/N; X[N/2] /= N for
 * even N; remaining bins 0; y = IDFT_N(X) (unnormalised backward). */
int orc_analytic(double complex *y, const float *x, unsigned N) {
    if (!x || !y || N == 0) return -1;
    for (unsigned n = 0; n < N; n++) y[n] = (double)x[n];
    fft64_c2c(y, N, -1);
    const double d = 1.0 / (double)N;
    unsigned n;
    y[0] *= d;
    for (n = 1; n < (N + 1) >> 1; n++) y[n] *= 2 * d;
    if (!(N & 1)) y[n++] *= d;
    for (; n < N; n++) y[n] = 0;
    fft64_c2c(y, N, +1);
    return 0;
}

void orc_ampnorm(double complex *y, unsigned N, int rule) {
    double mx = 0, sm = 0;   /* max and sum of |y|^2 */
    for (unsigned n = 0; n < N; n++) {
        double a = creal(y[n]), b = cimag(y[n]);
        double m = a * a + b * b;
        if (mx < m) mx = m;
        sm += m;
    }
    if (rule == ORC_AMP_SUMTHR) mx = sm;
    if (rule == ORC_AMP_F_REG) {
        /* src/FFTapps.c:185-204 */
        double eps = 1e-6 * sqrt(mx);
        for (unsigned n = 0; n < N; n++) {
            double a = creal(y[n]), b = cimag(y[n]);
            double f = 1.0 / (sqrt(a * a + b * b) + eps);
            y[n] = isnormal(f) ? y[n] * f : 0;
        }
    } else if (rule == ORC_AMP_D_REG) {
        /* src/FFTapps.c:153-174 */
        double eps = 1e-6 * mx;
        for (unsigned n = 0; n < N; n++) {
            double a = creal(y[n]), b = cimag(y[n]);
            double f = 1.0 / sqrt(a * a + b * b + eps);
            y[n] = isnormal(f) ? y[n] * f : 0;
        }
    } else {
        /* src/ccs_cuda.cu:190-232: threshold e = 1e-6*mabs, mabs = 0, max|y|^2 or sum|y|^2 */
        double e = (rule == ORC_AMP_THRESH || rule == ORC_AMP_SUMTHR) ? 1e-6 * mx : 0.0;
        for (unsigned n = 0; n < N; n++) {
            double a = creal(y[n]), b = cimag(y[n]);
            double m = a * a + b * b;
            y[n] = (m > e) ? y[n] / sqrt(m) : 0;
        }
    }
}

int orc_phase(double complex *y, const float *x, unsigned N, int rule) {
    int rc = orc_analytic(y, x, N);
    if (rc) return rc;
    orc_ampnorm(y, N, rule);
    return 0;
}

/* PCC2, src/FFTapps.c:785-881: phase signals, zero padding to Nz, FFT,
 * conj(X1) X2 (:851), IFFT (:852), lags scaled by 1/(Nz*N) (:832,855-856). */
int orc_pcc2_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2, unsigned Nz, int rule) {
    int lag0; unsigned L;
    lag_window(Lag1, Lag2, &lag0, &L);
    if ((unsigned)abs(Lag1) >= N || (unsigned)abs(Lag2) >= N) return -3;   /* :803 */
    if (Nz == 0) Nz = orc_nz_rule(N, Lag1, Lag2);
    const double sc = 1.0 / ((double)Nz * (double)N);
    int err = 0;
    #pragma omp parallel for schedule(dynamic, 1) reduction(|:err)
    for (unsigned tr = 0; tr < Tr; tr++) {
        double complex *a = (double complex *)calloc(Nz, sizeof(double complex));
        double complex *b = (double complex *)calloc(Nz, sizeof(double complex));
        if (!a || !b) { free(a); free(b); err |= 1; continue; }
        orc_phase(a, x1 + (size_t)tr * N, N, rule);
        orc_phase(b, x2 + (size_t)tr * N, N, rule);
        for (unsigned n = N; n < Nz; n++) { a[n] = 0; b[n] = 0; }
        fft64_c2c(a, Nz, -1);
        fft64_c2c(b, Nz, -1);
        for (unsigned n = 0; n < Nz; n++) a[n] = conj(a[n]) * b[n];
        fft64_c2c(a, Nz, +1);
        double *yy = y + (size_t)tr * L;
        for (unsigned l = 0; l < L; l++) {
            int lag = lag0 + (int)l;
            unsigned idx = (lag < 0) ? (unsigned)(lag + (int)Nz) : (unsigned)lag;
            yy[l] = sc * creal(a[idx]);
        }
        free(a); free(b);
    }
    return err ? -2 : 0;
}

/* Direct lag sums, src/FFTapps.c:223-336 and src/ccs_cuda.cu:260-321,388-453:
 * y[lag] = sum_overlap (|p1[n]+p2[n+lag]|^v - |p1[n]-p2[n+lag]|^v) / D,
 * D = 2^(v/2)*(N-|lag|) (CPU, :305,334) or 2*(N-|lag|) (GPU, :320,452). */
static void pccv_one(double *y, const double complex *p1, const double complex *p2, unsigned N,
                     double v, int Lag1, int Lag2, int norm_gpu) {
    int Li = Lag2 - Lag1 + 1;
    if (Lag2 > (int)N) Li -= (Lag2 - (int)N);                 /* :286 */
    int l1 = (Lag1 >= -(int)N) ? 0 : -(Lag1 + (int)N);       /* :287 */
    const double V = v / 2;
    for (int l = 0; l < l1 && l < Li; l++) y[l] = 0;
    for (int l = l1; l < Li; l++) {
        int lag = Lag1 + l;
        unsigned n1, n2;
        if (lag < 0) { n1 = (unsigned)(-lag); n2 = N; }
        else         { n1 = 0; n2 = N - (unsigned)lag; }
        double acc = 0;
        for (unsigned i = 0; i < n2 - n1; i++) {
            /* p2 is shifted by lag relative to p1 (:237-238 with xan1 = station 2) */
            double complex a = p2[n1 + (unsigned)((int)i + lag)];
            double complex b = p1[n1 + i];
            double complex s = a + b, d = a - b;
            double s2 = creal(s) * creal(s) + cimag(s) * cimag(s);
            double d2 = creal(d) * creal(d) + cimag(d) * cimag(d);
            if (v == 1.0) acc += sqrt(s2) - sqrt(d2);
            else if (v == 2.0) acc += s2 - d2;
            else acc += pow(s2, V) - pow(d2, V);
        }
        double D = norm_gpu ? 2.0 * (double)(n2 - n1) : pow(2.0, V) * (double)(n2 - n1);
        y[l] = acc / D;
    }
}

int orc_pccv_phase(double *y, const double complex *p1, const double complex *p2, unsigned N,
                   double v, int Lag1, int Lag2, int norm_gpu) {
    pccv_one(y, p1, p2, N, v, Lag1, Lag2, norm_gpu);
    return 0;
}

int orc_pccv_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 double v, int Lag1, int Lag2, int rule, int norm_gpu) {
    if (Lag1 > (int)N || Lag2 < -(int)N) return 0;            /* :478 */
    int L = Lag2 - Lag1 + 1;
    if (L < 0) return -1;
    int err = 0;
    #pragma omp parallel for schedule(dynamic, 1) reduction(|:err)
    for (unsigned tr = 0; tr < Tr; tr++) {
        double complex *a = (double complex *)malloc((size_t)N * sizeof(double complex));
        double complex *b = (double complex *)malloc((size_t)N * sizeof(double complex));
        if (!a || !b) { free(a); free(b); err |= 1; continue; }
        orc_phase(a, x1 + (size_t)tr * N, N, rule);
        orc_phase(b, x2 + (size_t)tr * N, N, rule);
        pccv_one(y + (size_t)tr * (unsigned)L, a, b, N, v, Lag1, Lag2, norm_gpu);
        free(a); free(b);
    }
    return err ? -2 : 0;
}

/* GNCC, src/FFTapps.c:883-978: FP64 cross-correlation via zero-padded DFTs
 * (cc_lowlevel :338-353, scaled 1/Nz), divided by sqrt(E1*E2) with E the
 * energy of each trace over the overlap of that lag (gn_lowlevel :372-399). */
int orc_gncc_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2) {
    int lag0; unsigned L;
    lag_window(Lag1, Lag2, &lag0, &L);
    if ((unsigned)abs(Lag1) >= N || (unsigned)abs(Lag2) >= N) return -3;   /* :907 */
    const unsigned Nz = orc_nz_rule(N, Lag1, Lag2);
    int err = 0;
    #pragma omp parallel for schedule(dynamic, 1) reduction(|:err)
    for (unsigned tr = 0; tr < Tr; tr++) {
        const float *a1 = x1 + (size_t)tr * N, *a2 = x2 + (size_t)tr * N;
        double complex *A = (double complex *)calloc(Nz, sizeof(double complex));
        double complex *B = (double complex *)calloc(Nz, sizeof(double complex));
        double *P1 = (double *)malloc((size_t)(N + 1) * sizeof(double));
        double *P2 = (double *)malloc((size_t)(N + 1) * sizeof(double));
        if (!A || !B || !P1 || !P2) { free(A); free(B); free(P1); free(P2); err |= 1; continue; }
        for (unsigned n = 0; n < N; n++) { A[n] = (double)a1[n]; B[n] = (double)a2[n]; }
        fft64_c2c(A, Nz, -1);
        fft64_c2c(B, Nz, -1);
        for (unsigned n = 0; n < Nz; n++) A[n] = conj(A[n]) * B[n];
        fft64_c2c(A, Nz, +1);
        P1[0] = 0; P2[0] = 0;
        for (unsigned n = 0; n < N; n++) {
            P1[n + 1] = P1[n] + (double)a1[n] * (double)a1[n];
            P2[n + 1] = P2[n] + (double)a2[n] * (double)a2[n];
        }
        double *yy = y + (size_t)tr * L;
        for (unsigned l = 0; l < L; l++) {
            int lag = lag0 + (int)l;
            unsigned idx = (lag < 0) ? (unsigned)(lag + (int)Nz) : (unsigned)lag;
            /* overlap: x1[n11,n12) and x2[n21,n22) (:896-902) */
            unsigned n11 = 0, n21 = 0, n12 = N, n22 = N;
            if (lag > 0) { n21 = (unsigned)lag; n12 -= (unsigned)lag; }
            else { n11 = (unsigned)(-lag); n22 -= (unsigned)(-lag); }
            double e1 = P1[n12] - P1[n11], e2 = P2[n22] - P2[n21];
            yy[l] = (creal(A[idx]) / (double)Nz) / sqrt(e1 * e2);
        }
        free(A); free(B); free(P1); free(P2);
    }
    return err ? -2 : 0;
}

/* 1-bit GNCC, src/FFTapps.c:980-1073: signs s1 = x1>=0 ? +1 : -1 (:1037),
 * s2 = x2>0 ? +1 : -1 (:1042); the overlap norms are overlap counts, so
 * y = (sum s1[n] s2[n+lag]) / (N-|lag|).  The numerator is computed exactly. */
static void cc1b_num_one(int64_t *num, const float *a1, const float *a2, unsigned N, int lag0, unsigned L) {
    for (unsigned l = 0; l < L; l++) {
        int lag = lag0 + (int)l;
        unsigned n1 = lag < 0 ? (unsigned)(-lag) : 0;
        unsigned n2 = lag < 0 ? N : N - (unsigned)lag;
        int64_t acc = 0;
        for (unsigned n = n1; n < n2; n++) {
            int s1 = (a1[n] >= 0) ? 1 : -1;
            int s2 = (a2[(int)n + lag] > 0) ? 1 : -1;
            acc += s1 * s2;
        }
        num[l] = acc;
    }
}

int orc_cc1b_num(int64_t *num, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2) {
    int lag0; unsigned L;
    lag_window(Lag1, Lag2, &lag0, &L);
    if ((unsigned)abs(Lag1) >= N || (unsigned)abs(Lag2) >= N) return -3;   /* :1006 */
    #pragma omp parallel for schedule(dynamic, 1)
    for (unsigned tr = 0; tr < Tr; tr++)
        cc1b_num_one(num + (size_t)tr * L, x1 + (size_t)tr * N, x2 + (size_t)tr * N, N, lag0, L);
    return 0;
}

int orc_cc1b_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2) {
    int lag0; unsigned L;
    lag_window(Lag1, Lag2, &lag0, &L);
    if ((unsigned)abs(Lag1) >= N || (unsigned)abs(Lag2) >= N) return -3;
    int64_t *num = (int64_t *)malloc((size_t)Tr * L * sizeof(int64_t));
    if (!num) return -2;
    orc_cc1b_num(num, x1, x2, N, Tr, Lag1, Lag2);
    for (unsigned tr = 0; tr < Tr; tr++)
        for (unsigned l = 0; l < L; l++) {
            int lag = lag0 + (int)l;
            y[(size_t)tr * L + l] = (double)num[(size_t)tr * L + l] / (double)(N - (unsigned)abs(lag));
        }
    free(num);
    return 0;
}

/* ---- wavelet family, src/FWTa/wavelet_def_v7.c ---------------------------- */

/* erfi by its Maclaurin series, 2/sqrt(pi) * sum z^(2n+1) / (n! (2n+1)),
 * 500 terms as in wavelet_def_v7.c:104-117. */
static double orc_erfi(double z) {
    double term = z, out = z, zz = z * z;
    for (unsigned n = 1; n < 500; n++) {
        term *= zz / n;
        out += term / (2 * n + 1);
    }
    return out * 2 / sqrt(ORC_PI);
}

unsigned orc_wavelet_family(int type, unsigned J, unsigned V, unsigned Nz, double s0,
                            double op1, double *scale, unsigned *Ls, int *center,
                            double complex *taps) {
    const unsigned S = J * V;
    /* setscales0 :299-309 */
    double s = s0, q = pow(2.0, 1.0 / (double)V);
    for (unsigned k = 0; k < S; k++) { scale[k] = s; s *= q; }
    /* setwaveletlength0 :312-322 (5 sigmas, capped at Nz) */
    unsigned total = 0;
    for (unsigned k = 0; k < S; k++) {
        unsigned l = 2 * (unsigned)ceil(5 * scale[k]) + 1;
        Ls[k] = l > Nz ? Nz : l;
        total += Ls[k];
    }
    double complex *w = taps;
    for (unsigned k = 0; k < S; k++) {
        const unsigned L = Ls[k];
        const int u0 = (int)(L / 2);
        center[k] = u0;
        if (!w) continue;
        const double sc = scale[k];
        for (int u = -u0; u < (int)L - u0; u++) {
            double d = (double)u / sc;
            double complex val;
            if (type == -1) {          /* MorletFun :38-52 */
                double kk = 1 / sqrt(sqrt(ORC_PI) * sc);
                val = kk * cexp(I * op1 * d) * exp(-0.5 * d * d);
            } else if (type == -2) {   /* Complete_MorletFun :71-87 */
                double kk = 1 / sqrt(sqrt(ORC_PI) * sc);
                double ze = exp(-op1 * op1 / 2);
                val = kk * exp(-0.5 * d * d) * (cexp(I * op1 * d) - ze);
            } else {                   /* MexicanHatFun :119-131 */
                double kk = 2 / sqrt(3 * sqrt(ORC_PI) * sc);
                val = kk * ((d * d - 1) * exp(-d * d / 2) * (1 + I * orc_erfi(d / sqrt(2.0)))
                            - I * sqrt(2 / ORC_PI) * d);
            }
            *w++ = val;
        }
    }
    return total;
}

unsigned orc_wpcc_setup(unsigned N, int Lag1, int Lag2, double pmin, double pmax,
                        unsigned V, int type, double op1_in, unsigned *Nz_out,
                        double *s0_out, double *op1_out, unsigned *J_out) {
    /* src/FFTapps.c:1087-1112 */
    unsigned ua1 = (unsigned)abs(Lag1), ua2 = (unsigned)abs(Lag2);
    if (ua1 >= N || ua2 >= N) return 0;
    unsigned M = ua1 > ua2 ? ua1 : ua2;
    unsigned Nz = 1u << (unsigned)ceil(log2((double)(N + M)));
    double s0, op1 = op1_in;
    if (type == -3) s0 = pmin / (sqrt(2.0) * ORC_PI);
    else if (type == -1 || type == -2) {
        if (op1 == 0) op1 = ORC_PI * sqrt(2 / log(2.0));
        s0 = pmin * op1 / (2 * ORC_PI);
    } else return 0;
    unsigned J = (unsigned)round(1. / (double)V + log(pmax / pmin) / log(2.0));
    unsigned S = V * J;
    if (S == 0) return 0;
    double *scale = (double *)malloc(S * sizeof(double));
    unsigned *Ls = (unsigned *)malloc(S * sizeof(unsigned));
    int *center = (int *)malloc(S * sizeof(int));
    orc_wavelet_family(type, J, V, Nz, s0, op1, scale, Ls, center, NULL);
    unsigned Ls0 = Ls[S - 1];
    if (Nz - (N + M) < Ls0) Nz *= 2;     /* :1112 */
    free(scale); free(Ls); free(center);
    *Nz_out = Nz; *s0_out = s0; *op1_out = op1; *J_out = J;
    return S;
}

/* WPCC, src/FFTapps.c:1076-1255 (CPU path).  Wavelet spectra from the taps
 * placed circularly around index 0 (:1140-1147); each trace is scaled by 1/Nz
 * and placed at offset Ls0 = Ls[S-1] (:1185-1197); per scale s the band is
 * IDFT(X W_s), amplitude-normalised and transformed back, and the cross
 * spectrum sum_s conj(P1_s) P2_s / (scale_s Nz) is inverted (:1200-1220);
 * lags are scaled by C = 1/(K0 N), K0 = sum_s 1/scale_s (:1114-1120,1223-1224). */
int orc_wpcc_band(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                  int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type,
                  double op1, int rule, unsigned s_lo, unsigned s_hi) {
    unsigned Nz, J; double s0, op1v;
    unsigned S = orc_wpcc_setup(N, Lag1, Lag2, pmin, pmax, V, type, op1, &Nz, &s0, &op1v, &J);
    if (S == 0) return -3;
    /* the family is built with the pre-doubling Nz as length cap (:1108) */
    unsigned ua1 = (unsigned)abs(Lag1), ua2 = (unsigned)abs(Lag2);
    unsigned M = ua1 > ua2 ? ua1 : ua2;
    unsigned Nz0 = 1u << (unsigned)ceil(log2((double)(N + M)));
    double *scale = (double *)malloc(S * sizeof(double));
    unsigned *Ls = (unsigned *)malloc(S * sizeof(unsigned));
    int *center = (int *)malloc(S * sizeof(int));
    unsigned ntap = orc_wavelet_family(type, J, V, Nz0, s0, op1v, scale, Ls, center, NULL);
    double complex *taps = (double complex *)malloc((size_t)ntap * sizeof(double complex));
    orc_wavelet_family(type, J, V, Nz0, s0, op1v, scale, Ls, center, taps);
    const unsigned Ls0 = Ls[S - 1];
    double K0 = 0;
    for (unsigned s = 0; s < S; s++) K0 += 1 / scale[s];
    const double C = 1. / (K0 * (double)N);
    int lag0 = (Lag2 >= Lag1) ? Lag1 : Lag2;
    unsigned L = (unsigned)abs(Lag2 - Lag1 + 1);   /* :1084 */

    double complex *fw = (double complex *)calloc((size_t)S * Nz, sizeof(double complex));
    {
        const double complex *pc = taps;
        for (unsigned s = 0; s < S; s++) {
            double complex *f = fw + (size_t)s * Nz;
            int c = center[s]; unsigned l = Ls[s];
            for (unsigned n = 0; n < l - (unsigned)c; n++) f[n] = pc[c + n];
            for (int n = 0; n < c; n++) f[Nz - c + n] = pc[n];
            fft64_c2c(f, Nz, -1);
            pc += l;
        }
    }
    const double da2 = 1. / (double)Nz;
    #pragma omp parallel for schedule(dynamic, 1)
    for (unsigned tr = 0; tr < Tr; tr++) {
        double complex *in1 = (double complex *)calloc(Nz, sizeof(double complex));
        double complex *in2 = (double complex *)calloc(Nz, sizeof(double complex));
        double complex *w1 = (double complex *)malloc((size_t)Nz * sizeof(double complex));
        double complex *w2 = (double complex *)malloc((size_t)Nz * sizeof(double complex));
        double complex *yw = (double complex *)calloc(Nz, sizeof(double complex));
        const float *a1 = x1 + (size_t)tr * N, *a2 = x2 + (size_t)tr * N;
        for (unsigned n = 0; n < N; n++) { in1[Ls0 + n] = da2 * a1[n]; in2[Ls0 + n] = da2 * a2[n]; }
        fft64_c2c(in1, Nz, -1);
        fft64_c2c(in2, Nz, -1);
        for (unsigned s = s_lo; s < S && s < s_hi; s++) {
            const double complex *f = fw + (size_t)s * Nz;
            for (unsigned n = 0; n < Nz; n++) { w1[n] = in1[n] * f[n]; w2[n] = in2[n] * f[n]; }
            fft64_c2c(w1, Nz, +1); orc_ampnorm(w1, Nz, rule); fft64_c2c(w1, Nz, -1);
            fft64_c2c(w2, Nz, +1); orc_ampnorm(w2, Nz, rule); fft64_c2c(w2, Nz, -1);
            const double d3 = 1. / (scale[s] * (double)Nz);
            for (unsigned n = 0; n < Nz; n++) yw[n] += d3 * conj(w1[n]) * w2[n];
        }
        fft64_c2c(yw, Nz, +1);
        double *yy = y + (size_t)tr * L;
        for (unsigned l = 0; l < L; l++) {
            int lag = lag0 + (int)l;
            unsigned idx = (lag < 0) ? (unsigned)(lag + (int)Nz) : (unsigned)lag;
            yy[l] = C * creal(yw[idx]);
        }
        free(in1); free(in2); free(w1); free(w2); free(yw);
    }
    free(fw); free(taps); free(scale); free(Ls); free(center);
    return 0;
}

int orc_wpcc_set(double *y, const float *x1, const float *x2, unsigned N, unsigned Tr,
                 int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type,
                 double op1, int rule) {
    return orc_wpcc_band(y, x1, x2, N, Tr, Lag1, Lag2, pmin, pmax, V, type, op1, rule, 0, ~0u);
}

/* ---- stacking of correlation traces ---------------------------------------
 * The consumer of the obin files (src/PCC_fullpair_1b.c:568-569) stacks the
 * per-window correlations of a channel pair.  Its source is not part of the
 * reference; the stacks here restate the published methods on the reference's
 * own wavelet library (src/FWTa):
 *   linear:  mean_j c_j[n]
 *   PWS:     linear * |mean_j a_j[n] / |a_j[n]||^nu, a_j the analytic signal of
 *            trace j (Schimmel & Paulssen 1997), by the analytic-signal rule of
 *            src/FFTapps.c:45-80
 *   ts-PWS:  inverse CWT of  |mean_j W_j / |W_j||^nu * mean_j W_j,  W_j the CWT of
 *            trace j (Ventosa, Schimmel & Stutzmann 2017), with the CWT of
 *            complex_1D_wavelet_dec (src/FWTa/wavelet_v7.c:43-64, cdotx_dc
 *            src/FWTa/cdotx.c:35-71: circular, conjugate taps) and the inverse of
 *            Re_complex_1D_wavelet_rec (wavelet_v7.c:124-150: the dual frame of
 *            FillDualFrame wavelet_def_v7.c:152-190 through re_cdotx_cc,
 *            cdotx.c:176-211, weighted by ln(a0) / (2 Cpsi V scale_s), a0 = 2).
 * Phasors of zero modulus count as zero. */

/* Morlet_Cpsi (src/FWTa/wavelet_def_v7.c:133-144, the same running sum) and
 * MexicanHat_Cpsi (:146-148). */
double orc_cpsi(int type, double w0) {
    if (type == -3) return (4. / 3.) * sqrt(ORC_PI);
    double c = 0;
    for (double w = 0.01; w < 100; w += 0.01) {
        double a = w - w0;
        c += exp(-a * a) / w;
    }
    return c * 0.01 * sqrt(ORC_PI) / 2;
}

/* Family of a ts-PWS stack over traces of L samples: s0 and the default w0
 * from pmin as src/FFTapps.c:1097-1105, J = round(1/V + log2(pmax/pmin)) (:1106),
 * taps capped at L (CreateWaveletFamily with N = L).  Returns S or 0. */
unsigned orc_stack_family(unsigned L, double pmin, double pmax, unsigned V, int type, double op1_in,
                          double *s0_out, double *op1_out, unsigned *J_out) {
    double s0, op1 = op1_in;
    if (type == -3) s0 = pmin / (sqrt(2.0) * ORC_PI);
    else if (type == -1 || type == -2) {
        if (op1 == 0) op1 = ORC_PI * sqrt(2 / log(2.0));
        s0 = pmin * op1 / (2 * ORC_PI);
    } else return 0;
    if (V == 0 || !(pmax > pmin) || !(pmin > 0) || L == 0) return 0;
    unsigned J = (unsigned)round(1. / (double)V + log(pmax / pmin) / log(2.0));
    *s0_out = s0; *op1_out = op1; *J_out = J;
    return J * V;
}

/* CWT of one real trace: W[s*L + n] = sum_l x[(n - c_s + l) mod L] conj(w_s[l]). */
void orc_cwt(double complex *W, const double *x, unsigned L, unsigned S, const unsigned *Ls,
             const int *center, const double complex *taps) {
    const double complex *w = taps;
    for (unsigned s = 0; s < S; s++) {
        for (unsigned n = 0; n < L; n++) {
            double complex acc = 0;
            for (unsigned l = 0; l < Ls[s]; l++) {
                long m = ((long)n - center[s] + (long)l) % (long)L;
                if (m < 0) m += L;
                acc += x[m] * conj(w[l]);
            }
            W[(size_t)s * L + n] = acc;
        }
        w += Ls[s];
    }
}

/* Inverse: x[n] = sum_s ln2 / (2 Cpsi V scale_s) Re sum_l w_s[l] W[s][(n + c_s - l) mod L]. */
void orc_icwt(double *x, const double complex *W, unsigned L, unsigned S, unsigned V, double cpsi,
              const double *scale, const unsigned *Ls, const int *center, const double complex *taps) {
    for (unsigned n = 0; n < L; n++) x[n] = 0;
    const double complex *w = taps;
    for (unsigned s = 0; s < S; s++) {
        const double aux = log(2.0) / (2 * cpsi * V * scale[s]);
        for (unsigned n = 0; n < L; n++) {
            double acc = 0;
            for (unsigned l = 0; l < Ls[s]; l++) {
                long m = ((long)n + center[s] - (long)l) % (long)L;
                if (m < 0) m += L;
                acc += creal(w[l] * W[(size_t)s * L + m]);
            }
            x[n] += aux * acc;
        }
        w += Ls[s];
    }
}

static double complex unit(double complex z) {
    const double a = cabs(z);
    return a > 0 ? z / a : 0;
}

int orc_stack(double *out, const float *y, unsigned K, unsigned L, int mode, double nu, double pmin,
              double pmax, unsigned V, int type, double op1) {
    if (!out || !y || K == 0 || L == 0) return -1;
    double *lin = (double *)calloc(L, sizeof(double));
    for (unsigned j = 0; j < K; j++)
        for (unsigned n = 0; n < L; n++) lin[n] += (double)y[(size_t)j * L + n];
    for (unsigned n = 0; n < L; n++) lin[n] /= K;
    if (mode == 0) {
        memcpy(out, lin, L * sizeof(double));
        free(lin);
        return 0;
    }
    if (mode == 1) {
        double complex *a = (double complex *)malloc(L * sizeof(double complex));
        double complex *u = (double complex *)calloc(L, sizeof(double complex));
        for (unsigned j = 0; j < K; j++) {
            orc_analytic(a, y + (size_t)j * L, L);
            for (unsigned n = 0; n < L; n++) u[n] += unit(a[n]);
        }
        for (unsigned n = 0; n < L; n++) out[n] = lin[n] * pow(cabs(u[n]) / K, nu);
        free(a); free(u); free(lin);
        return 0;
    }
    if (mode != 2) { free(lin); return -3; }
    double s0, op;
    unsigned J;
    const unsigned S = orc_stack_family(L, pmin, pmax, V, type, op1, &s0, &op, &J);
    if (!S) { free(lin); return -3; }
    double *scale = (double *)malloc(S * sizeof(double));
    unsigned *Ls = (unsigned *)malloc(S * sizeof(unsigned));
    int *center = (int *)malloc(S * sizeof(int));
    const unsigned nt = orc_wavelet_family(type, J, V, L, s0, op, scale, Ls, center, NULL);
    double complex *taps = (double complex *)malloc(nt * sizeof(double complex));
    orc_wavelet_family(type, J, V, L, s0, op, scale, Ls, center, taps);
    double complex *W = (double complex *)malloc((size_t)S * L * sizeof(double complex));
    double complex *U = (double complex *)calloc((size_t)S * L, sizeof(double complex));
    double complex *Wl = (double complex *)malloc((size_t)S * L * sizeof(double complex));
    double *x = (double *)malloc(L * sizeof(double));
    for (unsigned j = 0; j < K; j++) {
        for (unsigned n = 0; n < L; n++) x[n] = (double)y[(size_t)j * L + n];
        orc_cwt(W, x, L, S, Ls, center, taps);
        for (size_t i = 0; i < (size_t)S * L; i++) U[i] += unit(W[i]);
    }
    orc_cwt(Wl, lin, L, S, Ls, center, taps);        /* mean_j W_j by linearity */
    for (size_t i = 0; i < (size_t)S * L; i++) Wl[i] *= pow(cabs(U[i]) / K, nu);
    orc_icwt(out, Wl, L, S, V, orc_cpsi(type, op), scale, Ls, center, taps);
    free(scale); free(Ls); free(center); free(taps); free(W); free(U); free(Wl); free(x); free(lin);
    return 0;
}
