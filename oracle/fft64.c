/*
 * fft64 — FP64 DFT for the CPU oracle (test infrastructure only; see fft64.h).
 *
 * Stockham autosort, one pass per radix factor R (Ns = product of the radices
 * already applied):
 *     for j in [0, n/R):  k = j mod Ns
 *         v[r] = a[j + r*n/R] * w^(r*k),   w = exp(sign*2*pi*i/(Ns*R))
 *         v    = DFT_R(v)
 *         b[(j/Ns)*Ns*R + k + r*Ns] = v[r]
 * which leaves the result in natural order.  Lengths with a prime factor above 7
 * go through Bluestein's chirp-z identity with a power-of-two inner transform.
 */
#include "fft64.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define FFT64_PI 3.14159265358979323846264338327950288

typedef struct plan64 {
    unsigned n;
    int nrad;
    unsigned rad[64];
    double complex *tw;      /* exp(-2*pi*i*t/n), t in [0, n) */
    /* Bluestein */
    int blue;
    unsigned m;              /* inner power-of-two length */
    double complex *chirp;   /* exp(-pi*i*k^2/n), k in [0, n) */
    double complex *bspec;   /* DFT_m of the conjugate chirp filter */
    struct plan64 *inner;
    struct plan64 *next;
} plan64;

static plan64 *g_plans = NULL;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static int factorise(unsigned n, unsigned *rad) {
    int k = 0;
    while (n % 4 == 0) { rad[k++] = 4; n /= 4; }
    while (n % 2 == 0) { rad[k++] = 2; n /= 2; }
    while (n % 3 == 0) { rad[k++] = 3; n /= 3; }
    while (n % 5 == 0) { rad[k++] = 5; n /= 5; }
    while (n % 7 == 0) { rad[k++] = 7; n /= 7; }
    return (n == 1) ? k : -1;
}

static plan64 *plan_get(unsigned n);

static plan64 *plan_build(unsigned n) {
    plan64 *p = (plan64 *)calloc(1, sizeof(plan64));
    if (!p) return NULL;
    p->n = n;
    p->nrad = factorise(n, p->rad);
    if (p->nrad >= 0) {
        p->tw = (double complex *)malloc((size_t)n * sizeof(double complex));
        for (unsigned t = 0; t < n; t++) {
            double a = -2.0 * FFT64_PI * (double)t / (double)n;
            p->tw[t] = cos(a) + I * sin(a);
        }
        return p;
    }
    /* Bluestein */
    p->blue = 1;
    unsigned m = 1;
    while (m < 2 * n - 1) m <<= 1;
    p->m = m;
    p->chirp = (double complex *)malloc((size_t)n * sizeof(double complex));
    p->bspec = (double complex *)calloc(m, sizeof(double complex));
    for (unsigned k = 0; k < n; k++) {
        /* k^2 mod 2n keeps the angle exact for large k */
        unsigned long long kk = ((unsigned long long)k * k) % (2ull * n);
        double a = -FFT64_PI * (double)kk / (double)n;
        p->chirp[k] = cos(a) + I * sin(a);
    }
    p->bspec[0] = conj(p->chirp[0]);
    for (unsigned k = 1; k < n; k++) {
        p->bspec[k] = conj(p->chirp[k]);
        p->bspec[m - k] = conj(p->chirp[k]);
    }
    p->inner = plan_get(m);
    return p;
}

static plan64 *plan_get(unsigned n) {
    /* caller may or may not hold the lock: plan_get is only called with it held */
    for (plan64 *p = g_plans; p; p = p->next)
        if (p->n == n) return p;
    plan64 *p = plan_build(n);
    if (!p) return NULL;
    if (p->blue) {
        /* the filter spectrum needs the inner plan, which now exists */
        p->next = g_plans;
        g_plans = p;
        return p;
    }
    p->next = g_plans;
    g_plans = p;
    return p;
}

static void stockham(const plan64 *p, double complex *a, double complex *b, int sign) {
    const unsigned n = p->n;
    unsigned Ns = 1;
    double complex *src = a, *dst = b;
    for (int s = 0; s < p->nrad; s++) {
        const unsigned R = p->rad[s];
        const unsigned m = n / R;
        const unsigned step = n / (Ns * R);   /* twiddle table stride for w */
        double complex root[7];
        for (unsigned q = 0; q < R; q++) {
            double ang = sign * 2.0 * FFT64_PI * (double)q / (double)R;
            root[q] = cos(ang) + I * sin(ang);
        }
        for (unsigned j = 0; j < m; j++) {
            unsigned k = j % Ns;
            double complex v[7], o[7];
            for (unsigned r = 0; r < R; r++) {
                double complex w = p->tw[((unsigned long long)r * k * step) % n];
                if (sign > 0) w = conj(w);
                v[r] = src[j + r * m] * w;
            }
            for (unsigned q = 0; q < R; q++) {
                double complex acc = 0;
                for (unsigned r = 0; r < R; r++) acc += v[r] * root[(q * r) % R];
                o[q] = acc;
            }
            unsigned base = (j / Ns) * Ns * R + k;
            for (unsigned r = 0; r < R; r++) dst[base + r * Ns] = o[r];
        }
        double complex *t = src; src = dst; dst = t;
        Ns *= R;
    }
    if (src != a) memcpy(a, src, (size_t)n * sizeof(double complex));
}

static int run_plan(const plan64 *p, double complex *x, int sign) {
    if (!p->blue) {
        double complex *tmp = (double complex *)malloc((size_t)p->n * sizeof(double complex));
        if (!tmp) return -1;
        stockham(p, x, tmp, sign);
        free(tmp);
        return 0;
    }
    const unsigned n = p->n, m = p->m;
    double complex *a = (double complex *)calloc(m, sizeof(double complex));
    double complex *bs = (double complex *)malloc((size_t)m * sizeof(double complex));
    if (!a || !bs) { free(a); free(bs); return -1; }
    /* forward: X[k] = c[k] * sum_j (x[j] c[j]) conj(c[k-j]),  c = exp(-pi i k^2/n)
     * backward uses the conjugate chirp. */
    for (unsigned k = 0; k < n; k++) {
        double complex c = (sign < 0) ? p->chirp[k] : conj(p->chirp[k]);
        a[k] = x[k] * c;
    }
    memcpy(bs, p->bspec, (size_t)m * sizeof(double complex));
    if (sign > 0) {
        for (unsigned k = 0; k < m; k++) bs[k] = conj(bs[k]);
    }
    run_plan(p->inner, bs, -1);
    run_plan(p->inner, a, -1);
    for (unsigned k = 0; k < m; k++) a[k] *= bs[k];
    run_plan(p->inner, a, +1);
    const double sc = 1.0 / (double)m;
    for (unsigned k = 0; k < n; k++) {
        double complex c = (sign < 0) ? p->chirp[k] : conj(p->chirp[k]);
        x[k] = a[k] * sc * c;
    }
    free(a);
    free(bs);
    return 0;
}

int fft64_c2c(double complex *x, unsigned n, int sign) {
    if (n == 0 || x == NULL) return -1;
    if (n == 1) return 0;
    pthread_mutex_lock(&g_lock);
    plan64 *p = plan_get(n);
    pthread_mutex_unlock(&g_lock);
    if (!p) return -1;
    return run_plan(p, x, sign < 0 ? -1 : +1);
}

int fft64_r2c(double complex *y, const double *x, unsigned n) {
    double complex *t = (double complex *)malloc((size_t)n * sizeof(double complex));
    if (!t) return -1;
    for (unsigned i = 0; i < n; i++) t[i] = x[i];
    int rc = fft64_c2c(t, n, -1);
    for (unsigned i = 0; i <= n / 2; i++) y[i] = t[i];
    free(t);
    return rc;
}

int fft64_c2r(double *y, const double complex *x, unsigned n) {
    double complex *t = (double complex *)malloc((size_t)n * sizeof(double complex));
    if (!t) return -1;
    for (unsigned i = 0; i <= n / 2; i++) t[i] = x[i];
    for (unsigned i = n / 2 + 1; i < n; i++) t[i] = conj(x[n - i]);
    /* FFTW's c2r ignores the imaginary parts of the DC and Nyquist bins */
    t[0] = creal(t[0]);
    if (!(n & 1)) t[n / 2] = creal(t[n / 2]);
    int rc = fft64_c2c(t, n, +1);
    for (unsigned i = 0; i < n; i++) y[i] = creal(t[i]);
    free(t);
    return rc;
}

void fft64_cleanup(void) {
    pthread_mutex_lock(&g_lock);
    plan64 *p = g_plans;
    while (p) {
        plan64 *nx = p->next;
        free(p->tw);
        free(p->chirp);
        free(p->bspec);
        free(p);
        p = nx;
    }
    g_plans = NULL;
    pthread_mutex_unlock(&g_lock);
}
