/*
 * FFTW-3 API subset implemented on the oracle's FP64 DFT (test infrastructure
 * only; see fftw3.h).
 */
#include <complex.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"
#include "../fft64.h"

enum { K_C2C = 0, K_R2C = 1, K_C2R = 2 };

struct fftw_shim_plan_s {
    int kind;
    int single;    /* 1: fftwf_* arrays (float), 0: double */
    int n;
    int sign;
    void *in;
    void *out;
};

void *fftw_malloc(size_t n) { void *p = NULL; if (posix_memalign(&p, 64, n ? n : 1)) return NULL; return p; }
void fftw_free(void *p) { free(p); }
void *fftwf_malloc(size_t n) { return fftw_malloc(n); }
void fftwf_free(void *p) { free(p); }

static struct fftw_shim_plan_s *mk(int kind, int single, int n, int sign, void *in, void *out) {
    struct fftw_shim_plan_s *p = (struct fftw_shim_plan_s *)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->kind = kind; p->single = single; p->n = n; p->sign = sign; p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
    (void)flags; return mk(K_C2C, 0, n, sign, in, out);
}
fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags) {
    (void)flags; return mk(K_R2C, 0, n, -1, in, out);
}
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags) {
    (void)flags; return mk(K_C2R, 0, n, +1, in, out);
}
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags) {
    (void)flags; return mk(K_C2C, 1, n, sign, in, out);
}
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags) {
    (void)flags; return mk(K_R2C, 1, n, -1, in, out);
}
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags) {
    (void)flags; return mk(K_C2R, 1, n, +1, in, out);
}

static void run(const struct fftw_shim_plan_s *p) {
    const unsigned n = (unsigned)p->n;
    const unsigned nh = n / 2 + 1;
    if (p->kind == K_C2C) {
        double complex *t = (double complex *)malloc((size_t)n * sizeof(double complex));
        if (p->single) { const float complex *a = (const float complex *)p->in; for (unsigned i = 0; i < n; i++) t[i] = a[i]; }
        else memcpy(t, p->in, (size_t)n * sizeof(double complex));
        fft64_c2c(t, n, p->sign);
        if (p->single) { float complex *b = (float complex *)p->out; for (unsigned i = 0; i < n; i++) b[i] = (float complex)t[i]; }
        else memcpy(p->out, t, (size_t)n * sizeof(double complex));
        free(t);
    } else if (p->kind == K_R2C) {
        double *r = (double *)malloc((size_t)n * sizeof(double));
        double complex *t = (double complex *)malloc((size_t)nh * sizeof(double complex));
        if (p->single) { const float *a = (const float *)p->in; for (unsigned i = 0; i < n; i++) r[i] = a[i]; }
        else memcpy(r, p->in, (size_t)n * sizeof(double));
        fft64_r2c(t, r, n);
        if (p->single) { float complex *b = (float complex *)p->out; for (unsigned i = 0; i < nh; i++) b[i] = (float complex)t[i]; }
        else memcpy(p->out, t, (size_t)nh * sizeof(double complex));
        free(r); free(t);
    } else {
        double complex *t = (double complex *)malloc((size_t)nh * sizeof(double complex));
        double *r = (double *)malloc((size_t)n * sizeof(double));
        if (p->single) { const float complex *a = (const float complex *)p->in; for (unsigned i = 0; i < nh; i++) t[i] = a[i]; }
        else memcpy(t, p->in, (size_t)nh * sizeof(double complex));
        fft64_c2r(r, t, n);
        if (p->single) { float *b = (float *)p->out; for (unsigned i = 0; i < n; i++) b[i] = (float)r[i]; }
        else memcpy(p->out, r, (size_t)n * sizeof(double));
        free(r); free(t);
    }
}

void fftw_execute(const fftw_plan p) { if (p) run(p); }
void fftwf_execute(const fftwf_plan p) { if (p) run(p); }
void fftw_destroy_plan(fftw_plan p) { free(p); }
void fftwf_destroy_plan(fftwf_plan p) { free(p); }
