/*
 * ref_wt — test harness over the reference's own wavelet library (src/FWTa),
 * compiled from the reference sources by `make -C oracle wt` into
 * oracle/_ref/libref_wt.so.  TEST INFRASTRUCTURE ONLY: it pins the oracle's
 * CWT and inverse CWT (oracle64.c orc_cwt / orc_icwt) and its ts-PWS stack
 * against CreateWaveletFamily, complex_1D_wavelet_dec and
 * Re_complex_1D_wavelet_rec themselves.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "wavelet_v7.h"

/* Family as src/FFTapps.c:1107 builds it (continuous frame, circular). */
static t_WaveletFamily *family(int type, unsigned J, unsigned V, unsigned L, double s0, double op1) {
    return CreateWaveletFamily(type, J, V, L, s0, 0.5, 0, op1, 1);
}

/* W (S x L) = the reference CWT of x; xrec (L) = its reference inverse. */
int ref_wt_pair(double complex *W, double *xrec, const double *x, unsigned L, int type, unsigned J, unsigned V,
                double s0, double op1) {
    t_WaveletFamily *pWF = family(type, J, V, L, s0, op1);
    if (!pWF) return -1;
    t_CWTvar *y = CreateComplexWaveletVar(pWF, L);
    double *xx = (double *)malloc(L * sizeof(double));
    memcpy(xx, x, L * sizeof(double));
    int er = complex_1D_wavelet_dec(y, xx, L, pWF);
    for (unsigned s = 0; s < pWF->Ns && !er; s++) memcpy(W + (size_t)s * L, y->d[s], L * sizeof(double complex));
    if (!er) er = Re_complex_1D_wavelet_rec(xrec, y, L, pWF);
    free(xx);
    DestroyComplexWaveletVar(y);
    DestroyWaveletFamily(pWF);
    return er;
}

/* ts-PWS of K traces of L samples (row-major, float) on the reference transforms:
 * inverse of |mean_j W_j/|W_j||^nu * CWT(mean_j c_j). */
int ref_wt_tspws(double *out, const float *c, unsigned K, unsigned L, double nu, int type, unsigned J, unsigned V,
                 double s0, double op1) {
    t_WaveletFamily *pWF = family(type, J, V, L, s0, op1);
    if (!pWF) return -1;
    const unsigned S = pWF->Ns;
    t_CWTvar *y = CreateComplexWaveletVar(pWF, L);
    double complex *U = (double complex *)calloc((size_t)S * L, sizeof(double complex));
    double *x = (double *)malloc(L * sizeof(double));
    double *lin = (double *)calloc(L, sizeof(double));
    int er = 0;
    for (unsigned j = 0; j < K && !er; j++) {
        for (unsigned n = 0; n < L; n++) {
            x[n] = (double)c[(size_t)j * L + n];
            lin[n] += x[n] / K;
        }
        er = complex_1D_wavelet_dec(y, x, L, pWF);
        for (unsigned s = 0; s < S && !er; s++)
            for (unsigned n = 0; n < L; n++) {
                const double complex w = y->d[s][n];
                const double a = cabs(w);
                if (a > 0) U[(size_t)s * L + n] += w / a;
            }
    }
    if (!er) er = complex_1D_wavelet_dec(y, lin, L, pWF);
    for (unsigned s = 0; s < S && !er; s++)
        for (unsigned n = 0; n < L; n++) y->d[s][n] *= pow(cabs(U[(size_t)s * L + n]) / K, nu);
    if (!er) er = Re_complex_1D_wavelet_rec(out, y, L, pWF);
    free(U); free(x); free(lin);
    DestroyComplexWaveletVar(y);
    DestroyWaveletFamily(pWF);
    return er;
}
