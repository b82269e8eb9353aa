/*
 * Drop-in replacement of the reference's GPU boundary (FastPCC src/ccs_cuda.h:8-18).
 *
 * libfastpcc_gb300.so exports these four functions with the reference's
 * signatures and semantics, so src/FFTapps.c built with -DCUDAON links against
 * it in place of ccs_cuda.o:
 *
 *   pcc_highlevel        replaces src/ccs_cuda.cu:539-606   (PCC at power v; caller src/FFTapps.c:543)
 *   pcc1_highlevel       replaces src/ccs_cuda.cu:657-724   (PCC1;           caller src/FFTapps.c:680)
 *   pcc1_highlevel2      replaces src/ccs_cuda.cu:796-870   (no live caller; src/FFTapps.c:745 is disabled)
 *   cuda_tspcc2_set_freq replaces src/ccs_cuda.cu:898-1036  (WPCC;           caller src/FFTapps.c:1122)
 *
 * x1, x2 for the PCC calls are the analytic signals of station 1 and 2 (not
 * amplitude-normalised); window tr is read only after sem_wait(&anok[tr])
 * (anok may be NULL when the rows are ready).  y rows hold L = Lag2-Lag1+1
 * floats.  Return 0 on success, -1 on a CUDA failure (the caller then runs the
 * CPU path, src/FFTapps.c:588,725), -2 from cuda_tspcc2_set_freq for a
 * downsampled frame (Down_smp[s] != 1).  No function resets the device.
 */
#ifndef CCS_CUDA_H
#define CCS_CUDA_H

#include <complex.h>
#include <semaphore.h>

#ifdef __cplusplus
extern "C" {
#endif

int pcc_highlevel(float **y, _Complex float **x1, _Complex float **x2, int N, unsigned int Tr, float v, int Lag1,
                  int Lag2, sem_t *anok);
int pcc1_highlevel(float **y, _Complex float **x1, _Complex float **x2, int N, unsigned int Tr, int Lag1, int Lag2,
                   sem_t *anok);
void pcc1_highlevel2(float **y, float **x1, float **x2, int N, unsigned int Tr, int Lag1, int Lag2);
int cuda_tspcc2_set_freq(float **y0, float **x01, float **x02, unsigned int N, unsigned int Tr, unsigned int Nz,
                         const int Lag1, const int Lag2, unsigned int S, double *scale, _Complex double **wc,
                         unsigned int *Ls, int *center, unsigned int *Down_smp, float C);

#ifdef __cplusplus
}
#endif
#endif
