/* PCC at power 1 by direct lag sums on the CPU, in the reference's own
 * precision: single-precision terms |a + b| - |a - b| with sqrtf, summed in
 * double (reference src/FFTapps.c:251-278, pcc1f_lowlevel).  Test
 * infrastructure: the timed CPU baseline of the benchmark and its tests; the
 * product never links it.
 *
 * y[l] = sum over the overlap of (|p2[n + lag] + p1[n]| - |p2[n + lag] - p1[n]|)
 *        / (2 (N - |lag|)),  lag = Lag1 + l,  p1, p2 interleaved complex float rows
 * (the reference calls pcc1f_lowlevel(y, fxa2, fxa1, ...), so its first phase
 * argument is station 2).  Terms are added in float over blocks of 256 so the
 * loop vectorises; each block's sum goes into a double accumulator.  Windows
 * and lags are spread over the host's threads. */
#include <math.h>
#include <stdint.h>

void cpu_pcc1f_set(float *y, const float *p1, const float *p2, int N, int Tr, int Lag1, int Lag2, int64_t ldy) {
    const int L = Lag2 - Lag1 + 1;
    #pragma omp parallel for schedule(dynamic, 8) collapse(2)
    for (int tr = 0; tr < Tr; tr++) {
        for (int l = 0; l < L; l++) {
            const int lag = Lag1 + l;
            if (lag >= N || lag <= -N) { y[(int64_t)tr * ldy + l] = 0.0f; continue; }
            const int n1 = lag < 0 ? -lag : 0;
            const int n2 = lag < 0 ? N : N - lag;
            const float *a = p2 + 2 * ((int64_t)tr * N + n1 + lag);
            const float *b = p1 + 2 * ((int64_t)tr * N + n1);
            const int cnt = n2 - n1;
            double acc = 0.0;
            for (int s = 0; s < cnt; s += 256) {
                const int e = (cnt - s) < 256 ? (cnt - s) : 256;
                float part = 0.0f;
                for (int n = 0; n < e; n++) {
                    const float ax = a[2 * (s + n)], ay = a[2 * (s + n) + 1];
                    const float bx = b[2 * (s + n)], by = b[2 * (s + n) + 1];
                    const float sx = ax + bx, sy = ay + by, dx = ax - bx, dy = ay - by;
                    part += sqrtf(sx * sx + sy * sy) - sqrtf(dx * dx + dy * dy);
                }
                acc += (double)part;
            }
            y[(int64_t)tr * ldy + l] = (float)acc / (float)(2 * cnt);
        }
    }
}
