/*
 * Host generator of the Gaussian random field medium (test infrastructure:
 * makes the 1024^3 input of the large-configuration fixtures).  The same
 * operations, in the same order, as pmmoto_gb300/domain_generation/grf.py on
 * the device -- integer hash noise, then along axes 0, 1, 2 the periodic
 * 65-tap binomial convolution acc = w_0 x[i-32]; acc = acc + w_k x[i+k-32]
 * (k = 1..64), every product and sum rounded once.  Built with
 * -ffp-contract=off, so no multiply-add is fused; the result is bit-identical
 * to the device's.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TAPS 65
#define HALF 32

static uint32_t lowbias32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

void grf_noise(double *out, int64_t n, uint32_t seed)
{
    const uint32_t off = seed * 0x9E3779B9U;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const uint32_t h = lowbias32(lowbias32((uint32_t)i + off));
        out[i] = (double)h * 2.3283064365386963e-10 - 0.5; /* h * 2^-32 - 1/2 */
    }
}

/* One periodic convolution pass along `axis` of the (s0, s1, s2) volume. */
void grf_smooth_axis(const double *in, double *out, int64_t s0, int64_t s1, int64_t s2, int axis, const double *w)
{
    if (axis == 0 || axis == 1) {
        /* planes (axis 0) or rows (axis 1) are contiguous: each output
           element accumulates its taps in order k = 0..64 */
        const int64_t n = axis == 0 ? s0 : s1;
        const int64_t outer = axis == 0 ? 1 : s0;
        const int64_t inner = axis == 0 ? s1 * s2 : s2;
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t o = 0; o < outer; o++)
            for (int64_t i = 0; i < n; i++) {
                double *acc = out + (o * n + i) * inner;
                const double *x0 = in + (o * n + ((i - HALF) % n + n) % n) * inner;
                for (int64_t e = 0; e < inner; e++)
                    acc[e] = w[0] * x0[e];
                for (int k = 1; k < TAPS; k++) {
                    const double *xk = in + (o * n + ((i + k - HALF) % n + n) % n) * inner;
                    const double wk = w[k];
                    for (int64_t e = 0; e < inner; e++)
                        acc[e] = acc[e] + wk * xk[e];
                }
            }
        return;
    }
    /* axis 2: each line copied with a wrapped margin, then the same order */
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * (size_t)(s2 + 2 * HALF));
#pragma omp for schedule(static)
        for (int64_t l = 0; l < s0 * s1; l++) {
            const double *x = in + l * s2;
            for (int64_t j = 0; j < s2 + 2 * HALF; j++)
                buf[j] = x[((j - HALF) % s2 + s2) % s2];
            double *acc = out + l * s2;
            for (int64_t j = 0; j < s2; j++)
                acc[j] = w[0] * buf[j];
            for (int k = 1; k < TAPS; k++) {
                const double wk = w[k];
                for (int64_t j = 0; j < s2; j++)
                    acc[j] = acc[j] + wk * buf[j + k];
            }
        }
        free(buf);
    }
}
