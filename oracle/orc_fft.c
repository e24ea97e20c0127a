/*
 * Oracle FFT (test infrastructure only).
 *
 * A plain double-precision, unnormalised, mixed-radix Cooley-Tukey transform
 * (decimation in time, smallest prime factor first; generic primes fall back
 * to a direct DFT butterfly). Multi-dimensional transforms apply the 1-D
 * transform along each axis of a row-major array (last index fastest), which
 * is the FFTW layout the reference plans with fftw_plan_dft_2d/3d
 * (src/common/pk_estimation.cpp:66,144, src/common/init.cpp:289,293,359,363).
 *
 * Sign convention follows FFTW: sign = -1 is FFTW_FORWARD (exp(-2 pi i jk/n)),
 * sign = +1 is FFTW_BACKWARD. Neither direction is normalised.
 * It is cross-checked against numpy.fft in the CPU test suite.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

typedef struct { double re, im; } cplx;

static int smallest_factor(int n) {
    if (n % 2 == 0) return 2;
    for (int p = 3; (long)p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* out[k] = sum_j in[j*stride] * W^(j*k*step), W = exp(sign*2*pi*i/N_top), n points. */
static void fft_rec(const cplx *in, cplx *out, int n, long stride, const cplx *tw, int N_top, cplx *scratch) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = smallest_factor(n);
    int m = n / p;
    for (int j1 = 0; j1 < p; ++j1)
        fft_rec(in + j1 * stride, out + (long)j1 * m, m, stride * p, tw, N_top, scratch);
    int step = N_top / n;               /* W_n = W_N^(N/n) */
    cplx *t = scratch;                  /* p entries */
    cplx *r = scratch + p;              /* p entries */
    for (int k2 = 0; k2 < m; ++k2) {
        for (int j1 = 0; j1 < p; ++j1) {
            cplx y = out[(long)j1 * m + k2];
            long e = ((long)j1 * k2 * step) % N_top;
            cplx w = tw[e];
            t[j1].re = y.re * w.re - y.im * w.im;
            t[j1].im = y.re * w.im + y.im * w.re;
        }
        for (int k1 = 0; k1 < p; ++k1) {
            double sr = 0.0, si = 0.0;
            for (int j1 = 0; j1 < p; ++j1) {
                long e = ((long)j1 * k1 * m * step) % N_top;   /* W_p^(j1 k1) */
                cplx w = tw[e];
                sr += t[j1].re * w.re - t[j1].im * w.im;
                si += t[j1].re * w.im + t[j1].im * w.re;
            }
            r[k1].re = sr; r[k1].im = si;
        }
        for (int k1 = 0; k1 < p; ++k1) out[k2 + (long)m * k1] = r[k1];
    }
}

static int max_prime(int n) {
    int best = 1;
    while (n > 1) { int p = smallest_factor(n); if (p > best) best = p; n /= p; }
    return best;
}

/* In-place 1-D transforms of `count` lines: element j of line l sits at
 * data[base(l) + j*stride]. */
void orc_fft_nd(double *data, int ndims, const int *dims, int sign) {
    cplx *a = (cplx *)data;
    long total = 1;
    for (int d = 0; d < ndims; ++d) total *= dims[d];
    for (int axis = 0; axis < ndims; ++axis) {
        int n = dims[axis];
        if (n == 1) continue;
        long stride = 1;
        for (int d = axis + 1; d < ndims; ++d) stride *= dims[d];
        long outer = total / ((long)n * stride);
        cplx *tw = (cplx *)malloc(sizeof(cplx) * n);
        for (int k = 0; k < n; ++k) {
            double ang = sign * 2.0 * M_PI * (double)k / (double)n;
            tw[k].re = cos(ang); tw[k].im = sin(ang);
        }
        int P = max_prime(n);
        long lines = outer * stride;
        #pragma omp parallel
        {
            cplx *lin = (cplx *)malloc(sizeof(cplx) * n);
            cplx *lout = (cplx *)malloc(sizeof(cplx) * n);
            cplx *scr = (cplx *)malloc(sizeof(cplx) * 2 * P);
            #pragma omp for schedule(static)
            for (long l = 0; l < lines; ++l) {
                long o = l / stride, s = l % stride;
                long base = o * (long)n * stride + s;
                for (int j = 0; j < n; ++j) lin[j] = a[base + (long)j * stride];
                fft_rec(lin, lout, n, 1, tw, n, scr);
                for (int j = 0; j < n; ++j) a[base + (long)j * stride] = lout[j];
            }
            free(lin); free(lout); free(scr);
        }
        free(tw);
    }
}
