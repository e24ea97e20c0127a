/*
 * CPU oracle for the standard-lattice hot path of Axion-Strings.
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the checker, never the product.
 *
 * Index conventions are the reference's (src/common/common.hpp:81-119):
 *   2D offset2(i,j) = i + N*j          (i fastest)
 *   3D offset3(i,j,k) = (i*N + j)*N + k (k fastest)
 * Offsets are 64-bit here; the reference uses int.
 * Build with -ffp-contract=off so results do not depend on the host ISA.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"
#include "orc_philox.h"

#define STD_MIN(a, b) (((b) < (a)) ? (b) : (a))   /* std::min(a,b) */

static inline long wrap(long i, long N) { return ((i % N) + N) % N; }

static long lattice_length(const orc_params *p) {
    long N = p->N;
    return (p->NDIMS == 3) ? N * N * N : N * N;
}

double orc_normal_draw(uint64_t seed, int a, int64_t m) { return orc_normal(seed, a, m); }

/* Stencil coefficient table of build_coefficient_matrix (s_integrate.cpp:9-14):
 * float expressions stored as data_t. Returns the number of coefficients. */
static int stencil_coefficients(int setting, int ndims, double c[5]) {
    switch (setting) {
    case 0: c[0] = (double)(-2.0f * ndims); c[1] = 1.0f; return 2;
    case 1: c[0] = (double)(-5.0f / 2.0f * ndims); c[1] = (double)(4.0f / 3.0f); c[2] = (double)(-1.0f / 12.0f); return 3;
    case 2: c[0] = (double)(-49.0f / 18.0f * ndims); c[1] = (double)(3.0f / 2.0f); c[2] = (double)(-3.0f / 20.0f);
            c[3] = (double)(1.0f / 90.0f); return 4;
    default: c[0] = (double)(-205.0f / 72.0f * ndims); c[1] = (double)(8.0f / 5.0f); c[2] = (double)(-1.0f / 5.0f);
            c[3] = (double)(8.0f / 315.0f); c[4] = (double)(-1.0f / 560.0f); return 5;
    }
}

/* Row m of A*phi, summed in the COO insertion order of s_integrate.cpp:38-76
 * (2D) / :93-143 (3D): centre, then for each l the +l/-l neighbours along each
 * axis in the order the reference appends them. */
static double stencil_row(const double *phi, long m, int ndims, long N, const double *c, int nc) {
    double acc = c[0] * phi[m];
    if (ndims == 2) {
        long i = m % N, j = m / N;
        for (int l = 1; l < nc; ++l) {
            acc += c[l] * phi[wrap(i + l, N) + N * j];
            acc += c[l] * phi[wrap(i - l, N) + N * j];
            acc += c[l] * phi[i + N * wrap(j + l, N)];
            acc += c[l] * phi[i + N * wrap(j - l, N)];
        }
    } else {
        long i = m / (N * N), j = (m / N) % N, k = m % N;
        for (int l = 1; l < nc; ++l) {
            acc += c[l] * phi[(wrap(i + l, N) * N + j) * N + k];
            acc += c[l] * phi[(wrap(i - l, N) * N + j) * N + k];
            acc += c[l] * phi[(i * N + wrap(j + l, N)) * N + k];
            acc += c[l] * phi[(i * N + wrap(j - l, N)) * N + k];
            acc += c[l] * phi[(i * N + j) * N + wrap(k + l, N)];
            acc += c[l] * phi[(i * N + j) * N + wrap(k - l, N)];
        }
    }
    return acc;
}

void orc_laplacian_spectral(const orc_params *p, const double *field, double *ret) {
    int N = p->N, nd = p->NDIMS;
    long len = lattice_length(p);
    float L = N * p->space_step;                                   /* s_integrate.cpp:183 */
    double *k = (double *)malloc(sizeof(double) * N);
    double *data = (double *)malloc(sizeof(double) * 2 * len);
    for (int i = 0; i < N; ++i) k[i] = (-N / 2.0f + i) * 2.0f * M_PI / L;   /* :193 / :241 */
    for (long m = 0; m < len; ++m) {                               /* :205-208, shift :210 */
        long s = nd == 2 ? (m % N) + (m / N) : (m / ((long)N * N)) + ((m / N) % N) + (m % N);
        double sg = (s & 1) ? -1.0 : 1.0;
        data[2 * m] = field[m] * sg;
        data[2 * m + 1] = 0.0 * sg;
    }
    int dims[3] = {N, N, N};
    orc_fft_nd(data, nd, dims, -1);                                /* FFTW_FORWARD */
    for (long m = 0; m < len; ++m) {                               /* :214-220 / :262-268 */
        double ksq;
        if (nd == 2) {
            long i = m % N, j = m / N;                             /* coordinate2 */
            ksq = k[i] * k[i] + k[j] * k[j];
        } else {
            long i = m / ((long)N * N), j = (m / N) % N, kk = m % N;   /* coordinate3 */
            ksq = k[i] * k[i] + k[j] * k[j] + k[kk] * k[kk];
        }
        data[2 * m] *= -ksq;
        data[2 * m + 1] *= -ksq;
    }
    orc_fft_nd(data, nd, dims, +1);                                /* FFTW_BACKWARD */
    for (long m = 0; m < len; ++m) {                               /* shift :226, / length :228-231 */
        long s = nd == 2 ? (m % N) + (m / N) : (m / ((long)N * N)) + ((m / N) % N) + (m % N);
        double v = (s & 1) ? -data[2 * m] : data[2 * m];
        ret[m] = v / len;
    }
    free(data);
    free(k);
}

void orc_laplacian(const orc_params *p, const double *phi, double *out) {
    if (p->laplacian == 1) {
        orc_laplacian_spectral(p, phi, out);
        return;
    }
    double c[5];
    int nc = stencil_coefficients(p->stencil_setting, p->NDIMS, c);
    long len = lattice_length(p), N = p->N;
    double dx = (double)p->space_step;
    double alpha = 1.0f / (dx * dx);          /* 1.0f / pow_2(dx), s_integrate.cpp:322 */
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) out[m] = alpha * stencil_row(phi, m, p->NDIMS, N, c, nc);
}

/* Potential coefficient -(lambda / tau^(2 prs)) written in the operand order of
 * s_integrate.cpp:333 (-1.0f / pow_2(tau) * lambda). */
static double potential_coefficient(const orc_params *p, double tau) {
    double inv = p->prs ? (-1.0f / (tau * tau)) : -1.0;
    return inv * (double)p->lambda;
}

void orc_vvsl_step(const orc_params *p, double *phi1, double *phi2, double *pi1, double *pi2,
                   double *ker1, double *ker2, double *ker1n, double *ker2n, double *tau) {
    long len = lattice_length(p);
    float dt = p->time_step;
    double ddt = dt;
    /* drift, s_integrate.cpp:311-315 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        phi1[i] += ddt * (pi1[i] + 0.5f * ker1[i] * ddt);
        phi2[i] += ddt * (pi2[i] + 0.5f * ker2[i] * ddt);
    }
    *tau = *tau + ddt;                                    /* s_integrate.cpp:317 */
    orc_laplacian(p, phi1, ker1n);                        /* s_integrate.cpp:322 */
    orc_laplacian(p, phi2, ker2n);                        /* s_integrate.cpp:324 */
    double t = *tau;
    double coef = potential_coefficient(p, t);
    double T0 = p->T_initial;
    double shift = (T0 * T0) / (3.0f);
    /* potential, s_integrate.cpp:331-335 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        double a = phi1[i], b = phi2[i];
        double br = a * a + b * b - t * t + shift;
        ker1n[i] += coef * a * br;
        ker2n[i] += coef * b * br;
    }
    /* kick, s_integrate.cpp:337-341 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        pi1[i] += 0.5f * (ker1[i] + ker1n[i]) * ddt;
        pi2[i] += 0.5f * (ker2[i] + ker2n[i]) * ddt;
    }
    /* rotate kernels, s_integrate.cpp:343-347 */
    memcpy(ker1, ker1n, sizeof(double) * len);
    memcpy(ker2, ker2n, sizeof(double) * len);
}

void orc_vvsl_hamiltonian_step(const orc_params *p, double *phi1, double *phi2, double *pi1, double *pi2,
                               double *ker1, double *ker2, double *ker1n, double *ker2n, double *tau) {
    long len = lattice_length(p);
    float dt = p->time_step;
    double ddt = dt;
    *tau = *tau + ddt;                                    /* s_integrate.cpp:364 */
    double t = *tau, tsq = t * t;
    /* drift with the advanced tau, s_integrate.cpp:366-370 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        phi1[i] += ddt / tsq * (pi1[i] + 0.5f * ddt * ker1[i]);
        phi2[i] += ddt / tsq * (pi2[i] + 0.5f * ddt * ker2[i]);
    }
    /* (tau^2/dx^2) A phi, s_integrate.cpp:374-376; with the spectral
       Laplacian (no counterpart in the reference's Hamiltonian form) tau^2 L phi */
    if (p->laplacian == 1) {
        orc_laplacian_spectral(p, phi1, ker1n);
        orc_laplacian_spectral(p, phi2, ker2n);
        for (long m = 0; m < len; ++m) {
            ker1n[m] *= tsq;
            ker2n[m] *= tsq;
        }
    } else {
        double c[5];
        int nc = stencil_coefficients(p->stencil_setting, p->NDIMS, c);
        double dx = (double)p->space_step;
        double alpha = tsq / (dx * dx);
        long N = p->N;
        #pragma omp parallel for schedule(static)
        for (long m = 0; m < len; ++m) {
            ker1n[m] = alpha * stencil_row(phi1, m, p->NDIMS, N, c, nc);
            ker2n[m] = alpha * stencil_row(phi2, m, p->NDIMS, N, c, nc);
        }
    }
    double T0 = p->T_initial;
    double shift = (T0 * T0) / (3.0f * tsq);
    double lam = (double)p->lambda;
    /* potential, s_integrate.cpp:378-382 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        double a = phi1[i], b = phi2[i];
        double br = a * a + b * b - 1.0f + shift;
        ker1n[i] += -tsq * lam * a * br;
        ker2n[i] += -tsq * lam * b * br;
    }
    /* kick, s_integrate.cpp:384-388 */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        pi1[i] += 0.5f * (ker1[i] + ker1n[i]) * ddt;
        pi2[i] += 0.5f * (ker2[i] + ker2n[i]) * ddt;
    }
    /* rotate kernels, s_integrate.cpp:390-394 */
    memcpy(ker1, ker1n, sizeof(double) * len);
    memcpy(ker2, ker2n, sizeof(double) * len);
}

/* Float build of the same step (data_t = float, tau float). The SpMV runs in
 * float like mkl_sparse_s_mv; the potential term is evaluated in double as the
 * reference's pow_2(double) promotes it, then rounded into the float kernel. */
void orc_vvsl_step_f32(const orc_params *p, float *phi1, float *phi2, float *pi1, float *pi2,
                       float *ker1, float *ker2, float *ker1n, float *ker2n, float *tau) {
    long len = lattice_length(p), N = p->N;
    float dt = p->time_step;
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        phi1[i] += dt * (pi1[i] + 0.5f * ker1[i] * dt);
        phi2[i] += dt * (pi2[i] + 0.5f * ker2[i] * dt);
    }
    *tau = *tau + dt;
    double cd[5];
    int nc = stencil_coefficients(p->stencil_setting, p->NDIMS, cd);
    float c[5];
    for (int l = 0; l < nc; ++l) c[l] = (float)cd[l];
    double dx = (double)p->space_step;
    float alpha = (float)(1.0f / (dx * dx));
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) {
        float a1 = c[0] * phi1[m], a2 = c[0] * phi2[m];
        if (p->NDIMS == 2) {
            long i = m % N, j = m / N;
            for (int l = 1; l < nc; ++l) {
                long o[4] = { wrap(i + l, N) + N * j, wrap(i - l, N) + N * j, i + N * wrap(j + l, N), i + N * wrap(j - l, N) };
                for (int q = 0; q < 4; ++q) { a1 += c[l] * phi1[o[q]]; a2 += c[l] * phi2[o[q]]; }
            }
        } else {
            long i = m / (N * N), j = (m / N) % N, k = m % N;
            for (int l = 1; l < nc; ++l) {
                long o[6] = { (wrap(i + l, N) * N + j) * N + k, (wrap(i - l, N) * N + j) * N + k,
                              (i * N + wrap(j + l, N)) * N + k, (i * N + wrap(j - l, N)) * N + k,
                              (i * N + j) * N + wrap(k + l, N), (i * N + j) * N + wrap(k - l, N) };
                for (int q = 0; q < 6; ++q) { a1 += c[l] * phi1[o[q]]; a2 += c[l] * phi2[o[q]]; }
            }
        }
        ker1n[m] = alpha * a1;
        ker2n[m] = alpha * a2;
    }
    double t = *tau;
    double coef = potential_coefficient(p, t);
    double T0 = p->T_initial;
    double shift = (T0 * T0) / (3.0f);
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        double a = phi1[i], b = phi2[i];
        double br = a * a + b * b - t * t + shift;
        ker1n[i] = (float)((double)ker1n[i] + coef * a * br);
        ker2n[i] = (float)((double)ker2n[i] + coef * b * br);
    }
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        pi1[i] += 0.5f * (ker1[i] + ker1n[i]) * dt;
        pi2[i] += 0.5f * (ker2[i] + ker2n[i]) * dt;
    }
    memcpy(ker1, ker1n, sizeof(float) * len);
    memcpy(ker2, ker2n, sizeof(float) * len);
}

/* ------------------------------------------------ timing port of the CPU path */

struct orc_csr {
    long rows;
    int per_row;      /* 1 + 2 * NDIMS * radius entries in every row */
    int *col;         /* MKL_INT column indices, rows * per_row */
    float *val;
};

/* The periodic matrix of build_coefficient_matrix (s_integrate.cpp:5-149) with
 * every entry of a row stored, which is how mkl_sparse_?_mv applies the
 * reference's symmetric/upper handle: row m lists the centre and then, for
 * each l, the +l/-l neighbours along each axis (stencil_row's order). */
orc_csr *orc_csr_build(const orc_params *p) {
    double cd[5];
    int nc = stencil_coefficients(p->stencil_setting, p->NDIMS, cd);
    long N = p->N, len = lattice_length(p);
    orc_csr *A = (orc_csr *)malloc(sizeof(orc_csr));
    if (!A) return NULL;
    A->rows = len;
    A->per_row = 1 + 2 * p->NDIMS * (nc - 1);
    A->col = (int *)malloc(sizeof(int) * (size_t)len * A->per_row);
    A->val = (float *)malloc(sizeof(float) * (size_t)len * A->per_row);
    if (!A->col || !A->val) {
        orc_csr_free(A);
        return NULL;
    }
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) {
        int *c = A->col + m * A->per_row;
        float *v = A->val + m * A->per_row;
        int q = 0;
        c[q] = (int)m; v[q++] = (float)cd[0];
        for (int l = 1; l < nc; ++l) {
            long o[6];
            int no;
            if (p->NDIMS == 2) {
                long i = m % N, j = m / N;
                o[0] = wrap(i + l, N) + N * j; o[1] = wrap(i - l, N) + N * j;
                o[2] = i + N * wrap(j + l, N); o[3] = i + N * wrap(j - l, N);
                no = 4;
            } else {
                long i = m / (N * N), j = (m / N) % N, k = m % N;
                o[0] = (wrap(i + l, N) * N + j) * N + k; o[1] = (wrap(i - l, N) * N + j) * N + k;
                o[2] = (i * N + wrap(j + l, N)) * N + k; o[3] = (i * N + wrap(j - l, N)) * N + k;
                o[4] = (i * N + j) * N + wrap(k + l, N); o[5] = (i * N + j) * N + wrap(k - l, N);
                no = 6;
            }
            for (int e = 0; e < no; ++e) { c[q] = (int)o[e]; v[q++] = (float)cd[l]; }
        }
    }
    return A;
}

void orc_csr_free(orc_csr *A) {
    if (!A) return;
    free(A->col);
    free(A->val);
    free(A);
}

/* y = alpha * A x (mkl_wrapper_sparse_mv, mkl_wrapper.cpp:11-17, beta = 0). */
static void csr_mv_f32(const orc_csr *A, float alpha, const float *x, float *y) {
    int w = A->per_row;
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < A->rows; ++m) {
        const int *c = A->col + m * w;
        const float *v = A->val + m * w;
        float acc = 0.0f;
        for (int q = 0; q < w; ++q) acc += v[q] * x[c[q]];
        y[m] = alpha * acc;
    }
}

/* vvsl_field_rescaled (s_integrate.cpp:305-348) as the reference runs it:
 * six passes over the lattice with the Laplacian as two sparse
 * matrix-vector products (s_integrate.cpp:321-324), float data. Used to time
 * the CPU path: it has the reference's passes and memory traffic (the
 * matrix's indices and values streamed per step), where orc_vvsl_step_f32
 * recomputes neighbour offsets with integer divisions. Arithmetic equals
 * orc_vvsl_step_f32 but for the summation order within a row. */
void orc_ref_step_f32(const orc_params *p, const orc_csr *A, float *phi1, float *phi2, float *pi1, float *pi2,
                      float *ker1, float *ker2, float *ker1n, float *ker2n, float *tau) {
    long len = lattice_length(p);
    float dt = p->time_step;
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        phi1[i] += dt * (pi1[i] + 0.5f * ker1[i] * dt);
        phi2[i] += dt * (pi2[i] + 0.5f * ker2[i] * dt);
    }
    *tau = *tau + dt;
    double dx = (double)p->space_step;
    float alpha = (float)(1.0f / (dx * dx));
    csr_mv_f32(A, alpha, phi1, ker1n);
    csr_mv_f32(A, alpha, phi2, ker2n);
    double t = *tau;
    double coef = potential_coefficient(p, t);
    double T0 = p->T_initial;
    double shift = (T0 * T0) / (3.0f);
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        double a = phi1[i], b = phi2[i];
        double br = a * a + b * b - t * t + shift;
        ker1n[i] = (float)((double)ker1n[i] + coef * a * br);
        ker2n[i] = (float)((double)ker2n[i] + coef * b * br);
    }
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        pi1[i] += 0.5f * (ker1[i] + ker1n[i]) * dt;
        pi2[i] += 0.5f * (ker2[i] + ker2n[i]) * dt;
    }
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < len; ++i) {
        ker1[i] = ker1n[i];
        ker2[i] = ker2n[i];
    }
}

/* ---------------------------------------------------------------- strings */

/* min(|d|, 1-|d|) of string_finding.cpp:22-24 */
static inline double circ(double a, double b) {
    double d = fabs(b - a);
    return STD_MIN(d, 1 - d);
}

int64_t orc_cores(const orc_params *p, const double *f, uint8_t *mask) {
    long N = p->N, len = lattice_length(p);
    int thr = p->thr;
    double accept = (double)(0.5f * (1.0f - thr / 100.0f));   /* string_finding.cpp:8,40 */
    int64_t n = 0;
    if (p->NDIMS == 2) {
        #pragma omp parallel for schedule(static) reduction(+:n)
        for (long m = 0; m < len; ++m) {
            long i = m % N, j = m / N;
            double n1 = (f[i + N * j] + M_PI) / (2 * M_PI);
            double n2 = (f[wrap(i + 1, N) + N * j] + M_PI) / (2 * M_PI);
            double n3 = (f[wrap(i + 1, N) + N * wrap(j + 1, N)] + M_PI) / (2 * M_PI);
            double n4 = (f[i + N * wrap(j + 1, N)] + M_PI) / (2 * M_PI);
            double s = circ(n1, n2) + circ(n2, n3) + circ(n3, n4);
            uint8_t flag = s > accept;
            if (mask) mask[m] = flag;
            n += flag;
        }
    } else {
        #pragma omp parallel for schedule(static) reduction(+:n)
        for (long m = 0; m < len; ++m) {
            long i = m / (N * N), j = (m / N) % N, k = m % N;
            long ip = wrap(i + 1, N), jp = wrap(j + 1, N), kp = wrap(k + 1, N);
#define O3(a, b, c) (((a) * N + (b)) * N + (c))
            double c000 = (f[O3(i, j, k)] + M_PI) / (2.0f * M_PI);
            double c100 = (f[O3(ip, j, k)] + M_PI) / (2.0f * M_PI);
            double c110 = (f[O3(ip, jp, k)] + M_PI) / (2.0f * M_PI);
            double c010 = (f[O3(i, jp, k)] + M_PI) / (2.0f * M_PI);
            double c011 = (f[O3(i, jp, kp)] + M_PI) / (2.0f * M_PI);
            double c001 = (f[O3(i, j, kp)] + M_PI) / (2.0f * M_PI);
#undef O3
            /* plaquette a: (i,j,k)->(i+1,j,k)->(i+1,j+1,k)->(i,j+1,k)    :49-52
             * plaquette b: (i,j,k)->(i+1,j,k)->(i,j+1,k+1)->(i,j,k+1)    :54-57 (sic)
             * plaquette c: (i,j,k)->(i,j+1,k)->(i,j+1,k+1)->(i,j,k+1)    :59-62 */
            double sa = circ(c000, c100) + circ(c100, c110) + circ(c110, c010);
            double sb = circ(c000, c100) + circ(c100, c011) + circ(c011, c001);
            double sc = circ(c000, c010) + circ(c010, c011) + circ(c011, c001);
            uint8_t flag = (sa > accept || sb > accept || sc > accept);
            if (mask) mask[m] = flag;
            n += flag;
        }
    }
    return n;
}

int64_t orc_num_cores2(int N, const uint8_t *mask) {
    long len = (long)N * N;
    int64_t n = 0, pairs = 0;
    long prev = -1;
    for (long m = 0; m < len; ++m) {
        if (!mask[m]) continue;
        ++n;
        if (prev >= 0) {
            long dx = (m % N) - (prev % N), dy = (m / N) - (prev / N);
            if (dy == 0 && dx == 1) ++pairs;
            if (dy == 1 && dx == 0) ++pairs;
        }
        prev = m;
    }
    return n - pairs;
}

float orc_xi(const orc_params *p, int64_t n_plaquettes, int64_t num_cores, double tau) {
    float t_phys = (float)(0.5f * (tau * tau));        /* physics.cpp:43-45 */
    float a = (float)tau;                              /* physics.cpp:47-50 */
    float side = p->N * p->space_step * a;
    if (p->NDIMS == 2) {
        float area = (float)((double)side * (double)side);
        return (float)((int)num_cores * ((double)t_phys * (double)t_phys) / area);
    }
    float total_length = (int)n_plaquettes * 2.0f / 3.0f;
    float physical_length = total_length * a;
    float volume = (float)((double)side * (double)side * (double)side);
    return (float)(physical_length * ((double)t_phys * (double)t_phys) / volume);
}

/* ---------------------------------------------------------------- spectra */

static void checkerboard(double *c, const orc_params *p) {
    long N = p->N, len = lattice_length(p);
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) {
        long s = (p->NDIMS == 2) ? (m % N) + (m / N) : (m / (N * N)) + ((m / N) % N) + (m % N);
        if (s & 1) { c[2 * m] = -c[2 * m]; c[2 * m + 1] = -c[2 * m + 1]; }
    }
}

void orc_powerspec(const orc_params *p, const double *re, const double *im,
                   double *pk, double *ks, int *count) {
    long N = p->N, len = lattice_length(p);
    int nb = (int)(N / 2);
    float L = N * p->space_step;
    double *c = (double *)malloc(sizeof(double) * 2 * len);
    for (long m = 0; m < len; ++m) { c[2 * m] = re[m]; c[2 * m + 1] = im ? im[m] : 0.0; }
    checkerboard(c, p);                                  /* pk_estimation.cpp:74,152 */
    int dims[3] = { (int)N, (int)N, (int)N };
    orc_fft_nd(c, p->NDIMS, dims, -1);                   /* FFTW_FORWARD */
    double *kv = (double *)malloc(sizeof(double) * N);
    for (long i = 0; i < N; ++i) kv[i] = (double)(-N / 2.0f + i);   /* :59,137 */
    for (int b = 0; b < nb; ++b) { pk[b] = 0; ks[b] = 0; count[b] = 0; }
    for (long m = 0; m < len; ++m) {                    /* :88-101, :166-179 */
        double kmag;
        if (p->NDIMS == 2) {
            long i = m % N, j = m / N;
            kmag = sqrt(kv[i] * kv[i] + kv[j] * kv[j]);
        } else {
            long i = m / (N * N), j = (m / N) % N, k = m % N;
            kmag = sqrt(kv[i] * kv[i] + kv[j] * kv[j] + kv[k] * kv[k]);
        }
        if (kmag == 0.0f || kmag >= N / 2) continue;
        int idx = (int)floor(kmag) - 1;
        pk[idx] += c[2 * m] * c[2 * m] + c[2 * m + 1] * c[2 * m + 1];
        ks[idx] += kmag;
        count[idx]++;
    }
    for (int b = 0; b < nb; ++b) {                       /* :117-121, :195-199 */
        ks[b] /= count[b];
        if (p->NDIMS == 2) pk[b] /= 2.0f * M_PI * ks[b];
        else pk[b] /= 4.0f * M_PI * (ks[b] * ks[b]);
        ks[b] *= 2.0f * M_PI / L;
    }
    free(kv);
    free(c);
}

/* k-grid of init.cpp:280-282 / :350-352 */
static void init_kgrid(const orc_params *p, double *kv) {
    long N = p->N;
    float L = p->space_step * N;
    for (long i = 0; i < N; ++i) kv[i] = (double)((-N / 2.0f + i) * 2.0f) * M_PI / L;
}

static double kgrid_mag(const orc_params *p, const double *kv, long m) {
    long N = p->N;
    if (p->NDIMS == 2) { long i = m % N, j = m / N; return sqrt(kv[i] * kv[i] + kv[j] * kv[j]); }
    long i = m / (N * N), j = (m / N) % N, l = m % N;
    return sqrt(kv[i] * kv[i] + kv[j] * kv[j] + kv[l] * kv[l]);
}

void orc_gaussian_thermal(const orc_params *p, uint64_t seed,
                          double *phi1, double *phi2, double *phidot1, double *phidot2) {
    long N = p->N, len = lattice_length(p);
    float T0 = p->T_initial;
    float meff2 = (float)(p->lambda * ((double)T0 * (double)T0 / 3.0f - 1.0f));   /* physics.cpp:30 */
    double *kv = (double *)malloc(sizeof(double) * N);
    init_kgrid(p, kv);
    double *a = (double *)malloc(sizeof(double) * 2 * len);
    double *b = (double *)malloc(sizeof(double) * 2 * len);
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) {                     /* init.cpp:295-315 / :365-385 */
        double k = kgrid_mag(p, kv, m);
        double amp = 0.0, amp_dot = 0.0;
        if (k != 0.0f) {
            double omegak = sqrt(k * k + (double)meff2);
            double bose = 1.0f / (exp(omegak / T0) - 1.0f);
            amp = sqrt(bose / omegak);
            amp_dot = sqrt(bose * omegak);
        }
        a[2 * m] = amp * orc_normal(seed, 0, m);
        a[2 * m + 1] = amp * orc_normal(seed, 1, m);
        b[2 * m] = amp_dot * orc_normal(seed, 2, m);
        b[2 * m + 1] = amp_dot * orc_normal(seed, 3, m);
    }
    int dims[3] = { (int)N, (int)N, (int)N };
    orc_fft_nd(a, p->NDIMS, dims, +1);                   /* FFTW_BACKWARD */
    orc_fft_nd(b, p->NDIMS, dims, +1);
    checkerboard(a, p);
    checkerboard(b, p);
    double norm = (p->NDIMS == 2) ? (double)N * (double)N : (double)N * (double)N * (double)N;
    for (long m = 0; m < len; ++m) {                     /* init.cpp:323-330 / :393-400 */
        phi1[m] = a[2 * m] / norm;
        phi2[m] = a[2 * m + 1] / norm;
        phidot1[m] = b[2 * m] / norm;
        phidot2[m] = b[2 * m + 1] / norm;
    }
    free(a); free(b); free(kv);
}

void orc_init_flat(const orc_params *p, uint64_t seed, double kcut,
                   double *phi1, double *phi2, double *phidot1, double *phidot2) {
    long N = p->N, len = lattice_length(p);
    double *kv = (double *)malloc(sizeof(double) * N);
    init_kgrid(p, kv);
    double *a = (double *)malloc(sizeof(double) * 2 * len);
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < len; ++m) {
        double k = kgrid_mag(p, kv, m);
        double amp = (k != 0.0 && k < kcut) ? 1.0 : 0.0;
        a[2 * m] = amp * orc_normal(seed, 0, m);
        a[2 * m + 1] = amp * orc_normal(seed, 1, m);
    }
    int dims[3] = { (int)N, (int)N, (int)N };
    orc_fft_nd(a, p->NDIMS, dims, +1);
    checkerboard(a, p);
    double norm = (p->NDIMS == 2) ? (double)N * (double)N : (double)N * (double)N * (double)N;
    double s = 0.0;
    for (long m = 0; m < len; ++m) {
        phi1[m] = a[2 * m] / norm;
        phi2[m] = a[2 * m + 1] / norm;
        s += phi1[m] * phi1[m] + phi2[m] * phi2[m];
    }
    double mean = s / (double)len;
    double scale = (mean > 0.0) ? 1.0 / sqrt(mean) : 0.0;
    for (long m = 0; m < len; ++m) {
        phi1[m] *= scale; phi2[m] *= scale;
        phidot1[m] = 0.0; phidot2[m] = 0.0;
    }
    free(a); free(kv);
}

/* ---------------------------------------------------------------- reductions */

void orc_background(const orc_params *p, const double *phi1, const double *phi2,
                    const double *phidot1, const double *phidot2, double out[6]) {
    long len = lattice_length(p);
    double s[6] = { 0, 0, 0, 0, 0, 0 };
    for (long i = 0; i < len; ++i) {                     /* s_run.cpp:140-147 */
        s[0] += phi1[i];
        s[1] += phi2[i];
        s[2] += phidot1[i];
        s[3] += phidot2[i];
        s[4] += fabs(atan2(phi1[i], phi2[i]));
        s[5] += sqrt(phi1[i] * phi1[i] + phi2[i] * phi2[i]);
    }
    for (int q = 0; q < 6; ++q) out[q] = s[q] / len;
}

void orc_energies(const orc_params *p, const double *psi1, const double *psi2,
                  const double *pi1, const double *pi2, double tau, double out[3]) {
    long N = p->N, len = lattice_length(p);
    double dx = p->space_step;
    double lam = (double)p->lambda * (p->prs ? 1.0 : tau * tau);
    double it = 1.0 / tau;
    double ek = 0, eg = 0, ev = 0;
    for (long m = 0; m < len; ++m) {
        double f1 = psi1[m] * it, f2 = psi2[m] * it;
        double d1 = (pi1[m] - f1) * it, d2 = (pi2[m] - f2) * it;
        ek += 0.5 * (d1 * d1 + d2 * d2);
        double g = 0.0;
        long nb[3];
        int nn;
        if (p->NDIMS == 2) {
            long i = m % N, j = m / N;
            nb[0] = wrap(i + 1, N) + N * j; nb[1] = i + N * wrap(j + 1, N); nn = 2;
        } else {
            long i = m / (N * N), j = (m / N) % N, k = m % N;
            nb[0] = (wrap(i + 1, N) * N + j) * N + k; nb[1] = (i * N + wrap(j + 1, N)) * N + k;
            nb[2] = (i * N + j) * N + wrap(k + 1, N); nn = 3;
        }
        for (int q = 0; q < nn; ++q) {
            double g1 = (psi1[nb[q]] * it - f1) / dx, g2 = (psi2[nb[q]] * it - f2) / dx;
            g += g1 * g1 + g2 * g2;
        }
        eg += 0.5 * g;
        double r = f1 * f1 + f2 * f2 - 1.0;
        ev += 0.25 * lam * r * r;
    }
    out[0] = ek / len; out[1] = eg / len; out[2] = ev / len;
}

void orc_axion_spectrum(const orc_params *p, const double *psi1, const double *psi2,
                        const double *pi1, const double *pi2, double tau, int nbins,
                        double *kmean, double *pk, int64_t *count) {
    long N = p->N, len = lattice_length(p);
    int d = p->NDIMS;
    double dx = p->space_step;
    double L = (double)N * dx;
    double *c = (double *)malloc(sizeof(double) * 2 * len);
    for (long m = 0; m < len; ++m) {
        double r = sqrt(psi1[m] * psi1[m] + psi2[m] * psi2[m]);
        c[2 * m] = (r > 0.0) ? (psi2[m] * pi1[m] - psi1[m] * pi2[m]) / (tau * r) : 0.0;
        c[2 * m + 1] = 0.0;
    }
    int dims[3] = { (int)N, (int)N, (int)N };
    orc_fft_nd(c, d, dims, -1);
    /* bin edges in units of |n|: t_b = (kmax/kmin)^(b/nbins), b = 1..nbins-1 */
    double ratio = sqrt((double)d) * (double)N / 2.0;
    double *edge2 = (double *)malloc(sizeof(double) * (nbins > 1 ? nbins : 1));
    for (int b = 1; b < nbins; ++b) { double t = exp(log(ratio) * (double)b / (double)nbins); edge2[b] = t * t; }
    double *ksum = (double *)calloc(nbins, sizeof(double));
    double *psum = (double *)calloc(nbins, sizeof(double));
    for (int b = 0; b < nbins; ++b) count[b] = 0;
    for (long m = 0; m < len; ++m) {
        long q[3];
        if (d == 2) { q[0] = m % N; q[1] = m / N; }
        else { q[0] = m / (N * N); q[1] = (m / N) % N; q[2] = m % N; }
        long n2 = 0;
        for (int a = 0; a < d; ++a) { long f = (q[a] < N / 2) ? q[a] : q[a] - N; n2 += f * f; }
        if (n2 == 0) continue;
        int b = 0;
        while (b + 1 < nbins && (double)n2 >= edge2[b + 1]) ++b;
        psum[b] += c[2 * m] * c[2 * m] + c[2 * m + 1] * c[2 * m + 1];
        ksum[b] += 2.0 * M_PI * sqrt((double)n2) / L;
        count[b]++;
    }
    double norm = pow(L, d) / pow((double)len, 2.0);
    for (int b = 0; b < nbins; ++b) {
        if (count[b]) { kmean[b] = ksum[b] / count[b]; pk[b] = norm * psum[b] / count[b]; }
        else { kmean[b] = 0.0; pk[b] = 0.0; }
    }
    free(ksum); free(psum); free(edge2); free(c);
}

/* Exported Philox block for known-answer tests. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox4x32_10(ctr, key, out); }
