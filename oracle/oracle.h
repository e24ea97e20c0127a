/*
 * CPU oracle for the standard-lattice hot path of Axion-Strings.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * algorithms, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg as the checker. Nothing in the product path links, loads or
 * calls it.
 *
 * Each function cites the reference file:line it restates. Where the reference
 * calls a third-party library (Intel MKL sparse BLAS and VSL, FFTW3), the
 * restatement follows the library's documented semantics:
 *   - MKL symmetric/upper COO SpMV  -> direct periodic stencil sum (same matrix)
 *   - MKL VSL SFMT19937 + ICDF      -> orc_normal() (Philox + Box-Muller), see
 *                                      orc_philox.h; the MKL bitstream is not
 *                                      reproducible here (parity unpinned for
 *                                      the random numbers themselves)
 *   - FFTW c2c plans                -> orc_fft_nd() (orc_fft.c)
 */
#ifndef AXS_ORACLE_H
#define AXS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Subset of the reference `struct parameters` (src/common/common.hpp:30-69)
 * that the hot path reads, plus `prs`, which selects the potential coefficient
 * lambda / tau^(2*prs) of the AMR integrator (src/amr/amr_integrate.cpp:112-113).
 * prs = 1 is exactly the standard integrator (src/standard/s_integrate.cpp:333). */
typedef struct orc_params {
    int   NDIMS;
    int   N;
    float lambda;
    float T_initial;
    float space_step;
    float time_step;
    int   stencil_setting;
    int   thr;
    int   prs;
    int   laplacian;   /* 0: finite-difference stencil; 1: compute_laplacian_fft (s_integrate.cpp:179-296) */
} orc_params;

/* Unnormalised in-place complex FFT of a row-major array (interleaved re/im);
 * sign -1 = FFTW_FORWARD, +1 = FFTW_BACKWARD. */
void orc_fft_nd(double *data, int ndims, const int *dims, int sign);

double orc_normal_draw(uint64_t seed, int a, int64_t m);
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* (1/dx^2) * A * phi, A the periodic finite-difference matrix of
 * build_coefficient_matrix (src/standard/s_integrate.cpp:5-149) applied as in
 * vvsl_field_rescaled (s_integrate.cpp:322); with p->laplacian = 1 the
 * spectral Laplacian below instead (the reference's `#else` branch, :327-329). */
void orc_laplacian(const orc_params *p, const double *phi, double *out);
/* compute_laplacian_fft (s_integrate.cpp:179-296): checkerboard shift, forward
 * FFT, times -k^2 with k = (-N/2 + i) 2 pi / L evaluated as there, backward
 * FFT, shift, / N^NDIMS. */
void orc_laplacian_spectral(const orc_params *p, const double *field, double *ret);

/* One velocity-Verlet step, vvsl_field_rescaled (s_integrate.cpp:305-348). */
void orc_vvsl_step(const orc_params *p, double *phi1, double *phi2, double *pi1, double *pi2,
                   double *ker1, double *ker2, double *ker1n, double *ker2n, double *tau);
/* One step of vvsl_hamiltonian_form (s_integrate.cpp:358-395): phi and
 * pi = tau^2 phi', tau advanced before the drift. */
void orc_vvsl_hamiltonian_step(const orc_params *p, double *phi1, double *phi2, double *pi1, double *pi2,
                               double *ker1, double *ker2, double *ker1n, double *ker2n, double *tau);
/* The same step with float fields and float tau, as the reference compiles
 * without USE_DOUBLE_PRECISION (src/common/common.hpp:19-23). */
void orc_vvsl_step_f32(const orc_params *p, float *phi1, float *phi2, float *pi1, float *pi2,
                       float *ker1, float *ker2, float *ker1n, float *ker2n, float *tau);

/* Timing port of the CPU path (bench.py's CPU legs): build_coefficient_matrix's
 * matrix (s_integrate.cpp:5-149) as CSR with full rows, and the float step of
 * vvsl_field_rescaled in the reference's six passes with the Laplacian as two
 * sparse matrix-vector products (s_integrate.cpp:321-324). */
typedef struct orc_csr orc_csr;
orc_csr *orc_csr_build(const orc_params *p);
void orc_csr_free(orc_csr *A);
void orc_ref_step_f32(const orc_params *p, const orc_csr *A, float *phi1, float *phi2, float *pi1, float *pi2,
                      float *ker1, float *ker2, float *ker1n, float *ker2n, float *tau);

/* cores2 / cores3 (src/common/string_finding.cpp:3-86). mask[m] = 1 where the
 * cell with base corner m is flagged. Returns the number of flagged cells. */
int64_t orc_cores(const orc_params *p, const double *theta, uint8_t *mask);
/* 2D core count after the neighbouring-plaquette correction over the list in
 * ascending offset order (src/standard/s_run.cpp:101-109). */
int64_t orc_num_cores2(int N, const uint8_t *mask);
/* xi exactly as computed in float by s_run.cpp:111-114 (2D) and :123-129 (3D). */
float orc_xi(const orc_params *p, int64_t n_plaquettes, int64_t num_cores, double tau);

/* output_powerspec(data_real, data_imag) (src/common/pk_estimation.cpp:37-214).
 * data_imag may be NULL. pk, ks: N/2 doubles; count: N/2 ints. */
void orc_powerspec(const orc_params *p, const double *data_real, const double *data_imag,
                   double *pk, double *ks, int *count);

/* gaussian_thermal (src/common/init.cpp:33-200) with orc_normal() deviates.
 * The 3D k=0 phidot amplitude, left unset by init.cpp:163-164 (which assign
 * `amplitude` twice), is 0. Built with GCC -O2 the reference keeps the value
 * of the loop's previous mode there, so its phidot1/phidot2 exceed these by a
 * constant (tests/golden/make_golden.py measures it). */
void orc_gaussian_thermal(const orc_params *p, uint64_t seed,
                          double *phi1, double *phi2, double *phidot1, double *phidot2);

/* Flat-spectrum initial condition (no reference counterpart): unit amplitude
 * for 0 < |k| < kcut in the reference's k-grid, zero elsewhere, then scaled so
 * that <|phi|^2> = 1; phidot = 0. */
void orc_init_flat(const orc_params *p, uint64_t seed, double kcut,
                   double *phi1, double *phi2, double *phidot1, double *phidot2);

/* Background means of s_run.cpp:135-150: phi1, phi2, phidot1, phidot2,
 * |atan2(phi1,phi2)|, |phi|. */
void orc_background(const orc_params *p, const double *phi1, const double *phi2,
                    const double *phidot1, const double *phidot2, double out[6]);

/* Energy densities (no reference counterpart), averaged over the lattice, of
 * the unrescaled field phi = psi/tau: kinetic 1/2|phi'|^2, gradient
 * 1/2|grad phi|^2 (forward differences), potential
 * lambda/4 * tau^(2(1-prs)) * (|phi|^2-1)^2. */
void orc_energies(const orc_params *p, const double *psi1, const double *psi2,
                  const double *pi1, const double *pi2, double tau, double out[3]);

/* Axion kinetic-energy spectrum (no reference counterpart):
 * f = |phi| dtheta/dtau = (psi2*pi1 - psi1*pi2) / (tau |psi|), FFT, |F|^2 in
 * nbins log-spaced bins of |k| between 2pi/L and sqrt(NDIMS) pi/dx.
 * pk = L^d/N^(2d) <|F|^2>_bin, kmean = <|k|>_bin, count = modes per bin. */
void orc_axion_spectrum(const orc_params *p, const double *psi1, const double *psi2,
                        const double *pi1, const double *pi2, double tau, int nbins,
                        double *kmean, double *pk, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif
