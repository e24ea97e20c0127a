/* Project-written stand-in for the FFTW3 subset the reference calls
 * (src/common/init.cpp, pk_estimation.cpp, src/standard/s_integrate.cpp).
 * Plans are executed by the oracle's own FFT (oracle/orc_fft.c) with FFTW's
 * sign convention and no normalisation. */
#ifndef AXS_SHIM_FFTW3_H
#define AXS_SHIM_FFTW3_H
#include <stddef.h>
typedef double fftw_complex[2];
typedef struct axs_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#ifdef __cplusplus
extern "C" {
#endif
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
#ifdef __cplusplus
}
#endif
#endif
