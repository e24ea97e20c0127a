/* Project-written implementations behind oracle/shim/fftw3.h (test
 * infrastructure only): plans record their geometry; execution copies the
 * input to the output array and runs the oracle FFT in place there. */
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"
#include "../oracle.h"

struct axs_fftw_plan_s { int rank; int dims[3]; double *in; double *out; int sign; };

static fftw_plan make_plan(int rank, const int *dims, fftw_complex *in, fftw_complex *out, int sign) {
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->rank = rank;
    for (int d = 0; d < rank; ++d) p->dims[d] = dims[d];
    p->in = (double *)in; p->out = (double *)out; p->sign = sign;
    return p;
}
extern "C" fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
    (void)flags; int d[2] = { n0, n1 }; return make_plan(2, d, in, out, sign);
}
extern "C" fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
    (void)flags; int d[3] = { n0, n1, n2 }; return make_plan(3, d, in, out, sign);
}
extern "C" void fftw_execute(const fftw_plan p) {
    long total = 1;
    for (int d = 0; d < p->rank; ++d) total *= p->dims[d];
    if (p->out != p->in) memcpy(p->out, p->in, sizeof(double) * 2 * total);
    orc_fft_nd(p->out, p->rank, p->dims, p->sign);
}
extern "C" void fftw_destroy_plan(fftw_plan p) { free(p); }
extern "C" void *fftw_malloc(size_t n) { return malloc(n); }
extern "C" void fftw_free(void *p) { free(p); }
extern "C" int fftw_init_threads(void) { return 1; }
extern "C" void fftw_plan_with_nthreads(int n) { (void)n; }
extern "C" void fftw_cleanup_threads(void) {}
