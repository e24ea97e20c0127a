/* Project-written stand-in for the subset of Intel MKL's C interface that the
 * reference calls (src/common/mkl_wrapper.cpp:3-41, src/tests/fdm_matrix.cpp).
 * Declarations only; the implementations are in shim_mkl.cpp. Used only to
 * compile the reference's own sources as a cross-check of the oracle. */
#ifndef AXS_SHIM_MKL_H
#define AXS_SHIM_MKL_H
typedef int MKL_INT;
typedef unsigned int MKL_UINT;
#ifdef __cplusplus
extern "C" {
#endif
void cblas_daxpy(const MKL_INT n, const double a, const double *x, const MKL_INT incx, double *y, const MKL_INT incy);
void cblas_saxpy(const MKL_INT n, const float a, const float *x, const MKL_INT incx, float *y, const MKL_INT incy);
void cblas_dcopy(const MKL_INT n, const double *x, const MKL_INT incx, double *y, const MKL_INT incy);
void cblas_scopy(const MKL_INT n, const float *x, const MKL_INT incx, float *y, const MKL_INT incy);
#ifdef __cplusplus
}
#endif
#endif
