/* Project-written stand-in for the MKL VSL random-number interface the
 * reference calls (src/common/init.cpp:40,49-52). The generator behind it is
 * the project's Philox-4x32-10 + Box-Muller (oracle/orc_philox.h), not
 * SFMT19937; MKL's bitstream cannot be reproduced here. */
#ifndef AXS_SHIM_MKL_VSL_H
#define AXS_SHIM_MKL_VSL_H
#include "mkl.h"
typedef void *VSLStreamStatePtr;
#define VSL_BRNG_SFMT19937 (1 << 20)
#define VSL_RNG_METHOD_GAUSSIAN_ICDF 2
#ifdef __cplusplus
extern "C" {
#endif
int vslNewStream(VSLStreamStatePtr *stream, const MKL_INT brng, const MKL_UINT seed);
int vslDeleteStream(VSLStreamStatePtr *stream);
int vdRngGaussian(const MKL_INT method, VSLStreamStatePtr stream, const MKL_INT n, double r[], const double a, const double sigma);
int vsRngGaussian(const MKL_INT method, VSLStreamStatePtr stream, const MKL_INT n, float r[], const float a, const float sigma);
#ifdef __cplusplus
}
#endif
#endif
