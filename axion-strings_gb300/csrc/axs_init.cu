// Initial conditions: Gaussian random fields built in k-space and brought to
// the lattice by an inverse cuFFT, as gaussian_thermal does with MKL VSL and
// FFTW (src/common/init.cpp:33-200). The deviates are the project's
// Philox-4x32-10 + Box-Muller stream (normal_draw), a function of
// (seed, array, offset) only. The field is always built in FP64 and rounded to
// the lattice precision, so FP32 and FP64 runs start from the same field.
#include <cmath>
#include <vector>

#include "axs_internal.h"

namespace axs {

// k-grid of init.cpp:280-282 (2D) / :350-352 (3D): (-N/2 + i) in float, times
// 2 in float, then * pi / L in double with L = dx * N in float.
__device__ __forceinline__ double kgrid(int i, int N, float Lf) {
    float f = (-N / 2.0f + (float)i) * 2.0f;
    return __ddiv_rn(__dmul_rn((double)f, 3.14159265358979323846), (double)Lf);
}

// buf[m] = amp(|k|) * (g_{2 pair}(m) + i g_{2 pair + 1}(m)) in the reference's
// shifted k layout (index i <-> k = (-N/2 + i) 2 pi / L).
__global__ void k_fill_kspace(double2 *__restrict__ buf, int N, int ndims, int64_t len, uint64_t seed, int pair,
                              float Lf, float meff2, float T0, int thermal, double kcut) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        double k2;
        if (ndims == 2) {
            double kx = kgrid((int)(m % N), N, Lf), ky = kgrid((int)(m / N), N, Lf);
            k2 = __dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky));
        } else {
            int64_t NN = (int64_t)N * N;
            double ki = kgrid((int)(m / NN), N, Lf), kj = kgrid((int)((m / N) % N), N, Lf), kl = kgrid((int)(m % N), N, Lf);
            k2 = __dadd_rn(__dadd_rn(__dmul_rn(ki, ki), __dmul_rn(kj, kj)), __dmul_rn(kl, kl));
        }
        double k = sqrt(k2);
        double amp = 0.0;
        if (thermal) {
            if (k != 0.0) {
                double omegak = sqrt(__dadd_rn(__dmul_rn(k, k), (double)meff2));   // init.cpp:302
                double bose = 1.0 / (exp(omegak / (double)T0) - 1.0);               // init.cpp:303
                amp = pair == 0 ? sqrt(bose / omegak) : sqrt(bose * omegak);        // init.cpp:304-305
            }
        } else {
            amp = (k != 0.0 && k < kcut) ? 1.0 : 0.0;
        }
        double2 v;
        double g0 = 0.0, g1 = 0.0;
        if (amp != 0.0) normal_pair(seed, pair, m, g0, g1);   // zero-amplitude modes need no deviates
        v.x = amp * g0;
        v.y = amp * g1;
        buf[m] = v;
    }
}

// Checkerboard shift (init.cpp:320-321 / 390-391) and 1/N^d normalisation
// (init.cpp:323-330 / 393-400); re -> component 0, im -> component 1 of dst,
// times `scale`. Optionally accumulates sum |v|^2 (before scaling) per block.
template <typename T>
__global__ void k_finish(const double2 *__restrict__ buf, T *__restrict__ dst, int N, int ndims, int64_t len, double norm,
                         double scale, int write, double *partials) {
    double acc[1] = {0.0};
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        int64_t s;
        if (ndims == 2) s = (m % N) + (m / N);
        else s = (m / ((int64_t)N * N)) + ((m / N) % N) + (m % N);
        double2 v = buf[m];
        if (s & 1) { v.x = -v.x; v.y = -v.y; }
        v.x = v.x / norm;
        v.y = v.y / norm;
        if (partials) acc[0] += v.x * v.x + v.y * v.y;
        if (write) {
            dst[2 * m] = (T)(v.x * scale);
            dst[2 * m + 1] = (T)(v.y * scale);
        }
    }
    if (partials) block_reduce_store<1>(acc, partials);
}

template <typename T>
static void finish(Lattice *L, double2 *buf, void *dst, double norm, double scale, int write, double *partials, int grid) {
    k_finish<T><<<grid, 256, 0, L->stream>>>(buf, (T *)dst, L->p.N, L->p.NDIMS, L->length, norm, scale, write, partials);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

void init_gaussian(Lattice *L, uint64_t seed, int thermal, double kcut) {
    const axs_params &p = L->p;
    int N = p.N;
    double2 *buf = (double2 *)dalloc((size_t)L->length * sizeof(double2));
    cufftHandle plan = 0;
    try {
        if (p.NDIMS == 2) AXS_CUFFT(cufftPlan2d(&plan, N, N, CUFFT_Z2Z));
        else AXS_CUFFT(cufftPlan3d(&plan, N, N, N, CUFFT_Z2Z));
        AXS_CUFFT(cufftSetStream(plan, L->stream));
        float Lf = p.space_step * N;                                                       // init.cpp:37
        float T0 = p.T_initial;
        float meff2 = (float)(p.lambda * ((double)T0 * (double)T0 / 3.0f - 1.0f));      // physics.cpp:30
        double norm = p.NDIMS == 2 ? (double)N * (double)N : (double)N * (double)N * (double)N;
        int g = reduce_grid(L->length);
        int gf = (int)std::min<int64_t>((L->length + 255) / 256, (int64_t)num_sms() * 16);
        for (int pair = 0; pair < (thermal ? 2 : 1); ++pair) {
            k_fill_kspace<<<gf, 256, 0, L->stream>>>(buf, N, p.NDIMS, L->length, seed, pair, Lf, meff2, T0, thermal, kcut);
            AXS_CUDA(cudaGetLastError());
            count_launches(1);
            AXS_CUFFT(cufftExecZ2Z(plan, (cufftDoubleComplex *)buf, (cufftDoubleComplex *)buf, CUFFT_INVERSE));
            void *dst = pair == 0 ? L->psi[L->cur] : L->pih;
            double scale = 1.0;
            if (!thermal) {
                if (!L->dpartials || L->partials_cap < (size_t)g * 8) {
                    dfree(L->dpartials);
                    L->partials_cap = (size_t)g * 8;
                    L->dpartials = (double *)dalloc(L->partials_cap * sizeof(double));
                }
                if (L->esz == 4) finish<float>(L, buf, dst, norm, 1.0, 0, L->dpartials, g);
                else finish<double>(L, buf, dst, norm, 1.0, 0, L->dpartials, g);
                double s = 0;
                sum_partials(L->dpartials, g, 1, &s, L->stream);
                double mean = s / (double)L->length;
                scale = mean > 0.0 ? 1.0 / sqrt(mean) : 0.0;
            }
            if (L->esz == 4) finish<float>(L, buf, dst, norm, scale, 1, nullptr, gf);
            else finish<double>(L, buf, dst, norm, scale, 1, nullptr, gf);
        }
        if (!thermal) AXS_CUDA(cudaMemsetAsync(L->pih, 0, (size_t)L->length * 2 * L->esz, L->stream));
        AXS_CUDA(cudaStreamSynchronize(L->stream));
    } catch (...) {
        if (plan) cufftDestroy(plan);
        dfree(buf);
        throw;
    }
    cufftDestroy(plan);
    dfree(buf);
}

}  // namespace axs
