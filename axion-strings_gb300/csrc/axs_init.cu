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
// 2 in float, then * pi / L in double with L = dx * N in float. IEEE float and
// double operations, so the host table is the same bits the device would form.
static std::vector<double> kgrid_table(int N, float Lf) {
    std::vector<double> kg(N);
    for (int i = 0; i < N; ++i) {
        volatile float f = (-N / 2.0f + (float)i) * 2.0f;
        volatile double num = (double)f * 3.14159265358979323846;
        kg[i] = num / (double)Lf;
    }
    return kg;
}

// buf[m] = amp(|k|) * (g_{2 pair}(m) + i g_{2 pair + 1}(m)) in the reference's
// shifted k layout (index i <-> k = kg[i] = (-N/2 + i) 2 pi / L). A block takes
// rows (all but the fastest index fixed), so the coordinates cost no 64-bit
// division per site, and the squared k-grid of the row is formed once. With
// the k_cut amplitude, modes with k^2 >= k2_out (a double at or above kcut^2)
// have sqrt(k^2) >= kcut and amplitude zero without a square root.
__global__ void k_fill_kspace(double2 *__restrict__ buf, const double *__restrict__ kg, int N, int ndims,
                              uint64_t seed, int pair, float meff2, float T0, int thermal, double kcut,
                              double k2_out) {
    const int64_t rows = ndims == 2 ? (int64_t)N : (int64_t)N * N;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        double kr2;   // the row's share of k^2: ky^2 (2D), ki^2 + kj^2 (3D), in the reference's order
        if (ndims == 2) {
            const double ky = kg[r];
            kr2 = __dmul_rn(ky, ky);
        } else {
            const int ri = (int)(r / N), rj = (int)(r - (int64_t)ri * N);
            const double ki = kg[ri], kj = kg[rj];
            kr2 = __dadd_rn(__dmul_rn(ki, ki), __dmul_rn(kj, kj));
        }
        for (int x = threadIdx.x; x < N; x += blockDim.x) {
            const int64_t m = r * N + x;
            const double kl = kg[x];
            const double k2 = ndims == 2 ? __dadd_rn(__dmul_rn(kl, kl), kr2) : __dadd_rn(kr2, __dmul_rn(kl, kl));
            double amp = 0.0;
            if (thermal) {
                const double k = sqrt(k2);
                if (k != 0.0) {
                    double omegak = sqrt(__dadd_rn(__dmul_rn(k, k), (double)meff2));   // init.cpp:302
                    double bose = 1.0 / (exp(omegak / (double)T0) - 1.0);               // init.cpp:303
                    amp = pair == 0 ? sqrt(bose / omegak) : sqrt(bose * omegak);        // init.cpp:304-305
                }
            } else if (k2 < k2_out) {
                const double k = sqrt(k2);
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
}

// Checkerboard shift (init.cpp:320-321 / 390-391) and 1/N^d normalisation
// (init.cpp:323-330 / 393-400); re -> component 0, im -> component 1 of dst,
// times `scale`. Optionally accumulates sum |v|^2 (before scaling) per block.
// Rows as in k_fill_kspace (N is even, so the sign follows x + the row's
// indices). When N^d is a power of two, x / N^d is x * (1 / N^d) exactly, and
// (x / N^d) * scale is x * (scale / N^d) to the bit: one multiplication per
// component (GB300's FP64 rate makes each one count); otherwise the division.
template <typename T>
__global__ void k_finish(const double2 *__restrict__ buf, T *__restrict__ dst, int N, int ndims, double norm,
                         int norm_pow2, double scale, int write, double *partials) {
    double acc[1] = {0.0};
    const double f = scale / norm;   // exact when norm_pow2
    const int64_t rows = ndims == 2 ? (int64_t)N : (int64_t)N * N;
    typedef typename Cplx<T>::type C;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        const int rs = ndims == 2 ? (int)r : (int)(r / N) + (int)(r % N);
        for (int x = threadIdx.x; x < N; x += blockDim.x) {
            const int64_t m = r * N + x;
            double2 v = buf[m];
            if ((rs + x) & 1) { v.x = -v.x; v.y = -v.y; }
            if (norm_pow2) {
                if (partials) acc[0] += v.x * v.x + v.y * v.y;   // times 1/norm^2 (exact) afterwards
                if (write) {
                    C o;
                    o.x = (T)(v.x * f);
                    o.y = (T)(v.y * f);
                    reinterpret_cast<C *>(dst)[m] = o;
                }
            } else {
                v.x = v.x / norm;
                v.y = v.y / norm;
                if (partials) acc[0] += v.x * v.x + v.y * v.y;
                if (write) {
                    C o;
                    o.x = (T)(v.x * scale);
                    o.y = (T)(v.y * scale);
                    reinterpret_cast<C *>(dst)[m] = o;
                }
            }
        }
    }
    if (partials) {
        if (norm_pow2) acc[0] *= (1.0 / norm) * (1.0 / norm);
        block_reduce_store<1>(acc, partials);
    }
}

template <typename T>
static void finish(Lattice *L, double2 *buf, void *dst, double norm, double scale, int write, double *partials, int grid) {
    const int N = L->p.N;
    const int pow2 = (N & (N - 1)) == 0;   // N^d is then a power of two
    k_finish<T><<<grid, 256, 0, L->stream>>>(buf, (T *)dst, N, L->p.NDIMS, norm, pow2, scale, write, partials);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

void init_gaussian(Lattice *L, uint64_t seed, int thermal, double kcut) {
    const axs_params &p = L->p;
    int N = p.N;
    double2 *buf = (double2 *)dalloc((size_t)L->length * sizeof(double2));
    double *dkg = nullptr;
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
        const std::vector<double> kg = kgrid_table(N, Lf);
        dkg = (double *)dalloc((size_t)N * sizeof(double));
        AXS_CUDA(cudaMemcpyAsync(dkg, kg.data(), (size_t)N * sizeof(double), cudaMemcpyHostToDevice, L->stream));
        const double k2_out = std::nextafter(kcut * kcut, HUGE_VAL);   // >= kcut^2 exactly
        for (int pair = 0; pair < (thermal ? 2 : 1); ++pair) {
            k_fill_kspace<<<gf, 256, 0, L->stream>>>(buf, dkg, N, p.NDIMS, seed, pair, meff2, T0, thermal, kcut, k2_out);
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
        dfree(dkg);
        throw;
    }
    cufftDestroy(plan);
    dfree(buf);
    dfree(dkg);
}

}  // namespace axs
