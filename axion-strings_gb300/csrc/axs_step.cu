// Leapfrog evolution of the complex field: the fused kick/drift step and its
// helpers. Replaces vvsl_field_rescaled (src/standard/s_integrate.cpp:305-348)
// and the COO Laplacian it applies (s_integrate.cpp:5-149, 322-324).
//
// Formulation. The reference keeps (psi, pi, ker) and per step runs
//   psi += dt (pi + dt/2 ker);  tau += dt;  ker' = lap(psi) + V'(psi, tau);
//   pi  += dt/2 (ker + ker');   ker = ker'
// with ker = 0 before the first step (calloc, s_run.cpp:44-47). Writing
// pih = pi + dt/2 ker (the momentum at the half step) the same recursion is
//   step 0:       psi_1 = psi_0 + dt pi_0,              pih_0 = pi_0
//   step n >= 1:  pih_n = pih_{n-1} + dt K(psi_n, tau_n),  psi_{n+1} = psi_n + dt pih_n
// so one pass reads psi (with stencil halo) and pih and writes both: 4 reals
// read + 4 written per site, no stored kernel arrays. The synchronised
// momentum the reference holds between steps is pi_n = pih_{n-1} + dt/2 K_n,
// produced on demand by k_sync_pi.
//
// Device layout: psi and pih are complex-interleaved arrays (re = field 1,
// im = field 2) in the reference's site order; psi is double-buffered.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <functional>

#include "axs_internal.h"
#include "axs_tma.cuh"

namespace axs {

// ============================================================== small kernels

template <typename T>
__global__ void k_drift0(const typename Cplx<T>::type *__restrict__ psi, typename Cplx<T>::type *__restrict__ out,
                         const typename Cplx<T>::type *__restrict__ pih, const double *clock_in, double *clock_out,
                         int64_t len, double dt, int form) {
    const double t1 = *clock_in + dt;
    const T d = (T)(form == 1 ? dt / (t1 * t1) : dt);   // the drift of make_coefs
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        auto a = psi[m];
        auto p = pih[m];
        a.x = fma(d, p.x, a.x);
        a.y = fma(d, p.y, a.y);
        out[m] = a;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *clock_out = *clock_in + dt;
}

// Stencil sums of both components at site m for radius R (R = 1 uses the
// shared lap5/lap7 association order). Unscaled by 1/dx^2. NB (R = 1): the
// neighbour sums alone, for site_update_fold.
template <typename T, int ND, int R, bool NB = false>
__device__ __forceinline__ void stencil_at(const typename Cplx<T>::type *__restrict__ psi, int64_t m, int N,
                                           int setting, T &L1, T &L2, typename Cplx<T>::type &centre) {
    typedef typename Cplx<T>::type C;
    int64_t NN = (int64_t)N * N;
    int64_t x, y, z = 0;
    if (ND == 2) { x = m % N; y = m / N; }
    else { x = m % N; y = (m / N) % N; z = m / NN; }
    int64_t rowbase = m - x;                       // start of the x-row
    int64_t planebase = (ND == 2) ? 0 : z * NN;    // start of the z-plane
    C c = psi[m];
    centre = c;
    if (R == 1) {
        C xm = psi[rowbase + wrapi(x - 1, N)], xp = psi[rowbase + wrapi(x + 1, N)];
        C ym = psi[planebase + wrapi(y - 1, N) * N + x], yp = psi[planebase + wrapi(y + 1, N) * N + x];
        if (ND == 2) {
            L1 = NB ? nsum5<T>(xm.x, xp.x, ym.x, yp.x) : lap5<T>(c.x, xm.x, xp.x, ym.x, yp.x);
            L2 = NB ? nsum5<T>(xm.y, xp.y, ym.y, yp.y) : lap5<T>(c.y, xm.y, xp.y, ym.y, yp.y);
        } else {
            int64_t yx = y * N + x;
            C zm = psi[wrapi(z - 1, N) * NN + yx], zp = psi[wrapi(z + 1, N) * NN + yx];
            L1 = NB ? nsum7<T>(xm.x, xp.x, ym.x, yp.x, zm.x, zp.x) : lap7<T>(c.x, xm.x, xp.x, ym.x, yp.x, zm.x, zp.x);
            L2 = NB ? nsum7<T>(xm.y, xp.y, ym.y, yp.y, zm.y, zp.y) : lap7<T>(c.y, xm.y, xp.y, ym.y, yp.y, zm.y, zp.y);
        }
        return;
    }
    T a1 = (T)stencil_coef(setting, ND, 0) * c.x;
    T a2 = (T)stencil_coef(setting, ND, 0) * c.y;
#pragma unroll
    for (int l = 1; l <= R; ++l) {
        C xm = psi[rowbase + wrapi(x - l, N)], xp = psi[rowbase + wrapi(x + l, N)];
        C ym = psi[planebase + wrapi(y - l, N) * N + x], yp = psi[planebase + wrapi(y + l, N) * N + x];
        T s1 = (xm.x + xp.x) + (ym.x + yp.x), s2 = (xm.y + xp.y) + (ym.y + yp.y);
        if (ND == 3) {
            int64_t yx = y * N + x;
            C zm = psi[wrapi(z - l, N) * NN + yx], zp = psi[wrapi(z + l, N) * NN + yx];
            s1 = s1 + (zm.x + zp.x);
            s2 = s2 + (zm.y + zp.y);
        }
        T cl = (T)stencil_coef(setting, ND, l);
        a1 = fma(cl, s1, a1);
        a2 = fma(cl, s2, a2);
    }
    L1 = a1;
    L2 = a2;
}

// One step, one thread per site (grid-stride). Used for 2D, stencil radii
// 2..4 and lattice shapes the z-march kernel does not tile.
template <typename T, int ND, int R>
__global__ void __launch_bounds__(256) k_step_generic(const typename Cplx<T>::type *__restrict__ psi,
                                                      typename Cplx<T>::type *__restrict__ out,
                                                      typename Cplx<T>::type *__restrict__ pih,
                                                      const double *clock_in, double *clock_out, int N, int64_t len,
                                                      double dt, double inv_dx2, double lambda, double T0sq3, int prs,
                                                      int setting, int form) {
    double tau = *clock_in;
    StepCoefs<T> c = make_coefs<T>(tau, dt, dt, inv_dx2, lambda, T0sq3, prs, form);
    constexpr bool FOLD = sizeof(T) == 8 && R == 1;
    const T kctr = c.kdt_idx2 * (T)(-2 * ND);
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        T L1, L2;
        typename Cplx<T>::type ctr;
        stencil_at<T, ND, R, FOLD>(psi, m, N, setting, L1, L2, ctr);
        auto p = pih[m];
        typename Cplx<T>::type o;
        if constexpr (FOLD) site_update_fold<T>(ctr.x, ctr.y, L1, L2, p.x, p.y, o.x, o.y, c, kctr);
        else site_update<T>(ctr.x, ctr.y, L1, L2, p.x, p.y, o.x, o.y, c);
        pih[m] = p;
        out[m] = o;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *clock_out = tau + dt;
}

// Synchronised momentum pi_n = pih_{n-1} + dt/2 K(psi_n, tau_n) into `dst`.
template <typename T, int ND, int R>
__global__ void k_sync_pi(const typename Cplx<T>::type *__restrict__ psi, const typename Cplx<T>::type *__restrict__ pih,
                          typename Cplx<T>::type *__restrict__ dst, const double *clock, int N, int64_t len, double dt,
                          double inv_dx2, double lambda, double T0sq3, int prs, int setting, int form) {
    StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, inv_dx2, lambda, T0sq3, prs, form);
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        T L1, L2;
        typename Cplx<T>::type ctr;
        stencil_at<T, ND, R>(psi, m, N, setting, L1, L2, ctr);
        auto p = pih[m];
        sync_pi_site<T>(ctr.x, ctr.y, L1, L2, p.x, p.y, c);
        dst[m] = p;
    }
}

// ---- spectral Laplacian (compute_laplacian_fft, s_integrate.cpp:179-296)
//
// L phi = IFFT(-k^2 FFT(phi)) / N^d. psi is complex-interleaved (re = phi1,
// im = phi2) and -k^2 is real and even in k, so one complex transform pair
// gives both fields' Laplacians (re and im of the result). The reference's
// (-1)^(i+j+k) factors before and after its transforms only relabel the
// frequencies: in the unshifted layout index j holds frequency j (j < N/2) or
// j - N, whose k is the reference's k of shifted index j + N/2 (mod N).
// ksq[j] is that k^2 (host-computed as the reference computes k, in double;
// N doubles then the same N rounded to float).

// W *= -(k_z^2 + k_y^2 + k_x^2) (slowest axis first, as coordinate3 orders it;
// 2D: k_x^2 + k_y^2 with x fastest, as coordinate2).
template <typename T>
__global__ void k_kspace_laplacian(typename Cplx<T>::type *__restrict__ W, const void *__restrict__ ksq_tab, int N,
                                   int ndims, int64_t len) {
    const double *kd = reinterpret_cast<const double *>(ksq_tab);
    const float *kf = reinterpret_cast<const float *>(kd + N);
    const int64_t NN = (int64_t)N * N;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        int a, b, c = -1;   // slowest .. fastest
        if (ndims == 2) { a = (int)(m % N); b = (int)(m / N); }
        else { a = (int)(m / NN); b = (int)((m / N) % N); c = (int)(m % N); }
        auto w = W[m];
        if (sizeof(T) == 8) {
            double s = kd[a] + kd[b];
            if (c >= 0) s = s + kd[c];
            w.x = (T)((double)w.x * -s);
            w.y = (T)((double)w.y * -s);
        } else {
            float s = kf[a] + kf[b];
            if (c >= 0) s = s + kf[c];
            w.x = (T)((float)w.x * -s);
            w.y = (T)((float)w.y * -s);
        }
        W[m] = w;
    }
}

// One step with the spectral Laplacian: W holds N^d L psi (both components).
template <typename T>
__global__ void __launch_bounds__(256) k_step_spectral(const typename Cplx<T>::type *__restrict__ psi,
                                                       typename Cplx<T>::type *__restrict__ out,
                                                       typename Cplx<T>::type *__restrict__ pih,
                                                       const typename Cplx<T>::type *__restrict__ W,
                                                       const double *clock_in, double *clock_out, int64_t len,
                                                       double dt, double lambda, double T0sq3, int prs, int form) {
    const double tau = *clock_in;
    const StepCoefs<T> c = make_coefs<T>(tau, dt, dt, 1.0, lambda, T0sq3, prs, form);   // k already physical
    const T ilen = (T)len;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        const auto a = psi[m];
        const auto w = W[m];
        auto p = pih[m];
        typename Cplx<T>::type o;
        site_update<T>(a.x, a.y, w.x / ilen, w.y / ilen, p.x, p.y, o.x, o.y, c);   // ret = data / length, :228-231
        pih[m] = p;
        out[m] = o;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *clock_out = tau + dt;
}

// pi_n = pih + dt/2 K(psi_n) with the spectral Laplacian in W; written over W.
template <typename T>
__global__ void k_sync_pi_spectral(const typename Cplx<T>::type *__restrict__ psi,
                                   const typename Cplx<T>::type *__restrict__ pih, typename Cplx<T>::type *W,
                                   const double *clock, int64_t len, double dt, double lambda, double T0sq3, int prs,
                                   int form) {
    const StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, 1.0, lambda, T0sq3, prs, form);
    const T ilen = (T)len;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        const auto a = psi[m];
        const auto w = W[m];
        auto p = pih[m];
        sync_pi_site<T>(a.x, a.y, w.x / ilen, w.y / ilen, p.x, p.y, c);
        W[m] = p;
    }
}

// One component of the spectral Laplacian in W into a double array.
template <typename T>
__global__ void k_laplacian_spectral(const typename Cplx<T>::type *__restrict__ W, double *__restrict__ out, int comp,
                                     int64_t len) {
    const T ilen = (T)len;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        const auto w = W[m];
        out[m] = (double)((comp ? w.y : w.x) / ilen);
    }
}

// (1/dx^2) * stencil of one component, in double.
template <typename T, int ND, int R>
__global__ void k_laplacian(const typename Cplx<T>::type *__restrict__ psi, double *__restrict__ out, int comp, int N,
                            int64_t len, double inv_dx2, int setting) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        T L1, L2;
        typename Cplx<T>::type ctr;
        stencil_at<T, ND, R>(psi, m, N, setting, L1, L2, ctr);
        out[m] = inv_dx2 * (double)(comp ? L2 : L1);
    }
}

// Real host-order array <-> one component of a complex device array.
template <typename T, typename S>
__global__ void k_pack(const S *__restrict__ src, T *__restrict__ dst_cplx, int comp, int64_t len) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride)
        dst_cplx[2 * m + comp] = (T)src[m];
}
template <typename T, typename S>
__global__ void k_unpack(const T *__restrict__ src_cplx, S *__restrict__ dst, int comp, int64_t len) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride)
        dst[m] = (S)src_cplx[2 * m + comp];
}

// Two real host-order arrays <-> a complex device array (whole 8/16-byte
// sites, so no partial-sector writes). Either side may be host memory the
// device can address (page-locked, reached over NVLink-C2C) or device memory.
template <typename T, typename S>
__global__ void k_pack2(const S *__restrict__ a, const S *__restrict__ b, typename Cplx<T>::type *__restrict__ dst,
                        int64_t len) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        typename Cplx<T>::type v;
        v.x = (T)a[m];
        v.y = (T)b[m];
        dst[m] = v;
    }
}
template <typename T, typename S>
__global__ void k_unpack2(const typename Cplx<T>::type *__restrict__ src, S *__restrict__ a, S *__restrict__ b,
                          int64_t len) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        typename Cplx<T>::type v = src[m];
        a[m] = (S)v.x;
        b[m] = (S)v.y;
    }
}

// The same four sites per thread in 16-byte accesses (all three arrays 16-byte
// aligned, len a multiple of 4): page-locked host arrays are read and written
// over NVLink-C2C, where wide requests move more bytes per transaction.
template <typename S> struct Quad;
template <> struct Quad<float> {
    static __device__ __forceinline__ void load(const float *p, float (&v)[4]) {
        const float4 q = *reinterpret_cast<const float4 *>(p);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
    static __device__ __forceinline__ void store(float *p, const float (&v)[4]) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <> struct Quad<double> {
    static __device__ __forceinline__ void load(const double *p, double (&v)[4]) {
        const double2 q0 = reinterpret_cast<const double2 *>(p)[0], q1 = reinterpret_cast<const double2 *>(p)[1];
        v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
    static __device__ __forceinline__ void store(double *p, const double (&v)[4]) {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    }
};
template <typename T, typename S>
__global__ void k_pack2_x4(const S *__restrict__ a, const S *__restrict__ b, T *__restrict__ dst, int64_t len4) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < len4; q += stride) {
        S va[4], vb[4];
        Quad<S>::load(a + 4 * q, va);
        Quad<S>::load(b + 4 * q, vb);
        T lo[4] = {(T)va[0], (T)vb[0], (T)va[1], (T)vb[1]}, hi[4] = {(T)va[2], (T)vb[2], (T)va[3], (T)vb[3]};
        Quad<T>::store(dst + 8 * q, lo);
        Quad<T>::store(dst + 8 * q + 4, hi);
    }
}
// Upload of the momentum pair with the first step of a fresh state fused in:
// pih = (a, b) as k_pack2(_x4) stores it, and psi_next = psi + d pih with
// k_drift0's arithmetic (the reference's first step with ker_curr = 0 is a
// pure drift). The upload is bound by the host link, so the drift's device
// traffic costs nothing there. One thread writes the next clock.
template <typename T, typename S>
__global__ void k_pack2_drift(const S *__restrict__ a, const S *__restrict__ b, typename Cplx<T>::type *__restrict__ pih,
                              const typename Cplx<T>::type *__restrict__ psi, typename Cplx<T>::type *__restrict__ psi_next,
                              int64_t len, const double *clock_in, double *clock_out, double dt, int form) {
    const double t1 = *clock_in + dt;
    const T d = (T)(form == 1 ? dt / (t1 * t1) : dt);   // the drift of make_coefs
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        typename Cplx<T>::type v, q = psi[m];
        v.x = (T)a[m];
        v.y = (T)b[m];
        pih[m] = v;
        q.x = fma(d, v.x, q.x);
        q.y = fma(d, v.y, q.y);
        psi_next[m] = q;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *clock_out = *clock_in + dt;
}
template <typename T, typename S>
__global__ void k_pack2_drift_x4(const S *__restrict__ a, const S *__restrict__ b, T *__restrict__ pih,
                                 const T *__restrict__ psi, T *__restrict__ psi_next, int64_t len4,
                                 const double *clock_in, double *clock_out, double dt, int form) {
    const double t1 = *clock_in + dt;
    const T d = (T)(form == 1 ? dt / (t1 * t1) : dt);
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < len4; q += stride) {
        S va[4], vb[4];
        Quad<S>::load(a + 4 * q, va);
        Quad<S>::load(b + 4 * q, vb);
        T lo[4] = {(T)va[0], (T)vb[0], (T)va[1], (T)vb[1]}, hi[4] = {(T)va[2], (T)vb[2], (T)va[3], (T)vb[3]};
        Quad<T>::store(pih + 8 * q, lo);
        Quad<T>::store(pih + 8 * q + 4, hi);
        T slo[4], shi[4];
        Quad<T>::load(psi + 8 * q, slo);
        Quad<T>::load(psi + 8 * q + 4, shi);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            slo[i] = fma(d, lo[i], slo[i]);
            shi[i] = fma(d, hi[i], shi[i]);
        }
        Quad<T>::store(psi_next + 8 * q, slo);
        Quad<T>::store(psi_next + 8 * q + 4, shi);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *clock_out = *clock_in + dt;
}
template <typename T, typename S>
__global__ void k_unpack2_x4(const T *__restrict__ src, S *__restrict__ a, S *__restrict__ b, int64_t len4) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < len4; q += stride) {
        T lo[4], hi[4];
        Quad<T>::load(src + 8 * q, lo);
        Quad<T>::load(src + 8 * q + 4, hi);
        const S va[4] = {(S)lo[0], (S)lo[2], (S)hi[0], (S)hi[2]}, vb[4] = {(S)lo[1], (S)lo[3], (S)hi[1], (S)hi[3]};
        Quad<S>::store(a + 4 * q, va);
        Quad<S>::store(b + 4 * q, vb);
    }
}

// ============================================================== z-march kernel
//
// 3D, radius 1. A work item is (lattice, x-y tile of tx * TY sites, z-chunk).
// A CTA marches its tile through the z-chunk keeping the psi planes z-1, z,
// z+1 in a ring of S shared-memory slots. Each plane (tile plus one-row y halo
// and 16-byte x halo, periodic) arrives by 3-5 TMA tensor loads completing on
// the slot's mbarrier; thread 0 refills a slot as soon as the CTA has finished
// with the plane in it, so S-3 planes are in flight ahead of the consumer.
// pih streams through registers one plane ahead. CTAs are persistent and take
// items from a global counter in z-chunk-major order, so tiles that share
// halo rows run at the same time and meet their halos in L2.

template <typename T, int TY, int TXMAX, int S>
struct ZCfg {
    static constexpr int CS = 2 * (int)sizeof(T);             // bytes per complex site
    static constexpr int VS = 16 / CS;                        // sites per 16-byte vector
    static constexpr int EU = CS / 8;                         // tensor-map elements per site
    static constexpr int NT = 256;
    static constexpr int MAXV = (TXMAX * TY / VS + NT - 1) / NT;
    static constexpr int C_BYTES = (TY + 2) * TXMAX * CS;
    static constexpr int H_BYTES = TY * 16;                   // one x-halo strip
    static constexpr int H_PAD = (H_BYTES + 127) / 128 * 128; // strips start 128-byte aligned
    static constexpr int SLOT = ((C_BYTES + 2 * H_PAD) + 127) / 128 * 128;
    static constexpr int SMEM = S * SLOT + 128;               // + mbarriers and item broadcast
};

template <typename T, int TY, int TXMAX, int S>
__global__ void __launch_bounds__(256) k_zmarch(const ZLat *__restrict__ lats, int nlat, int64_t total_items,
                                                int *counters, int parity, int *derr) {
    typedef ZCfg<T, TY, TXMAX, S> K;
    typedef typename Cplx<T>::type C;
    typedef typename Vec16<T>::type V;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * K::SLOT);
    volatile int64_t *item_bc = reinterpret_cast<volatile int64_t *>(smem + S * K::SLOT + 64);
    const int tid = threadIdx.x;

    (void)parity;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // counters[0]: next work item; counters[1]: CTAs finished. The last CTA
    // to finish zeroes both, so every launch starts from a clean counter.
    int64_t qbase = 0;   // loads issued by this CTA before the current item
    for (;;) {
        if (tid == 0) *item_bc = (int64_t)atomicAdd(&counters[0], 1);
        __syncthreads();
        const int64_t item = *item_bc;
        if (item >= total_items) break;
        // ---- decode the item
        const int li = find_lat(lats, nlat, item);
        const ZLat &Lt = lats[li];
        const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
        const int64_t local = item - Lt.item_base;
        const int ncols = ntx * nty;
        const int zq = (int)(local / ncols), col = (int)(local % ncols);
        const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
        const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
        const int T_steps = zb - za;
        const int nload = T_steps + 2;
        const int bin = Lt.a_index ^ parity;   // input psi buffer / clock slot
        C *psi_out = reinterpret_cast<C *>(Lt.psi[bin ^ 1]);
        const C *pih = reinterpret_cast<const C *>(Lt.pih[bin]);
        C *pih_out = reinterpret_cast<C *>(Lt.pih[bin ^ 1]);
        const double tau = Lt.clock[bin];
        const StepCoefs<T> cf = make_coefs<T>(tau, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
        if (local == 0 && tid == 0) Lt.clock[bin ^ 1] = tau + Lt.dt;   // tau += dt, s_integrate.cpp:317
        const bool xhalo = tx < N;
        const uint32_t slot_bytes_tx = (uint32_t)((TY + 2) * tx * K::CS + (xhalo ? 2 * K::H_BYTES : 0));

        auto issue = [&](int64_t q) {   // load q of the CTA stream = plane za-1+(q-qbase)
            const int i = (int)(q - qbase);
            int z = za - 1 + i;
            z = z < 0 ? z + N : (z >= N ? z - N : z);
            const int s = (int)(q % S);
            unsigned char *slot = smem + s * K::SLOT;
            const uint32_t bar = smem_u32(&bars[s]);
            mbar_expect_tx(bar, slot_bytes_tx + (i == 0 ? (uint32_t)Lt.debug_tx_excess : 0u));
            const int ym = y0 == 0 ? N - 1 : y0 - 1;
            const int yp = (y0 + TY == N) ? 0 : y0 + TY;
            tma_load_3d(smem_u32(slot), &Lt.tm_row[bin], x0 * K::EU, ym, z, bar);
            tma_load_3d(smem_u32(slot + tx * K::CS), &Lt.tm_main[bin], x0 * K::EU, y0, z, bar);
            tma_load_3d(smem_u32(slot + (TY + 1) * tx * K::CS), &Lt.tm_row[bin], x0 * K::EU, yp, z, bar);
            if (xhalo) {
                const int xl = (x0 - K::VS + N) % N, xr = (x0 + tx) % N;
                tma_load_3d(smem_u32(slot + K::C_BYTES), &Lt.tm_xh[bin], xl * K::EU, y0, z, bar);
                tma_load_3d(smem_u32(slot + K::C_BYTES + K::H_PAD), &Lt.tm_xh[bin], xr * K::EU, y0, z, bar);
            }
        };

        int64_t issued = qbase;
        if (tid == 0) {
            const int64_t lim = qbase + min(nload, S);
            for (; issued < lim; ++issued) issue(issued);
        }
        const int nvx = tx / K::VS;
        const int nvec = nvx * TY;
        // prefetch pih for the first plane
        V pcur[K::MAXV];
#pragma unroll
        for (int k = 0; k < K::MAXV; ++k) {
            const int v = tid + k * K::NT;
            if (v < nvec) {
                const int yy = v / nvx, xx = (v % nvx) * K::VS;
                const int64_t off = ((int64_t)za * N + (y0 + yy)) * N + (x0 + xx);
                pcur[k] = *reinterpret_cast<const V *>(&pih[off]);
            }
        }
        bool ok = true, aborted = false;
        for (int t = 0; t < T_steps; ++t) {
            const int z = za + t;
            // planes z-1, z, z+1 = loads qbase+t, +t+1, +t+2
            if (t == 0) {
                ok = ok && mbar_wait_bounded(smem_u32(&bars[(qbase) % S]), (uint32_t)(((qbase) / S) & 1));
                ok = ok && mbar_wait_bounded(smem_u32(&bars[(qbase + 1) % S]), (uint32_t)(((qbase + 1) / S) & 1));
            }
            const int64_t qn = qbase + t + 2;
            ok = ok && mbar_wait_bounded(smem_u32(&bars[qn % S]), (uint32_t)((qn / S) & 1));
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(derr, DEVERR_TIMEOUT);
                aborted = true;
                break;
            }
            const C *Cm = reinterpret_cast<const C *>(smem + ((qbase + t) % S) * K::SLOT);
            const C *Cz = reinterpret_cast<const C *>(smem + ((qbase + t + 1) % S) * K::SLOT);
            const C *Cp = reinterpret_cast<const C *>(smem + ((qbase + t + 2) % S) * K::SLOT);
            const C *Lh = reinterpret_cast<const C *>(smem + ((qbase + t + 1) % S) * K::SLOT + K::C_BYTES);
            const C *Rh = reinterpret_cast<const C *>(smem + ((qbase + t + 1) % S) * K::SLOT + K::C_BYTES + K::H_PAD);
            V pnext[K::MAXV];
#pragma unroll
            for (int k = 0; k < K::MAXV; ++k) {
                const int v = tid + k * K::NT;
                if (v < nvec && t + 1 < T_steps) {
                    const int yy = v / nvx, xx = (v % nvx) * K::VS;
                    const int64_t off = ((int64_t)(z + 1) * N + (y0 + yy)) * N + (x0 + xx);
                    pnext[k] = *reinterpret_cast<const V *>(&pih[off]);
                }
            }
#pragma unroll
            for (int k = 0; k < K::MAXV; ++k) {
                const int v = tid + k * K::NT;
                if (v >= nvec) continue;
                const int yy = v / nvx, xx = (v % nvx) * K::VS;
                const int r = (1 + yy) * tx + xx;
                C ctr[K::VS], up[K::VS], dn[K::VS], zm[K::VS], zp[K::VS];
                *reinterpret_cast<V *>(ctr) = *reinterpret_cast<const V *>(&Cz[r]);
                *reinterpret_cast<V *>(up) = *reinterpret_cast<const V *>(&Cz[r - tx]);
                *reinterpret_cast<V *>(dn) = *reinterpret_cast<const V *>(&Cz[r + tx]);
                *reinterpret_cast<V *>(zm) = *reinterpret_cast<const V *>(&Cm[r]);
                *reinterpret_cast<V *>(zp) = *reinterpret_cast<const V *>(&Cp[r]);
                C left, right;
                if (xx > 0) left = Cz[r - 1];
                else left = xhalo ? Lh[yy * K::VS + K::VS - 1] : Cz[(1 + yy) * tx + tx - 1];
                if (xx + K::VS < tx) right = Cz[r + K::VS];
                else right = xhalo ? Rh[yy * K::VS] : Cz[(1 + yy) * tx];
                T pv[2 * K::VS];
                *reinterpret_cast<V *>(pv) = pcur[k];
                C outv[K::VS];
#pragma unroll
                for (int j = 0; j < K::VS; ++j) {
                    const C xm = (j == 0) ? left : ctr[j - 1];
                    const C xp = (j == K::VS - 1) ? right : ctr[j + 1];
                    if constexpr (sizeof(T) == 8) {   // FP64: the centre weight folded (site_update_fold)
                        const T S1 = nsum7<T>(xm.x, xp.x, up[j].x, dn[j].x, zm[j].x, zp[j].x);
                        const T S2 = nsum7<T>(xm.y, xp.y, up[j].y, dn[j].y, zm[j].y, zp[j].y);
                        site_update_fold<T>(ctr[j].x, ctr[j].y, S1, S2, pv[2 * j], pv[2 * j + 1], outv[j].x, outv[j].y,
                                            cf, cf.kdt_idx2 * (T)-6);
                    } else {
                        const T L1 = lap7<T>(ctr[j].x, xm.x, xp.x, up[j].x, dn[j].x, zm[j].x, zp[j].x);
                        const T L2 = lap7<T>(ctr[j].y, xm.y, xp.y, up[j].y, dn[j].y, zm[j].y, zp[j].y);
                        site_update<T>(ctr[j].x, ctr[j].y, L1, L2, pv[2 * j], pv[2 * j + 1], outv[j].x, outv[j].y, cf);
                    }
                }
                const int64_t off = ((int64_t)z * N + (y0 + yy)) * N + (x0 + xx);
                *reinterpret_cast<V *>(&pih_out[off]) = *reinterpret_cast<V *>(pv);
                *reinterpret_cast<V *>(&psi_out[off]) = *reinterpret_cast<V *>(outv);
            }
#pragma unroll
            for (int k = 0; k < K::MAXV; ++k) pcur[k] = pnext[k];
            __syncthreads();   // every thread is done with plane z-1's slot
            if (tid == 0) {
                const int64_t dead = (t == T_steps - 1) ? qbase + nload : qbase + t + 1;
                const int64_t lim = min(qbase + nload, dead + S);
                for (; issued < lim; ++issued) issue(issued);
            }
        }
        if (aborted) {
            // Wait (bounded) for this CTA's copies still in flight, then stop.
            if (tid == 0) {
                for (int64_t q = qbase; q < issued; ++q) mbar_wait_bounded(smem_u32(&bars[q % S]), (uint32_t)((q / S) & 1));
            }
            __syncthreads();
            break;
        }
        qbase += nload;
        __syncthreads();
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&counters[1], 1) == (int)gridDim.x - 1) {
            counters[0] = 0;
            counters[1] = 0;
            __threadfence();
        }
    }
}

// ============================================================== z-march, warp-specialised
//
// Same work items and halo boxes as k_zmarch, organised as a producer /
// consumer pipeline with no CTA-wide barrier in the steady state:
//  * warp NCW (one lane) is the producer: it takes items from the global
//    counter one item ahead of the consumers and issues, per plane, the TMA
//    loads of psi (tile + periodic halos) AND of pih (tile) into a ring slot,
//    after waiting on that slot's `empty` mbarrier;
//  * warps 0..NCW-1 are consumers: they wait on the slot's `full` mbarrier,
//    compute the plane, store psi_new and pih with 16-byte stores, and arrive
//    on `empty` when they are done with a plane.
// Items reach the consumers through a two-entry queue guarded by mbarriers.

template <typename T, int TY, int TXMAX, int S>
struct Z2Cfg {
    static constexpr int CS = 2 * (int)sizeof(T);
    static constexpr int VS = 16 / CS;
    static constexpr int EU = CS / 8;
    static constexpr int NCW = 8;                              // consumer warps
    static constexpr int NT = (NCW + 1) * 32;
    static constexpr int NC = NCW * 32;                        // consumer threads
    static constexpr int MAXV = (TXMAX * TY / VS + NC - 1) / NC;
    static constexpr int C_BYTES = (TY + 2) * TXMAX * CS;      // psi rows y0-1 .. y0+TY
    static constexpr int H_PAD = (TY * 16 + 127) / 128 * 128;  // one x-halo strip
    static constexpr int P_OFF = C_BYTES + 2 * H_PAD;          // pih tile
    static constexpr int SLOT = (P_OFF + TY * TXMAX * CS + 127) / 128 * 128;
    static constexpr int BAR_OFF = S * SLOT;
    static constexpr int SMEM = BAR_OFF + 256;
};

template <typename T, int TY, int TXMAX, int S>
__global__ void __launch_bounds__(Z2Cfg<T, TY, TXMAX, S>::NT)
    k_zmarch2(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity, int *derr) {
    typedef Z2Cfg<T, TY, TXMAX, S> K;
    typedef typename Cplx<T>::type C;
    typedef typename Vec16<T>::type V;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + K::BAR_OFF);
    uint64_t *empty = full + S;
    uint64_t *ifull = empty + S;                                 // [2]
    uint64_t *iempty = ifull + 2;                                // [2]
    volatile int64_t *items = reinterpret_cast<volatile int64_t *>(iempty + 2);   // [2]
    volatile int *abort_flag = reinterpret_cast<volatile int *>(items + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), K::NCW);
        }
        for (int k = 0; k < 2; ++k) {
            mbar_init(smem_u32(&ifull[k]), 1);
            mbar_init(smem_u32(&iempty[k]), K::NCW);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == K::NCW) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int64_t q = 0;
            bool ok = true;
            for (int64_t k = 0; ok; ++k) {
                if (k >= 2) ok = mbar_wait_bounded(smem_u32(&iempty[k & 1]), (uint32_t)(((k >> 1) - 1) & 1));
                if (!ok || *abort_flag) break;
                const int64_t item = (int64_t)atomicAdd(&counters[0], 1);
                items[k & 1] = item;
                mbar_arrive(smem_u32(&ifull[k & 1]));
                if (item >= total_items) break;
                const int li = find_lat(lats, nlat, item);
                const ZLat &Lt = lats[li];
                const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
                const int64_t local = item - Lt.item_base;
                const int ncols = ntx * nty;
                const int zq = (int)(local / ncols), col = (int)(local % ncols);
                const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
                const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
                const int nload = zb - za + 2;
                const int bin = Lt.a_index ^ parity;
                const bool xhalo = tx < N;
                const uint32_t psi_bytes = (uint32_t)((TY + 2) * tx * K::CS + (xhalo ? 2 * TY * 16 : 0));
                const uint32_t pih_bytes = (uint32_t)(TY * tx * K::CS);
                const int ym = y0 == 0 ? N - 1 : y0 - 1;
                const int yp = (y0 + TY == N) ? 0 : y0 + TY;
                for (int i = 0; i < nload; ++i, ++q) {
                    const int s = (int)(q % S);
                    if (q >= S) {
                        ok = mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)(((q / S) - 1) & 1));
                        if (!ok || *abort_flag) break;
                    }
                    int z = za - 1 + i;
                    z = z < 0 ? z + N : (z >= N ? z - N : z);
                    unsigned char *slot = smem + s * K::SLOT;
                    const uint32_t bar = smem_u32(&full[s]);
                    const bool with_pih = i >= 1 && i <= nload - 2;
                    mbar_expect_tx(bar, psi_bytes + (with_pih ? pih_bytes : 0u) +
                                            (i == 0 ? (uint32_t)Lt.debug_tx_excess : 0u));
                    tma_load_3d(smem_u32(slot), &Lt.tm_row[bin], x0 * K::EU, ym, z, bar);
                    tma_load_3d(smem_u32(slot + tx * K::CS), &Lt.tm_main[bin], x0 * K::EU, y0, z, bar);
                    tma_load_3d(smem_u32(slot + (TY + 1) * tx * K::CS), &Lt.tm_row[bin], x0 * K::EU, yp, z, bar);
                    if (xhalo) {
                        const int xl = (x0 - K::VS + N) % N, xr = (x0 + tx) % N;
                        tma_load_3d(smem_u32(slot + K::C_BYTES), &Lt.tm_xh[bin], xl * K::EU, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::C_BYTES + K::H_PAD), &Lt.tm_xh[bin], xr * K::EU, y0, z, bar);
                    }
                    if (with_pih) tma_load_3d(smem_u32(slot + K::P_OFF), &Lt.tm_pih[bin], x0 * K::EU, y0, z, bar);
                }
            }
            if (!ok) {
                atomicOr(derr, DEVERR_TIMEOUT);
                *abort_flag = 1;
            }
            // Drain: wait (bounded) for this CTA's last loads still in flight.
            for (int64_t d = q > S ? q - S : 0; d < q; ++d)
                mbar_wait_bounded(smem_u32(&full[d % S]), (uint32_t)((d / S) & 1));
        }
    } else {
        // ------------------------------------------------------------ consumers
        const int cid = tid;   // 0 .. NC-1
        int64_t q0 = 0;
        for (int64_t k = 0;; ++k) {
            const int w0 = warp_wait(smem_u32(&ifull[k & 1]), (uint32_t)((k >> 1) & 1), abort_flag);
            if (w0) {
                if (w0 == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                break;
            }
            bool ok = true;
            const int64_t item = items[k & 1];
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&iempty[k & 1]));
            if (item >= total_items) break;
            const int li = find_lat(lats, nlat, item);
            const ZLat &Lt = lats[li];
            const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
            const int64_t local = item - Lt.item_base;
            const int ncols = ntx * nty;
            const int zq = (int)(local / ncols), col = (int)(local % ncols);
            const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
            const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
            const int T_steps = zb - za;
            const int bin = Lt.a_index ^ parity;
            C *psi_out = reinterpret_cast<C *>(Lt.psi[bin ^ 1]);
            C *pih = reinterpret_cast<C *>(Lt.pih[bin ^ 1]);   // output; the input arrives by TMA
            const double tau = Lt.clock[bin];
            const StepCoefs<T> cf = make_coefs<T>(tau, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            if (local == 0 && cid == 0) Lt.clock[bin ^ 1] = tau + Lt.dt;   // tau += dt, s_integrate.cpp:317
            const bool xhalo = tx < N;
            const int nvx = tx / K::VS;
            const int nvec = nvx * TY;
            for (int t = 0; t < T_steps && ok; ++t) {
                const int64_t qn = q0 + t + 2;
                int w = 0;
                if (t == 0) {
                    w = warp_wait(smem_u32(&full[q0 % S]), (uint32_t)((q0 / S) & 1), abort_flag);
                    if (!w) w = warp_wait(smem_u32(&full[(q0 + 1) % S]), (uint32_t)(((q0 + 1) / S) & 1), abort_flag);
                }
                if (!w) w = warp_wait(smem_u32(&full[qn % S]), (uint32_t)((qn / S) & 1), abort_flag);
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                const int z = za + t;
                const unsigned char *sz = smem + ((q0 + t + 1) % S) * K::SLOT;
                const C *Cm = reinterpret_cast<const C *>(smem + ((q0 + t) % S) * K::SLOT);
                const C *Cz = reinterpret_cast<const C *>(sz);
                const C *Cp = reinterpret_cast<const C *>(smem + (qn % S) * K::SLOT);
                const C *Lh = reinterpret_cast<const C *>(sz + K::C_BYTES);
                const C *Rh = reinterpret_cast<const C *>(sz + K::C_BYTES + K::H_PAD);
                const C *Ph = reinterpret_cast<const C *>(sz + K::P_OFF);
#pragma unroll
                for (int j = 0; j < K::MAXV; ++j) {
                    const int v = cid + j * K::NC;
                    if (v >= nvec) continue;
                    const int yy = v / nvx, xx = (v % nvx) * K::VS;
                    const int r = (1 + yy) * tx + xx;
                    C ctr[K::VS], up[K::VS], dn[K::VS], zm[K::VS], zp[K::VS];
                    *reinterpret_cast<V *>(ctr) = *reinterpret_cast<const V *>(&Cz[r]);
                    *reinterpret_cast<V *>(up) = *reinterpret_cast<const V *>(&Cz[r - tx]);
                    *reinterpret_cast<V *>(dn) = *reinterpret_cast<const V *>(&Cz[r + tx]);
                    *reinterpret_cast<V *>(zm) = *reinterpret_cast<const V *>(&Cm[r]);
                    *reinterpret_cast<V *>(zp) = *reinterpret_cast<const V *>(&Cp[r]);
                    C left, right;
                    if (xx > 0) left = Cz[r - 1];
                    else left = xhalo ? Lh[yy * K::VS + K::VS - 1] : Cz[(1 + yy) * tx + tx - 1];
                    if (xx + K::VS < tx) right = Cz[r + K::VS];
                    else right = xhalo ? Rh[yy * K::VS] : Cz[(1 + yy) * tx];
                    T pv[2 * K::VS];
                    *reinterpret_cast<V *>(pv) = *reinterpret_cast<const V *>(&Ph[yy * tx + xx]);
                    C outv[K::VS];
#pragma unroll
                    for (int jj = 0; jj < K::VS; ++jj) {
                        const C xm = (jj == 0) ? left : ctr[jj - 1];
                        const C xp = (jj == K::VS - 1) ? right : ctr[jj + 1];
                        if constexpr (sizeof(T) == 8) {   // FP64: the centre weight folded (site_update_fold)
                            const T S1 = nsum7<T>(xm.x, xp.x, up[jj].x, dn[jj].x, zm[jj].x, zp[jj].x);
                            const T S2 = nsum7<T>(xm.y, xp.y, up[jj].y, dn[jj].y, zm[jj].y, zp[jj].y);
                            site_update_fold<T>(ctr[jj].x, ctr[jj].y, S1, S2, pv[2 * jj], pv[2 * jj + 1], outv[jj].x,
                                                outv[jj].y, cf, cf.kdt_idx2 * (T)-6);
                        } else {
                            const T L1 = lap7<T>(ctr[jj].x, xm.x, xp.x, up[jj].x, dn[jj].x, zm[jj].x, zp[jj].x);
                            const T L2 = lap7<T>(ctr[jj].y, xm.y, xp.y, up[jj].y, dn[jj].y, zm[jj].y, zp[jj].y);
                            site_update<T>(ctr[jj].x, ctr[jj].y, L1, L2, pv[2 * jj], pv[2 * jj + 1], outv[jj].x,
                                           outv[jj].y, cf);
                        }
                    }
                    const int64_t off = ((int64_t)z * N + (y0 + yy)) * N + (x0 + xx);
                    *reinterpret_cast<V *>(&pih[off]) = *reinterpret_cast<V *>(pv);
                    *reinterpret_cast<V *>(&psi_out[off]) = *reinterpret_cast<V *>(outv);
                }
                // this warp is done with plane z-1 (load q0+t); at the last step
                // also with the item's last two planes
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&empty[(q0 + t) % S]));
                    if (t == T_steps - 1) {
                        mbar_arrive(smem_u32(&empty[(q0 + T_steps) % S]));
                        mbar_arrive(smem_u32(&empty[(q0 + T_steps + 1) % S]));
                    }
                }
            }
            if (!ok) break;
            q0 += T_steps + 2;
        }
    }
    __syncwarp();      // reconverge every warp (the producer's lane 0 ran alone) before the barrier
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&counters[1], 1) == (int)gridDim.x - 1) {
            counters[0] = 0;
            counters[1] = 0;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// Two steps per pass (temporal blocking with halo depth 2), complex float.
//
// One pass reads psi_n and pih_{n-1} and writes psi_{n+2} and pih_{n+1}: 32
// bytes per site for two site-updates instead of 64. A work item is an x-y
// tile of tx * TY sites marched through a z-chunk, as in k_zmarch2:
//  * the producer warp loads, per plane, psi_n over the tile plus a two-site
//    periodic halo (rows y0-2 .. y0+TY+1 as three row bands, two-site x strips
//    on both sides) and pih_{n-1} over the tile plus a one-site halo (rows
//    y0-1 .. y0+TY, and the x strips): up to 14 TMA boxes, none of which wraps;
//  * stage 1 (consumer warps) takes step n on plane m over the tile and its
//    one-site ring without the corners (the sites that the 7-point stencil of
//    stage 2 reads) and puts psi_{n+1} of the plane into a two-plane ring;
//  * stage 2 takes step n+1 on plane m-1 over the tile, from psi_{n+1} of
//    planes m-2, m-1, m and pih_n of plane m-1 (registers) and the in-plane
//    neighbours (shared memory), and stores psi_{n+2} and pih_{n+1}.
// Each consumer thread owns fixed 2-site vectors of the tile (and of the
// ring), so the z-neighbours of both stages stay in registers. Both stages call
// site_update / lap7 with the coefficients of a one-step launch at tau and
// tau + dt, so one pass of two steps and two passes of one step give the same
// bits. pih is read from pih[bin] and written to pih[bin ^ 1], which must be
// different buffers: a neighbouring tile may already have stored pih_{n+1}
// where this tile still reads pih_{n-1} in its halo.

template <int TY, int TXMAX, int S, int NCW, int MIDN = 2>
struct Z3Cfg {
    static constexpr int CS = 8;                                  // bytes per complex float site
    static constexpr int NC = NCW * 32;                           // consumer threads
    static constexpr int NT = NC + 32;
    static constexpr int NVX = TXMAX / 2;                         // 2-site vectors per row
    static constexpr int MAXV = (TY * NVX + NC - 1) / NC;         // tile vectors per thread
    static constexpr int MAXR = (2 * NVX + NC - 1) / NC;          // ring-row vectors per thread
    static constexpr int ST_M = (TY * 16 + 127) / 128 * 128;
    static constexpr int STRIP = 128 + ST_M + 128;                // psi x strip: rows 0-1 | 2..TY+1 | TY+2..TY+3
    static constexpr int PB = (TY + 4) * TXMAX * CS;              // psi_n band, rows y0-2 .. y0+TY+1
    static constexpr int SL_OFF = PB, SR_OFF = PB + STRIP;
    static constexpr int QB_OFF = PB + 2 * STRIP;                 // pih band, rows y0-1 .. y0+TY
    static constexpr int QL_OFF = QB_OFF + (TY + 2) * TXMAX * CS; // pih x strips, rows y0 .. y0+TY-1
    static constexpr int QR_OFF = QL_OFF + ST_M;
    static constexpr int SLOT = QR_OFF + ST_M;
    static constexpr int MB = (TY + 2) * TXMAX * CS;              // psi_{n+1} band, rows y0-1 .. y0+TY
    static constexpr int MID = (MB + 2 * TY * CS + 127) / 128 * 128;   // + columns x0-1 and x0+tx
    static constexpr int MID_OFF = S * SLOT;
    static constexpr int BAR_OFF = MID_OFF + MIDN * MID;          // MIDN planes of the psi_{n+1} ring
    static constexpr int SMEM = BAR_OFF + 256;
};

// Byte offset of row r (0 .. TY+3 for y0-2 .. y0+TY+1) within a psi x strip
// (two sites per row; rows 0-1, 2..TY+1 and TY+2..TY+3 are separate boxes).
template <int TY, int ST_M>
__device__ __forceinline__ int strip_off(int r) {
    return r < 2 ? r * 16 : (r < TY + 2 ? 128 + (r - 2) * 16 : 128 + ST_M + (r - TY - 2) * 16);
}

__device__ __forceinline__ float4 ldb4(const unsigned char *base, int off) {
    return *reinterpret_cast<const float4 *>(base + off);
}
__device__ __forceinline__ float2 ldb2(const unsigned char *base, int off) {
    return *reinterpret_cast<const float2 *>(base + off);
}
// (Streaming stores, st.global.cs, measured 0.25 % slower at 1024^3.)
__device__ __forceinline__ void st4(float2 *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }

// One step of the two sites (c.xy, c.zw); same operations as k_zmarch2.
__device__ __forceinline__ float4 update_vec2(float4 c, float4 zm, float4 zp, float4 up, float4 dn, float2 left,
                                              float2 right, float4 &p, const StepCoefs<float> &cf) {
    float4 o;
    float L1 = lap7<float>(c.x, left.x, c.z, up.x, dn.x, zm.x, zp.x);
    float L2 = lap7<float>(c.y, left.y, c.w, up.y, dn.y, zm.y, zp.y);
    site_update<float>(c.x, c.y, L1, L2, p.x, p.y, o.x, o.y, cf);
    L1 = lap7<float>(c.z, c.x, right.x, up.z, dn.z, zm.z, zp.z);
    L2 = lap7<float>(c.w, c.y, right.y, up.w, dn.w, zm.w, zp.w);
    site_update<float>(c.z, c.w, L1, L2, p.z, p.w, o.z, o.w, cf);
    return o;
}
__device__ __forceinline__ float2 update_site(float2 c, float2 xm, float2 xp, float2 ym, float2 yp, float2 zm,
                                              float2 zp, float2 &p, const StepCoefs<float> &cf) {
    float2 o;
    const float L1 = lap7<float>(c.x, xm.x, xp.x, ym.x, yp.x, zm.x, zp.x);
    const float L2 = lap7<float>(c.y, xm.y, xp.y, ym.y, yp.y, zm.y, zp.y);
    site_update<float>(c.x, c.y, L1, L2, p.x, p.y, o.x, o.y, cf);
    return o;
}

// The x neighbours of a thread's two-site vector are 8-byte loads 16 bytes
// apart across the lanes: left neighbours touch only the banks 2, 3 mod 4 and
// right neighbours only 0, 1 mod 4, so each load takes twice the wavefronts it
// needs. Lanes 8-15 of each half-warp therefore load their right neighbour in
// the first of the two loads and their left one in the second (offsets
// swapped once per work item), which spreads both loads over all 32 banks;
// the values are put back in place with selects.
__device__ __forceinline__ bool swap_lane() { return (threadIdx.x & 8) != 0; }
__device__ __forceinline__ void x_neighbours(const unsigned char *base, int oa, int ob, bool sw, float2 &left,
                                             float2 &right) {
    const float2 a = ldb2(base, oa), b = ldb2(base, ob);
    left = sw ? b : a;
    right = sw ? a : b;
}

// LEAN: the centre psi_n of the in-plane slot and psi_{n+1} of planes m-1 and
// m-2 are read back from shared memory (a three-plane psi_{n+1} ring) instead
// of being carried in registers, so the thread fits 128 registers and three
// CTAs share an SM (12 consumer warps instead of 8). Same arithmetic, same bits.
template <int TY, int TXMAX, int S, int NCW, int UNR, bool LEAN>
__device__ __forceinline__ void zmarch_2step_body(const ZLat *__restrict__ lats, int nlat, int64_t total_items,
                                                  int *counters, int parity, int *derr) {
    typedef Z3Cfg<TY, TXMAX, S, NCW, LEAN ? 3 : 2> K;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + K::BAR_OFF);
    uint64_t *empty = full + S;
    uint64_t *ifull = empty + S;                                 // [2]
    uint64_t *iempty = ifull + 2;                                // [2]
    uint64_t *midbar = iempty + 2;                               // consumer barrier of the psi_{n+1} ring
    volatile int64_t *items = reinterpret_cast<volatile int64_t *>(midbar + 1);   // [2]
    volatile int *abort_flag = reinterpret_cast<volatile int *>(items + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), NCW);
        }
        for (int k = 0; k < 2; ++k) {
            mbar_init(smem_u32(&ifull[k]), 1);
            mbar_init(smem_u32(&iempty[k]), NCW);
        }
        mbar_init(smem_u32(midbar), NCW);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int64_t q = 0;
            bool ok = true;
            for (int64_t k = 0; ok; ++k) {
                if (k >= 2) ok = mbar_wait_bounded(smem_u32(&iempty[k & 1]), (uint32_t)(((k >> 1) - 1) & 1));
                if (!ok || *abort_flag) break;
                const int64_t item = (int64_t)atomicAdd(&counters[0], 1);
                items[k & 1] = item;
                mbar_arrive(smem_u32(&ifull[k & 1]));
                if (item >= total_items) break;
                const int li = find_lat(lats, nlat, item);
                const ZLat &Lt = lats[li];
                const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
                const int64_t local = item - Lt.item_base;
                const int ncols = ntx * nty;
                const int zq = (int)(local / ncols), col = (int)(local % ncols);
                const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
                const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
                const int nload = zb - za + 4;
                const int bin = Lt.a_index ^ parity;
                const bool xhalo = tx < N;
                const uint32_t psi_bytes = (uint32_t)((TY + 4) * tx * K::CS + (xhalo ? 2 * (TY + 4) * 16 : 0));
                const uint32_t pih_bytes = (uint32_t)((TY + 2) * tx * K::CS + (xhalo ? 2 * TY * 16 : 0));
                const int ym2 = y0 >= 2 ? y0 - 2 : y0 - 2 + N;
                const int ym1 = y0 >= 1 ? y0 - 1 : N - 1;
                const int yp = (y0 + TY == N) ? 0 : y0 + TY;
                const int xl = x0 >= 2 ? x0 - 2 : x0 - 2 + N;
                const int xr = (x0 + tx == N) ? 0 : x0 + tx;
                for (int i = 0; i < nload; ++i, ++q) {
                    const int s = (int)(q % S);
                    if (q >= S) {
                        ok = mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)(((q / S) - 1) & 1));
                        if (!ok || *abort_flag) break;
                    }
                    int z = za - 2 + i;
                    z = z < 0 ? z + N : (z >= N ? z - N : z);
                    unsigned char *slot = smem + s * K::SLOT;
                    const uint32_t bar = smem_u32(&full[s]);
                    const bool with_pih = i >= 1 && i <= nload - 2;
                    mbar_expect_tx(bar, psi_bytes + (with_pih ? pih_bytes : 0u) +
                                            (i == 0 ? (uint32_t)Lt.debug_tx_excess : 0u));
                    tma_load_3d(smem_u32(slot), &Lt.t2_row2[bin], x0, ym2, z, bar);
                    tma_load_3d(smem_u32(slot + 2 * tx * K::CS), &Lt.tm_main[bin], x0, y0, z, bar);
                    tma_load_3d(smem_u32(slot + (TY + 2) * tx * K::CS), &Lt.t2_row2[bin], x0, yp, z, bar);
                    if (xhalo) {
                        tma_load_3d(smem_u32(slot + K::SL_OFF), &Lt.t2_str2[bin], xl, ym2, z, bar);
                        tma_load_3d(smem_u32(slot + K::SL_OFF + 128), &Lt.tm_xh[bin], xl, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::SL_OFF + 128 + K::ST_M), &Lt.t2_str2[bin], xl, yp, z, bar);
                        tma_load_3d(smem_u32(slot + K::SR_OFF), &Lt.t2_str2[bin], xr, ym2, z, bar);
                        tma_load_3d(smem_u32(slot + K::SR_OFF + 128), &Lt.tm_xh[bin], xr, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::SR_OFF + 128 + K::ST_M), &Lt.t2_str2[bin], xr, yp, z, bar);
                    }
                    if (with_pih) {
                        tma_load_3d(smem_u32(slot + K::QB_OFF), &Lt.t2_prow[bin], x0, ym1, z, bar);
                        tma_load_3d(smem_u32(slot + K::QB_OFF + tx * K::CS), &Lt.tm_pih[bin], x0, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::QB_OFF + (TY + 1) * tx * K::CS), &Lt.t2_prow[bin], x0, yp, z,
                                    bar);
                        if (xhalo) {
                            tma_load_3d(smem_u32(slot + K::QL_OFF), &Lt.t2_pstr[bin], xl, y0, z, bar);
                            tma_load_3d(smem_u32(slot + K::QR_OFF), &Lt.t2_pstr[bin], xr, y0, z, bar);
                        }
                    }
                }
            }
            if (!ok) {
                atomicOr(derr, DEVERR_TIMEOUT);
                *abort_flag = 1;
            }
            // Drain: wait (bounded) for this CTA's last loads still in flight.
            for (int64_t d = q > S ? q - S : 0; d < q; ++d)
                mbar_wait_bounded(smem_u32(&full[d % S]), (uint32_t)((d / S) & 1));
        }
    } else {
        // ------------------------------------------------------------ consumers
        // Every shared-memory and global offset a thread touches depends only
        // on the item's tile, so it is computed once per item; the plane loop
        // holds loads, arithmetic and stores.
        const int cid = tid;   // 0 .. NC-1
        int64_t q0 = 0;        // loads of the items before the current one
        int64_t g = 0;         // iterations done (completed phases of midbar)
        int gm = 0;            // g mod 3 (LEAN: plane of the psi_{n+1} ring written next)
        for (int64_t k = 0;; ++k) {
            int w = warp_wait(smem_u32(&ifull[k & 1]), (uint32_t)((k >> 1) & 1), abort_flag);
            if (w) {
                if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                break;
            }
            const int64_t item = items[k & 1];
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&iempty[k & 1]));
            if (item >= total_items) break;
            const int li = find_lat(lats, nlat, item);
            const ZLat &Lt = lats[li];
            const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
            const int64_t local = item - Lt.item_base;
            const int ncols = ntx * nty;
            const int zq = (int)(local / ncols), col = (int)(local % ncols);
            const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
            const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
            const int T_steps = zb - za;
            const int bin = Lt.a_index ^ parity;
            float2 *psi_out = reinterpret_cast<float2 *>(Lt.psi[bin ^ 1]);
            float2 *pih_out = reinterpret_cast<float2 *>(Lt.pih[bin ^ 1]);
            const double tau = Lt.clock[bin];
            const double tau1 = tau + Lt.dt;
            const StepCoefs<float> cf1 = make_coefs<float>(tau, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            const StepCoefs<float> cf2 = make_coefs<float>(tau1, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            if (local == 0 && cid == 0) Lt.clock[bin ^ 1] = tau1 + Lt.dt;   // tau += dt twice, s_integrate.cpp:317
            const bool xhalo = tx < N;
            const int nvx = tx / 2;
            const int nvec = nvx * TY, nring = 2 * nvx;
            const int txb = tx * K::CS;   // bytes per band row
            const int64_t NN = (int64_t)N * N;

            // Tile vectors: byte offsets of the centre, left and right neighbours
            // in an input slot (psi_n band rows y0-2 .. : centre row 2+yy; the
            // pih band starts one row later) and in a psi_{n+1} plane (row 1+yy),
            // and the global site offset at plane za. With sw, the left and
            // right offsets are stored swapped (x_neighbours puts them back).
            const bool sw = swap_lane();
            int t_c[K::MAXV], t_l[K::MAXV], t_r[K::MAXV], m_l[K::MAXV], m_r[K::MAXV];
            int64_t g_off[K::MAXV];
#pragma unroll
            for (int j = 0; j < K::MAXV; ++j) {
                const int v = cid + j * K::NC;
                const int yy = v < nvec ? v / nvx : 0, xx = v < nvec ? (v % nvx) * 2 : 0;
                const int rowb = (2 + yy) * txb, mrow = (1 + yy) * txb;
                t_c[j] = rowb + xx * K::CS;
                t_l[j] = xx > 0 ? t_c[j] - K::CS
                                : (xhalo ? K::SL_OFF + strip_off<TY, K::ST_M>(2 + yy) + K::CS : rowb + (tx - 1) * K::CS);
                t_r[j] = xx + 2 < tx ? t_c[j] + 2 * K::CS : (xhalo ? K::SR_OFF + strip_off<TY, K::ST_M>(2 + yy) : rowb);
                m_l[j] = xx > 0 ? mrow + (xx - 1) * K::CS : (xhalo ? K::MB + yy * K::CS : mrow + (tx - 1) * K::CS);
                m_r[j] = xx + 2 < tx ? mrow + (xx + 2) * K::CS : (xhalo ? K::MB + (TY + yy) * K::CS : mrow);
                g_off[j] = (int64_t)za * NN + (int64_t)(y0 + yy) * N + (x0 + xx);
                if (sw) {   // first load: the right neighbour (see x_neighbours)
                    const int a = t_l[j], b = m_l[j];
                    t_l[j] = t_r[j]; t_r[j] = a;
                    m_l[j] = m_r[j]; m_r[j] = b;
                }
            }
            // Ring-row vectors (rows y0-1 and y0+TY: band rows 1 and TY+2).
            int r_c[K::MAXR], r_l[K::MAXR], r_r[K::MAXR];
#pragma unroll
            for (int j = 0; j < K::MAXR; ++j) {
                const int u = cid + j * K::NC;
                const int br = (u < nring && u >= nvx) ? TY + 2 : 1;
                const int xx = u < nring ? (u % nvx) * 2 : 0;
                const int rowb = br * txb;
                r_c[j] = rowb + xx * K::CS;
                r_l[j] = xx > 0 ? r_c[j] - K::CS
                                : (xhalo ? K::SL_OFF + strip_off<TY, K::ST_M>(br) + K::CS : rowb + (tx - 1) * K::CS);
                r_r[j] = xx + 2 < tx ? r_c[j] + 2 * K::CS : (xhalo ? K::SR_OFF + strip_off<TY, K::ST_M>(br) : rowb);
                if (sw) {
                    const int a = r_l[j];
                    r_l[j] = r_r[j]; r_r[j] = a;
                }
            }
            // Ring-column site: x0-1 (column 1 of the left strips) or x0+tx
            // (column 0 of the right strips), row y0+cyy; it goes to the
            // threads after the ring-row vectors.
            const int ccol = xhalo ? (cid + K::NC - nring % K::NC) % K::NC : K::NC;
            const bool has_col = ccol < 2 * TY;
            int c_z = 0, c_xm = 0, c_xp = 0, c_ym = 0, c_yp = 0, c_q = 0, c_m = 0;
            if (has_col) {
                const int cside = ccol / TY, cyy = ccol % TY, r = 2 + cyy;
                const int so = cside ? K::SR_OFF : K::SL_OFF;
                const int own = cside ? 0 : K::CS;   // the site's byte within a two-site strip row
                c_z = so + strip_off<TY, K::ST_M>(r) + own;
                c_ym = so + strip_off<TY, K::ST_M>(r - 1) + own;
                c_yp = so + strip_off<TY, K::ST_M>(r + 1) + own;
                c_xm = cside ? r * txb + (tx - 1) * K::CS : so + strip_off<TY, K::ST_M>(r);
                c_xp = cside ? so + strip_off<TY, K::ST_M>(r) + K::CS : r * txb;
                c_q = (cside ? K::QR_OFF : K::QL_OFF) + cyy * 16 + own;
                c_m = K::MB + (cside * TY + cyy) * K::CS;
            }

            float4 a_zm[K::MAXV], a_c[K::MAXV];    // psi_n of planes m-1, m
            float4 b_m2[K::MAXV], b_m1[K::MAXV];   // psi_{n+1} of planes m-2, m-1
            float4 p_m1[K::MAXV];                  // pih_n of plane m-1
            float4 r_zm[K::MAXR], r_cv[K::MAXR];   // ring rows: psi_n of planes m-1, m
            float2 c_zm = make_float2(0.f, 0.f), c_cv = c_zm;   // ring column site
            const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < K::MAXV; ++j) { a_zm[j] = a_c[j] = b_m2[j] = b_m1[j] = p_m1[j] = zero4; }
#pragma unroll
            for (int j = 0; j < K::MAXR; ++j) { r_zm[j] = r_cv[j] = zero4; }

            // load q sits in slot q % S and completes phase (q / S) & 1 of full[slot]
            int s0 = (int)(q0 % S);
            uint32_t ph0 = (uint32_t)((q0 / S) & 1);
            int s1 = s0 + 1;
            uint32_t ph1 = ph0;
            if (s1 == S) { s1 = 0; ph1 ^= 1u; }
            // planes za-2 and za-1 (loads 0 and 1) prime the registers
            w = warp_wait(smem_u32(&full[s0]), ph0, abort_flag);
            if (!w) w = warp_wait(smem_u32(&full[s1]), ph1, abort_flag);
            if (w) {
                if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                break;
            }
            {
                const unsigned char *B0 = smem + s0 * K::SLOT, *B1 = smem + s1 * K::SLOT;
#pragma unroll
                for (int j = 0; j < K::MAXV; ++j)
                    if (cid + j * K::NC < nvec) {
                        a_zm[j] = ldb4(B0, t_c[j]);
                        if constexpr (!LEAN) a_c[j] = ldb4(B1, t_c[j]);
                    }
#pragma unroll
                for (int j = 0; j < K::MAXR; ++j)
                    if (cid + j * K::NC < nring) {
                        r_zm[j] = ldb4(B0, r_c[j]);
                        if constexpr (!LEAN) r_cv[j] = ldb4(B1, r_c[j]);
                    }
                if (has_col) {
                    c_zm = ldb2(B0, c_z);
                    if constexpr (!LEAN) c_cv = ldb2(B1, c_z);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&empty[s0]));

            // stage 1 of iteration i: in-plane from load i+1 (slot sc), zp from load i+2 (slot sn)
            int sc = s1, sn = s1 + 1;
            uint32_t phn = ph1;
            if (sn == S) { sn = 0; phn ^= 1u; }
            bool ok = true;
            // unrolling lets the compiler rename the rotating register planes
#pragma unroll UNR
            for (int i = 0; i <= T_steps + 1; ++i) {
                w = warp_wait(smem_u32(&full[sn]), phn, abort_flag);
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                const unsigned char *Sc = smem + sc * K::SLOT, *Sn = smem + sn * K::SLOT;
                // psi_{n+1} ring: plane m is written, m-1 (and in LEAN mode m-2) read
                const int gw = LEAN ? gm : (int)(g & 1);
                unsigned char *Mw = smem + K::MID_OFF + gw * K::MID;
                float4 b_new[K::MAXV], p_new[K::MAXV];
#pragma unroll
                for (int j = 0; j < K::MAXV; ++j) {
                    b_new[j] = p_new[j] = zero4;
                    if (cid + j * K::NC >= nvec) continue;
                    const float4 zp = ldb4(Sn, t_c[j]);
                    const float4 ac = LEAN ? ldb4(Sc, t_c[j]) : a_c[j];
                    const float4 up = ldb4(Sc, t_c[j] - txb), dn = ldb4(Sc, t_c[j] + txb);
                    float4 p = ldb4(Sc, K::QB_OFF + t_c[j] - txb);
                    float2 xl, xr;
                    x_neighbours(Sc, t_l[j], t_r[j], sw, xl, xr);
                    const float4 o = update_vec2(ac, a_zm[j], zp, up, dn, xl, xr, p, cf1);
                    *reinterpret_cast<float4 *>(Mw + t_c[j] - txb) = o;
                    b_new[j] = o;
                    p_new[j] = p;
                    a_zm[j] = ac;
                    if constexpr (!LEAN) a_c[j] = zp;
                }
#pragma unroll
                for (int j = 0; j < K::MAXR; ++j) {
                    if (cid + j * K::NC >= nring) continue;
                    const float4 zp = ldb4(Sn, r_c[j]);
                    const float4 rc = LEAN ? ldb4(Sc, r_c[j]) : r_cv[j];
                    const float4 up = ldb4(Sc, r_c[j] - txb), dn = ldb4(Sc, r_c[j] + txb);
                    float4 p = ldb4(Sc, K::QB_OFF + r_c[j] - txb);
                    float2 xl, xr;
                    x_neighbours(Sc, r_l[j], r_r[j], sw, xl, xr);
                    const float4 o = update_vec2(rc, r_zm[j], zp, up, dn, xl, xr, p, cf1);
                    *reinterpret_cast<float4 *>(Mw + r_c[j] - txb) = o;
                    r_zm[j] = rc;
                    if constexpr (!LEAN) r_cv[j] = zp;
                }
                if (has_col) {
                    const float2 zp = ldb2(Sn, c_z);
                    const float2 cc = LEAN ? ldb2(Sc, c_z) : c_cv;
                    float2 p = ldb2(Sc, c_q);
                    *reinterpret_cast<float2 *>(Mw + c_m) = update_site(cc, ldb2(Sc, c_xm), ldb2(Sc, c_xp), ldb2(Sc, c_ym),
                                                                        ldb2(Sc, c_yp), c_zm, zp, p, cf1);
                    c_zm = cc;
                    if constexpr (!LEAN) c_cv = zp;
                }
                // this warp is done with load i+1; at the last plane also with load i+2
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&empty[sc]));
                    if (i == T_steps + 1) mbar_arrive(smem_u32(&empty[sn]));
                }
                // stage 2 on plane m-1 = za-2+i (the planes za .. zb-1)
                if (i >= 2) {
                    const int gr = LEAN ? (gm == 0 ? 2 : gm - 1) : (int)((g - 1) & 1);   // plane m-1
                    const unsigned char *Mr = smem + K::MID_OFF + gr * K::MID;
                    const unsigned char *Mrr = smem + K::MID_OFF + (gr == 0 ? 2 : gr - 1) * K::MID;   // m-2 (LEAN)
#pragma unroll
                    for (int j = 0; j < K::MAXV; ++j) {
                        if (cid + j * K::NC >= nvec) continue;
                        const int mc = t_c[j] - txb;
                        const float4 up = ldb4(Mr, mc - txb), dn = ldb4(Mr, mc + txb);
                        const float4 bc = LEAN ? ldb4(Mr, mc) : b_m1[j], bz = LEAN ? ldb4(Mrr, mc) : b_m2[j];
                        float4 p = p_m1[j];
                        float2 xl, xr;
                        x_neighbours(Mr, m_l[j], m_r[j], sw, xl, xr);
                        const float4 o = update_vec2(bc, bz, b_new[j], up, dn, xl, xr, p, cf2);
                        st4(&pih_out[g_off[j]], p);
                        st4(&psi_out[g_off[j]], o);
                        g_off[j] += NN;
                    }
                }
#pragma unroll
                for (int j = 0; j < K::MAXV; ++j) {
                    if constexpr (!LEAN) {
                        b_m2[j] = b_m1[j];
                        b_m1[j] = b_new[j];
                    }
                    p_m1[j] = p_new[j];
                }
                // plane m of the psi_{n+1} ring is complete before anyone reads it;
                // plane m-1 is no longer read when the next stage 1 overwrites it
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(midbar));
                w = warp_wait(smem_u32(midbar), (uint32_t)(g & 1), abort_flag);
                ++g;
                gm = gm == 2 ? 0 : gm + 1;
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                sc = sn;
                if (++sn == S) { sn = 0; phn ^= 1u; }
            }
            if (!ok) break;
            q0 += T_steps + 4;
        }
    }
    __syncwarp();      // reconverge every warp (the producer's lane 0 ran alone) before the barrier
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&counters[1], 1) == (int)gridDim.x - 1) {
            counters[0] = 0;
            counters[1] = 0;
            __threadfence();
        }
    }
}

template <int TY, int TXMAX, int S, int NCW, int UNR>
__global__ void __launch_bounds__(Z3Cfg<TY, TXMAX, S, NCW>::NT)
    k_zmarch_2step(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity, int *derr) {
    zmarch_2step_body<TY, TXMAX, S, NCW, UNR, false>(lats, nlat, total_items, counters, parity, derr);
}
// Register cap for LEAN_CTAS resident CTAs of NCW + 1 warps: each of the four
// SM sub-partitions holds 16K registers and a quarter of the warps (rounded
// up), allocated in steps of 8 registers per thread.
template <int NCW, int LEAN_CTAS>
struct LeanRegs {
    static constexpr int WARPS = (LEAN_CTAS * (NCW + 1) + 3) / 4;
    static constexpr int R = 16384 / (32 * WARPS) / 8 * 8;
    static constexpr int VALUE = R > 255 ? 255 : R;
};
// five CTAs of three warps or three of five: 128 registers (one vector per
// thread with eight consumer warps, 96 registers, measured slower)
template <int NCW> struct LeanCtas { static constexpr int VALUE = NCW <= 2 ? 5 : 3; };
template <int TY, int TXMAX, int S, int NCW>
__global__ void __maxnreg__((LeanRegs<NCW, LeanCtas<NCW>::VALUE>::VALUE))
    k_zmarch_2step_lean(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity,
                        int *derr) {
    zmarch_2step_body<TY, TXMAX, S, NCW, 1, true>(lats, nlat, total_items, counters, parity, derr);
}
template <int TY, int TXMAX, int S, int NCW, int UNR, bool LEAN>
static void (*zm3_kernel())(const ZLat *, int, int64_t, int *, int, int *) {
    if constexpr (LEAN) return k_zmarch_2step_lean<TY, TXMAX, S, NCW>;
    else return k_zmarch_2step<TY, TXMAX, S, NCW, UNR>;
}

// ============================================================== three steps per pass
//
// Three leapfrog steps per pass (halo depth 3), complex float, x-tiled
// lattices (tx < N). A work item is a tx x TY tile marching a z-chunk, as in
// the two-step kernel. Per plane m:
//  stage 1: psi_{n+1}, pih_{n+1} at plane m over the tile, the two rows above
//           and the two below it (tile width), and the 2-site side vectors
//           [x0-2, x0-1], [x0+tx, x0+tx+1] of rows y0-1 .. y0+TY, from psi_n
//           of planes m-1, m, m+1 (a band of rows y0-3 .. y0+TY+2 and 4-site
//           x strips of rows y0-2 .. y0+TY+1) and pih_n; psi_{n+1} goes into a
//           three-plane ring;
//  stage 2: psi_{n+2}, pih_{n+2} at plane m-1 over the tile, the rows y0-1 and
//           y0+TY and the sites x0-1, x0+tx of the tile rows, psi_{n+2} into a
//           second three-plane ring;
//  stage 3: psi_{n+3}, pih_{n+3} of the tile at plane m-2, to global memory.
// A thread computes the same sites in every stage it takes part in: the z+1
// neighbour of stages 2 and 3 (written by the stage before in the same
// iteration) and the momentum handed from stage to stage stay in its
// registers, and the rings are read only at planes finished in earlier
// iterations, so one barrier per plane suffices, as in the two-step kernel.
// Centres and z-1 planes are read back from the rings (the two-step kernel's
// LEAN form). DRAM: 32 B per site per pass, 10.7 B per site-update.
template <int TY, int TXMAX, int S, int NCW>
struct Z5Cfg {
    static constexpr int CS = 8;                                   // bytes per complex float site
    static constexpr int NC = NCW * 32;                            // consumer threads
    static constexpr int NT = NC + 32;
    static constexpr int NVX = TXMAX / 2;                          // 2-site vectors per row
    static constexpr int MAXT = (TY * NVX + NC - 1) / NC;          // tile vectors per thread
    static constexpr int MAXE = (4 * NVX + 2 * (TY + 2) + NC - 1) / NC;   // other stage-1 vectors per thread
    // input slot
    static constexpr int PB = (TY + 6) * TXMAX * CS;               // psi_n band, rows y0-3 .. y0+TY+2
    static constexpr int SMID = (TY * 32 + 127) / 128 * 128;
    static constexpr int STRIP = 128 + SMID + 128;                 // 4-site psi strip: rows 0-1 | 2..TY+1 | TY+2..TY+3
    static constexpr int SL_OFF = PB, SR_OFF = PB + STRIP;
    static constexpr int QB_OFF = PB + 2 * STRIP;                  // pih_n band, rows y0-2 .. y0+TY+1
    static constexpr int QMID = (TY * 16 + 127) / 128 * 128;
    static constexpr int PSTRIP = 128 + QMID + 128;                // 2-site pih strip: row 0 | 1..TY | TY+1
    static constexpr int QL_OFF = QB_OFF + (TY + 4) * TXMAX * CS;
    static constexpr int QR_OFF = QL_OFF + PSTRIP;
    static constexpr int SLOT = QR_OFF + PSTRIP;
    // psi_{n+1} ring plane: band rows y0-2 .. y0+TY+1, then the left and the
    // right side vectors of rows y0-1 .. y0+TY
    static constexpr int M1B = (TY + 4) * TXMAX * CS;
    static constexpr int M1 = (M1B + 2 * (TY + 2) * 16 + 127) / 128 * 128;
    // psi_{n+2} ring plane: band rows y0-1 .. y0+TY, then the sites x0-1 and
    // x0+tx of the tile rows
    static constexpr int M2B = (TY + 2) * TXMAX * CS;
    static constexpr int M2 = (M2B + 2 * TY * CS + 127) / 128 * 128;
    static constexpr int M1_OFF = S * SLOT;
    static constexpr int M2_OFF = M1_OFF + 3 * M1;
    static constexpr int BAR_OFF = M2_OFF + 3 * M2;
    static constexpr int SMEM = BAR_OFF + 256;
};

// Byte offset of row r within a 4-site psi strip (r = 0 .. TY+3 for rows
// y0-2 .. y0+TY+1; the boxes of rows 0-1, 2..TY+1 and TY+2..TY+3 start on
// 128 bytes) and within a 2-site pih strip (r = 0 .. TY+1 for y0-1 .. y0+TY).
template <int TY, int SMID>
__device__ __forceinline__ int strip4_off(int r) {
    return r < 2 ? r * 32 : (r < TY + 2 ? 128 + (r - 2) * 32 : 128 + SMID + (r - TY - 2) * 32);
}
template <int TY, int QMID>
__device__ __forceinline__ int pstrip_off(int r) {
    return r < 1 ? 0 : (r < TY + 1 ? 128 + (r - 1) * 16 : 128 + QMID);
}

__device__ __forceinline__ void dswap(int &a, int &b) {
    const int t = a;
    a = b;
    b = t;
}

template <int TY, int TXMAX, int S, int NCW>
__device__ __forceinline__ void zmarch_3step_body(const ZLat *__restrict__ lats, int nlat, int64_t total_items,
                                                  int *counters, int parity, int *derr) {
    typedef Z5Cfg<TY, TXMAX, S, NCW> K;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + K::BAR_OFF);
    uint64_t *empty = full + S;
    uint64_t *ifull = empty + S;                                 // [2]
    uint64_t *iempty = ifull + 2;                                // [2]
    uint64_t *midbar = iempty + 2;                               // consumer barrier of the rings
    volatile int64_t *items = reinterpret_cast<volatile int64_t *>(midbar + 1);   // [2]
    volatile int *abort_flag = reinterpret_cast<volatile int *>(items + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), NCW);
        }
        for (int k = 0; k < 2; ++k) {
            mbar_init(smem_u32(&ifull[k]), 1);
            mbar_init(smem_u32(&iempty[k]), NCW);
        }
        mbar_init(smem_u32(midbar), NCW);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int64_t q = 0;
            bool ok = true;
            for (int64_t k = 0; ok; ++k) {
                if (k >= 2) ok = mbar_wait_bounded(smem_u32(&iempty[k & 1]), (uint32_t)(((k >> 1) - 1) & 1));
                if (!ok || *abort_flag) break;
                const int64_t item = (int64_t)atomicAdd(&counters[0], 1);
                items[k & 1] = item;
                mbar_arrive(smem_u32(&ifull[k & 1]));
                if (item >= total_items) break;
                const int li = find_lat(lats, nlat, item);
                const ZLat &Lt = lats[li];
                const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
                const int64_t local = item - Lt.item_base;
                const int ncols = ntx * nty;
                const int zq = (int)(local / ncols), col = (int)(local % ncols);
                const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
                const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
                const int nload = zb - za + 6;   // psi_n planes za-3 .. zb+2
                const int bin = Lt.a_index ^ parity;
                const uint32_t psi_bytes = (uint32_t)((TY + 6) * tx * K::CS + 2 * (TY + 4) * 32);
                const uint32_t pih_bytes = (uint32_t)((TY + 4) * tx * K::CS + 2 * (TY + 2) * 16);
                // halo rows and columns with the periodic wrap (x0, y0 are
                // multiples of tx, TY >= 3, so no box wraps inside itself;
                // every x coordinate is even: 16-byte aligned)
                const int ym3 = y0 >= 3 ? y0 - 3 : y0 - 3 + N;
                const int ym2 = y0 >= 2 ? y0 - 2 : y0 - 2 + N;
                const int ym1 = y0 >= 1 ? y0 - 1 : N - 1;
                const int yp = (y0 + TY == N) ? 0 : y0 + TY;
                const int xl4 = x0 >= 4 ? x0 - 4 : x0 - 4 + N;
                const int xl2 = x0 >= 2 ? x0 - 2 : x0 - 2 + N;
                const int xr = (x0 + tx == N) ? 0 : x0 + tx;
                for (int i = 0; i < nload; ++i, ++q) {
                    const int s = (int)(q % S);
                    if (q >= S) {
                        ok = mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)(((q / S) - 1) & 1));
                        if (!ok || *abort_flag) break;
                    }
                    int z = za - 3 + i;
                    z = z < 0 ? z + N : (z >= N ? z - N : z);
                    unsigned char *slot = smem + s * K::SLOT;
                    const uint32_t bar = smem_u32(&full[s]);
                    const bool with_pih = i >= 1 && i <= nload - 2;   // stage-1 planes za-2 .. zb+1
                    mbar_expect_tx(bar, psi_bytes + (with_pih ? pih_bytes : 0u) +
                                            (i == 0 ? (uint32_t)Lt.debug_tx_excess : 0u));
                    tma_load_3d(smem_u32(slot), &Lt.t3_row3[bin], x0, ym3, z, bar);
                    tma_load_3d(smem_u32(slot + 3 * tx * K::CS), &Lt.tm_main[bin], x0, y0, z, bar);
                    tma_load_3d(smem_u32(slot + (TY + 3) * tx * K::CS), &Lt.t3_row3[bin], x0, yp, z, bar);
                    tma_load_3d(smem_u32(slot + K::SL_OFF), &Lt.t3_str2[bin], xl4, ym2, z, bar);
                    tma_load_3d(smem_u32(slot + K::SL_OFF + 128), &Lt.t3_strm[bin], xl4, y0, z, bar);
                    tma_load_3d(smem_u32(slot + K::SL_OFF + 128 + K::SMID), &Lt.t3_str2[bin], xl4, yp, z, bar);
                    tma_load_3d(smem_u32(slot + K::SR_OFF), &Lt.t3_str2[bin], xr, ym2, z, bar);
                    tma_load_3d(smem_u32(slot + K::SR_OFF + 128), &Lt.t3_strm[bin], xr, y0, z, bar);
                    tma_load_3d(smem_u32(slot + K::SR_OFF + 128 + K::SMID), &Lt.t3_str2[bin], xr, yp, z, bar);
                    if (with_pih) {
                        tma_load_3d(smem_u32(slot + K::QB_OFF), &Lt.t3_prow2[bin], x0, ym2, z, bar);
                        tma_load_3d(smem_u32(slot + K::QB_OFF + 2 * tx * K::CS), &Lt.tm_pih[bin], x0, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::QB_OFF + (TY + 2) * tx * K::CS), &Lt.t3_prow2[bin], x0, yp, z,
                                    bar);
                        tma_load_3d(smem_u32(slot + K::QL_OFF), &Lt.t3_pst1[bin], xl2, ym1, z, bar);
                        tma_load_3d(smem_u32(slot + K::QL_OFF + 128), &Lt.t2_pstr[bin], xl2, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::QL_OFF + 128 + K::QMID), &Lt.t3_pst1[bin], xl2, yp, z, bar);
                        tma_load_3d(smem_u32(slot + K::QR_OFF), &Lt.t3_pst1[bin], xr, ym1, z, bar);
                        tma_load_3d(smem_u32(slot + K::QR_OFF + 128), &Lt.t2_pstr[bin], xr, y0, z, bar);
                        tma_load_3d(smem_u32(slot + K::QR_OFF + 128 + K::QMID), &Lt.t3_pst1[bin], xr, yp, z, bar);
                    }
                }
            }
            if (!ok) {
                atomicOr(derr, DEVERR_TIMEOUT);
                *abort_flag = 1;
            }
            // Drain: wait (bounded) for this CTA's last loads still in flight.
            for (int64_t d = q > S ? q - S : 0; d < q; ++d)
                mbar_wait_bounded(smem_u32(&full[d % S]), (uint32_t)((d / S) & 1));
        }
    } else {
        // ------------------------------------------------------------ consumers
        const int cid = tid;   // 0 .. NC-1
        int64_t q0 = 0;        // loads of the items before the current one
        int64_t g = 0;         // iterations done (completed phases of midbar)
        int gm = 0;            // g mod 3: the ring plane written next
        for (int64_t k = 0;; ++k) {
            int w = warp_wait(smem_u32(&ifull[k & 1]), (uint32_t)((k >> 1) & 1), abort_flag);
            if (w) {
                if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                break;
            }
            const int64_t item = items[k & 1];
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&iempty[k & 1]));
            if (item >= total_items) break;
            const int li = find_lat(lats, nlat, item);
            const ZLat &Lt = lats[li];
            const int N = Lt.N, tx = Lt.tx, ntx = Lt.ntx, nty = Lt.nty, nzc = Lt.nzc;
            const int64_t local = item - Lt.item_base;
            const int ncols = ntx * nty;
            const int zq = (int)(local / ncols), col = (int)(local % ncols);
            const int x0 = (col % ntx) * tx, y0 = (col / ntx) * TY;
            const int za = (int)((int64_t)zq * N / nzc), zb = (int)((int64_t)(zq + 1) * N / nzc);
            const int T_steps = zb - za;
            const int bin = Lt.a_index ^ parity;
            float2 *psi_out = reinterpret_cast<float2 *>(Lt.psi[bin ^ 1]);
            float2 *pih_out = reinterpret_cast<float2 *>(Lt.pih[bin ^ 1]);
            const double tau = Lt.clock[bin];
            const double tau1 = tau + Lt.dt, tau2 = tau1 + Lt.dt;
            const StepCoefs<float> cf1 = make_coefs<float>(tau, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            const StepCoefs<float> cf2 = make_coefs<float>(tau1, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            const StepCoefs<float> cf3 = make_coefs<float>(tau2, Lt.dt, Lt.dt, Lt.inv_dx2, Lt.lambda, Lt.T0sq3, Lt.prs, Lt.form);
            if (local == 0 && cid == 0) Lt.clock[bin ^ 1] = tau2 + Lt.dt;   // tau += dt three times, s_integrate.cpp:317
            const int nvx = tx / 2;
            const int nvec = nvx * TY;
            const int next = 4 * nvx + 2 * (TY + 2);
            const int txb = tx * K::CS;   // bytes per band row
            const int64_t NN = (int64_t)N * N;

            // Tile vectors: offsets in an input slot (psi_n band row 3+yy,
            // 4-site strip row 2+yy, pih_n band row 2+yy), in a psi_{n+1}
            // plane (band row 2+yy, side-vector row 1+yy), in a psi_{n+2}
            // plane (band row 1+yy, side sites of row yy), and the global
            // offset at plane za.
            int t_c[K::MAXT], t_l[K::MAXT], t_r[K::MAXT], t_q[K::MAXT];
            int u_c[K::MAXT], u_l[K::MAXT], u_r[K::MAXT];   // psi_{n+1} plane
            int w_c[K::MAXT], w_l[K::MAXT], w_r[K::MAXT];   // psi_{n+2} plane
            int64_t g_off[K::MAXT];
            // With sw, every vector's left and right x-neighbour offsets are
            // stored swapped (x_neighbours puts the values back): the loads of a
            // half-warp then cover all 32 banks.
            const bool sw = swap_lane();
#pragma unroll
            for (int j = 0; j < K::MAXT; ++j) {
                const int v = cid + j * K::NC;
                const int yy = v < nvec ? v / nvx : 0, xx = v < nvec ? (v % nvx) * 2 : 0;
                t_c[j] = (3 + yy) * txb + xx * K::CS;
                t_l[j] = xx > 0 ? t_c[j] - K::CS : K::SL_OFF + strip4_off<TY, K::SMID>(2 + yy) + 24;
                t_r[j] = xx + 2 < tx ? t_c[j] + 2 * K::CS : K::SR_OFF + strip4_off<TY, K::SMID>(2 + yy);
                t_q[j] = K::QB_OFF + (2 + yy) * txb + xx * K::CS;
                u_c[j] = (2 + yy) * txb + xx * K::CS;
                u_l[j] = xx > 0 ? u_c[j] - K::CS : K::M1B + (1 + yy) * 16 + 8;
                u_r[j] = xx + 2 < tx ? u_c[j] + 2 * K::CS : K::M1B + (TY + 2) * 16 + (1 + yy) * 16;
                w_c[j] = (1 + yy) * txb + xx * K::CS;
                w_l[j] = xx > 0 ? w_c[j] - K::CS : K::M2B + yy * K::CS;
                w_r[j] = xx + 2 < tx ? w_c[j] + 2 * K::CS : K::M2B + (TY + yy) * K::CS;
                g_off[j] = (int64_t)za * NN + (int64_t)(y0 + yy) * N + (x0 + xx);
                if (sw) {
                    dswap(t_l[j], t_r[j]);
                    dswap(u_l[j], u_r[j]);
                    dswap(w_l[j], w_r[j]);
                }
            }
            // Other stage-1 vectors: kind 0 the rows y0-1 and y0+TY (stages 1
            // and 2), kind 1 the rows y0-2 and y0+TY+1 (stage 1), kind 2 the
            // side vectors of rows y0-1 .. y0+TY (stage 1; stage 2 on the site
            // next to the tile, x0-1 or x0+tx, for the tile rows).
            int e_kind[K::MAXE], e_c[K::MAXE], e_l[K::MAXE], e_r[K::MAXE], e_u[K::MAXE], e_d[K::MAXE], e_q[K::MAXE];
            int e_m1[K::MAXE];                                            // psi_{n+1} offset (the vector)
            int f_c[K::MAXE], f_l[K::MAXE], f_r[K::MAXE], f_u[K::MAXE], f_d[K::MAXE], f_w[K::MAXE];   // stage 2
            bool e_s2[K::MAXE], e_hi[K::MAXE];   // takes part in stage 2; its stage-2 site is the vector's second
#pragma unroll
            for (int j = 0; j < K::MAXE; ++j) {
                const int u = cid + j * K::NC;
                e_kind[j] = -1;
                e_c[j] = e_l[j] = e_r[j] = e_u[j] = e_d[j] = e_q[j] = e_m1[j] = 0;
                f_c[j] = f_l[j] = f_r[j] = f_u[j] = f_d[j] = f_w[j] = 0;
                e_s2[j] = e_hi[j] = false;
                if (u >= next) continue;
                if (u < 4 * nvx) {
                    const bool outer = u >= 2 * nvx;
                    const int uu = outer ? u - 2 * nvx : u;
                    const bool below = uu >= nvx;
                    const int xx = (uu % nvx) * 2;
                    // rows: psi_n band b, strip s, pih band p, psi_{n+1} band m
                    const int b = outer ? (below ? TY + 4 : 1) : (below ? TY + 3 : 2);
                    const int s = b - 1, p = b - 1, m = b - 1;
                    e_kind[j] = outer ? 1 : 0;
                    e_c[j] = b * txb + xx * K::CS;
                    e_u[j] = e_c[j] - txb;
                    e_d[j] = e_c[j] + txb;
                    e_l[j] = xx > 0 ? e_c[j] - K::CS : K::SL_OFF + strip4_off<TY, K::SMID>(s) + 24;
                    e_r[j] = xx + 2 < tx ? e_c[j] + 2 * K::CS : K::SR_OFF + strip4_off<TY, K::SMID>(s);
                    e_q[j] = K::QB_OFF + p * txb + xx * K::CS;
                    e_m1[j] = m * txb + xx * K::CS;
                    if (!outer) {   // stage 2 on the same vector: psi_{n+1} row m, side-vector row m-1
                        e_s2[j] = true;
                        f_c[j] = e_m1[j];
                        f_u[j] = f_c[j] - txb;
                        f_d[j] = f_c[j] + txb;
                        f_l[j] = xx > 0 ? f_c[j] - K::CS : K::M1B + (m - 1) * 16 + 8;
                        f_r[j] = xx + 2 < tx ? f_c[j] + 2 * K::CS : K::M1B + (TY + 2) * 16 + (m - 1) * 16;
                        f_w[j] = (below ? TY + 1 : 0) * txb + xx * K::CS;
                    }
                } else {
                    const int kk = u - 4 * nvx;
                    const int side = kk / (TY + 2), r = kk % (TY + 2);   // row y0-1+r
                    const int so = side ? K::SR_OFF : K::SL_OFF;
                    const int vo = side ? 0 : 16;                        // the vector within the strip row
                    e_kind[j] = 2;
                    e_c[j] = so + strip4_off<TY, K::SMID>(r + 1) + vo;
                    e_u[j] = so + strip4_off<TY, K::SMID>(r) + vo;
                    e_d[j] = so + strip4_off<TY, K::SMID>(r + 2) + vo;
                    // x neighbours: left vector x0-3 (strip) and x0 (band);
                    // right vector x0+tx-1 (band) and x0+tx+2 (strip)
                    e_l[j] = side ? (r + 2) * txb + (tx - 1) * K::CS : so + strip4_off<TY, K::SMID>(r + 1) + 8;
                    e_r[j] = side ? so + strip4_off<TY, K::SMID>(r + 1) + 16 : (r + 2) * txb;
                    e_q[j] = (side ? K::QR_OFF : K::QL_OFF) + pstrip_off<TY, K::QMID>(r);
                    e_m1[j] = K::M1B + (side * (TY + 2) + r) * 16;
                    if (r >= 1 && r <= TY) {   // the site next to the tile, row y0-1+r of the tile rows
                        e_s2[j] = true;
                        e_hi[j] = side == 0;   // x0-1 is the left vector's second site, x0+tx the right's first
                        const int own = side ? 0 : 8;
                        f_c[j] = e_m1[j] + own;
                        f_u[j] = e_m1[j] - 16 + own;
                        f_d[j] = e_m1[j] + 16 + own;
                        f_l[j] = side ? (r + 1) * txb + (tx - 1) * K::CS : e_m1[j];
                        f_r[j] = side ? e_m1[j] + 8 : (r + 1) * txb;
                        f_w[j] = K::M2B + (side * TY + r - 1) * K::CS;
                    }
                }
                if (sw) {   // the vectors' x neighbours (a side vector's stage-2 site reads them plainly)
                    dswap(e_l[j], e_r[j]);
                    if (e_kind[j] == 0) dswap(f_l[j], f_r[j]);
                }
            }

            float4 a_zm[K::MAXT], e_zm[K::MAXE];   // psi_n of plane m-1 (stage 1's z-1 neighbour)
            float4 p1_t[K::MAXT], p1_e[K::MAXE];   // pih_{n+1} of plane m-1 (stage 2)
            float4 p2_t[K::MAXT];                  // pih_{n+2} of plane m-2 (stage 3)
            const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < K::MAXT; ++j) a_zm[j] = p1_t[j] = p2_t[j] = zero4;
#pragma unroll
            for (int j = 0; j < K::MAXE; ++j) e_zm[j] = p1_e[j] = zero4;

            // load q sits in slot q % S and completes phase (q / S) & 1 of full[slot]
            int s0 = (int)(q0 % S);
            uint32_t ph0 = (uint32_t)((q0 / S) & 1);
            int s1 = s0 + 1;
            uint32_t ph1 = ph0;
            if (s1 == S) { s1 = 0; ph1 ^= 1u; }
            // plane za-3 (load 0) primes the z-1 registers; load 1 is the first centre
            w = warp_wait(smem_u32(&full[s0]), ph0, abort_flag);
            if (!w) w = warp_wait(smem_u32(&full[s1]), ph1, abort_flag);
            if (w) {
                if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                break;
            }
            {
                const unsigned char *B0 = smem + s0 * K::SLOT;
#pragma unroll
                for (int j = 0; j < K::MAXT; ++j)
                    if (cid + j * K::NC < nvec) a_zm[j] = ldb4(B0, t_c[j]);
#pragma unroll
                for (int j = 0; j < K::MAXE; ++j)
                    if (e_kind[j] >= 0) e_zm[j] = ldb4(B0, e_c[j]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&empty[s0]));

            int sc = s1, sn = s1 + 1;
            uint32_t phn = ph1;
            if (sn == S) { sn = 0; phn ^= 1u; }
            bool ok = true;
            for (int i = 0; i <= T_steps + 3; ++i) {
                w = warp_wait(smem_u32(&full[sn]), phn, abort_flag);
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                const unsigned char *Sc = smem + sc * K::SLOT, *Sn = smem + sn * K::SLOT;
                const int g1 = gm, g0 = gm == 0 ? 2 : gm - 1, gz = g0 == 0 ? 2 : g0 - 1;   // planes m, m-1, m-2 of a ring
                unsigned char *R1w = smem + K::M1_OFF + g1 * K::M1;
                const unsigned char *R1c = smem + K::M1_OFF + g0 * K::M1, *R1z = smem + K::M1_OFF + gz * K::M1;
                unsigned char *R2w = smem + K::M2_OFF + g1 * K::M2;
                const unsigned char *R2c = smem + K::M2_OFF + g0 * K::M2, *R2z = smem + K::M2_OFF + gz * K::M2;
                // ---- stage 1 at plane m (load i+1), z+1 from load i+2
                float4 b1_t[K::MAXT], q1_t[K::MAXT], b1_e[K::MAXE], q1_e[K::MAXE];
#pragma unroll
                for (int j = 0; j < K::MAXT; ++j) {
                    b1_t[j] = q1_t[j] = zero4;
                    if (cid + j * K::NC >= nvec) continue;
                    const float4 ac = ldb4(Sc, t_c[j]);
                    float4 p = ldb4(Sc, t_q[j]);
                    float2 xl, xr;
                    x_neighbours(Sc, t_l[j], t_r[j], sw, xl, xr);
                    const float4 o = update_vec2(ac, a_zm[j], ldb4(Sn, t_c[j]), ldb4(Sc, t_c[j] - txb),
                                                 ldb4(Sc, t_c[j] + txb), xl, xr, p, cf1);
                    *reinterpret_cast<float4 *>(R1w + u_c[j]) = o;
                    b1_t[j] = o;
                    q1_t[j] = p;
                    a_zm[j] = ac;
                }
#pragma unroll
                for (int j = 0; j < K::MAXE; ++j) {
                    b1_e[j] = q1_e[j] = zero4;
                    if (e_kind[j] < 0) continue;
                    const float4 ac = ldb4(Sc, e_c[j]);
                    float4 p = ldb4(Sc, e_q[j]);
                    float2 xl, xr;
                    x_neighbours(Sc, e_l[j], e_r[j], sw, xl, xr);
                    const float4 o = update_vec2(ac, e_zm[j], ldb4(Sn, e_c[j]), ldb4(Sc, e_u[j]), ldb4(Sc, e_d[j]),
                                                 xl, xr, p, cf1);
                    *reinterpret_cast<float4 *>(R1w + e_m1[j]) = o;
                    b1_e[j] = o;
                    q1_e[j] = p;
                    e_zm[j] = ac;
                }
                // this warp is done with load i+1; at the last plane also with load i+2
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&empty[sc]));
                    if (i == T_steps + 3) mbar_arrive(smem_u32(&empty[sn]));
                }
                // ---- stage 2 at plane m-1 (planes za-1 .. zb)
                float4 b2_t[K::MAXT], q2_t[K::MAXT];
#pragma unroll
                for (int j = 0; j < K::MAXT; ++j) b2_t[j] = q2_t[j] = zero4;
                if (i >= 2) {
#pragma unroll
                    for (int j = 0; j < K::MAXT; ++j) {
                        if (cid + j * K::NC >= nvec) continue;
                        float4 p = p1_t[j];
                        float2 xl, xr;
                        x_neighbours(R1c, u_l[j], u_r[j], sw, xl, xr);
                        const float4 o = update_vec2(ldb4(R1c, u_c[j]), ldb4(R1z, u_c[j]), b1_t[j], ldb4(R1c, u_c[j] - txb),
                                                     ldb4(R1c, u_c[j] + txb), xl, xr, p, cf2);
                        *reinterpret_cast<float4 *>(R2w + w_c[j]) = o;
                        b2_t[j] = o;
                        q2_t[j] = p;
                    }
#pragma unroll
                    for (int j = 0; j < K::MAXE; ++j) {
                        if (!e_s2[j]) continue;
                        if (e_kind[j] == 0) {
                            float4 p = p1_e[j];
                            float2 xl, xr;
                            x_neighbours(R1c, f_l[j], f_r[j], sw, xl, xr);
                            const float4 o = update_vec2(ldb4(R1c, f_c[j]), ldb4(R1z, f_c[j]), b1_e[j], ldb4(R1c, f_u[j]),
                                                         ldb4(R1c, f_d[j]), xl, xr, p, cf2);
                            *reinterpret_cast<float4 *>(R2w + f_w[j]) = o;
                        } else {   // one site of a side vector
                            const bool hi = e_hi[j];
                            float2 p = hi ? make_float2(p1_e[j].z, p1_e[j].w) : make_float2(p1_e[j].x, p1_e[j].y);
                            const float2 zp = hi ? make_float2(b1_e[j].z, b1_e[j].w) : make_float2(b1_e[j].x, b1_e[j].y);
                            *reinterpret_cast<float2 *>(R2w + f_w[j]) =
                                update_site(ldb2(R1c, f_c[j]), ldb2(R1c, f_l[j]), ldb2(R1c, f_r[j]), ldb2(R1c, f_u[j]),
                                            ldb2(R1c, f_d[j]), ldb2(R1z, f_c[j]), zp, p, cf2);
                        }
                    }
                }
                // ---- stage 3 at plane m-2 (planes za .. zb-1)
                if (i >= 4) {
#pragma unroll
                    for (int j = 0; j < K::MAXT; ++j) {
                        if (cid + j * K::NC >= nvec) continue;
                        float4 p = p2_t[j];
                        float2 xl, xr;
                        x_neighbours(R2c, w_l[j], w_r[j], sw, xl, xr);
                        const float4 o = update_vec2(ldb4(R2c, w_c[j]), ldb4(R2z, w_c[j]), b2_t[j], ldb4(R2c, w_c[j] - txb),
                                                     ldb4(R2c, w_c[j] + txb), xl, xr, p, cf3);
                        st4(&pih_out[g_off[j]], p);
                        st4(&psi_out[g_off[j]], o);
                        g_off[j] += NN;
                    }
                }
                // the momentum moves one stage on
#pragma unroll
                for (int j = 0; j < K::MAXT; ++j) {
                    p2_t[j] = q2_t[j];
                    p1_t[j] = q1_t[j];
                }
#pragma unroll
                for (int j = 0; j < K::MAXE; ++j) p1_e[j] = q1_e[j];
                // plane m of ring 1 and plane m-1 of ring 2 are complete before
                // anyone reads them; the planes the next iteration overwrites are
                // no longer read
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(midbar));
                w = warp_wait(smem_u32(midbar), (uint32_t)(g & 1), abort_flag);
                ++g;
                gm = gm == 2 ? 0 : gm + 1;
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                sc = sn;
                if (++sn == S) { sn = 0; phn ^= 1u; }
            }
            if (!ok) break;
            q0 += T_steps + 6;
        }
    }
    __syncwarp();      // reconverge every warp (the producer's lane 0 ran alone) before the barrier
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&counters[1], 1) == (int)gridDim.x - 1) {
            counters[0] = 0;
            counters[1] = 0;
            __threadfence();
        }
    }
}

// Two CTAs of NCW + 1 warps per SM (registers per thread as LeanRegs counts
// them: each SM sub-partition holds 16K registers for a quarter of the warps).
template <int TY, int TXMAX, int S, int NCW>
__global__ void __maxnreg__((LeanRegs<NCW, 2>::VALUE))
    k_zmarch_3step(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity, int *derr) {
    zmarch_3step_body<TY, TXMAX, S, NCW>(lats, nlat, total_items, counters, parity, derr);
}

// ============================================================== host side

int current_device() {
    int dev = 0;
    AXS_CUDA(cudaGetDevice(&dev));
    return dev;
}

int num_sms() {
    static PerDevice sms;
    return sms.get([] {
        int n = 0;
        AXS_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, current_device()));
        return n;
    });
}

static int grid_for(int64_t len, int threads = 256) {
    int64_t want = (len + threads - 1) / threads;
    int64_t cap = (int64_t)num_sms() * 16;
    return (int)std::max<int64_t>(1, std::min(want, cap));
}

// ---- z-march variants -------------------------------------------------------
// gen 1: k_zmarch (CTA barriers); gen 2: k_zmarch2 (producer warp); gen 3:
// k_zmarch_2step (two steps per pass, complex float), whose odd last step of an
// interval runs on the gen-2 `partner` with the same tile and launch table.
// gen 4: k_zmarch2r (stencil radius r = 2..4, axs_step_r.cu). gen 5:
// k_zmarch_3step (three steps per pass), whose last one or two steps of an
// interval run on its gen-3 `partner` (same tile, same launch table). `lean`:
// gen 3, the lean two-step form; gen 4, the register z-ring with a ring of
// 2R + 2 or more slots (fewer slots always use it).
struct ZVariant {
    int gen, ty, txmax, slots, ncw, partner, r, lean;
};
static const ZVariant kZVariants[] = {
    {1, 8, 128, 4, 0, -1}, {1, 8, 128, 5, 0, -1}, {1, 16, 128, 4, 0, -1}, {1, 4, 256, 4, 0, -1},
    {1, 8, 256, 4, 0, -1}, {2, 8, 128, 4, 8, -1}, {2, 8, 128, 5, 8, -1}, {2, 4, 256, 5, 8, -1},
    {2, 8, 256, 5, 8, -1}, {2, 4, 128, 6, 8, -1}, {3, 8, 128, 4, 8, 6},  {3, 8, 128, 5, 8, 6},
    {3, 4, 256, 4, 8, 7},  {3, 8, 128, 4, 8, 6},  {3, 8, 128, 4, 8, 6},  {3, 8, 128, 5, 8, 6},
    {2, 8, 64, 5, 8, -1},  {3, 8, 64, 4, 4, 16},  {3, 8, 64, 5, 4, 16},  {3, 4, 128, 5, 4, 9},
    {4, 8, 128, 6, 8, -1, 2},  {4, 4, 128, 6, 8, -1, 2},  {4, 8, 64, 8, 8, -1, 3},  {4, 4, 128, 8, 8, -1, 3},
    {4, 4, 128, 10, 8, -1, 4}, {4, 8, 64, 10, 8, -1, 4},  {4, 4, 64, 10, 8, -1, 4},
    // 27-29: 32-wide tiles with two consumer warps (up to 4 CTAs per SM); 32
    // divides every N that is a multiple of 32, so ensembles of mixed sizes
    // keep every tile full
    {2, 8, 32, 5, 8, -1},  {3, 8, 32, 4, 2, 27},  {3, 8, 32, 5, 2, 27},
    // 30-31: LEAN two-step (centre values re-read from shared memory, 128
    // registers, one more CTA per SM)
    {3, 8, 64, 4, 4, 16, 0, 1},  {3, 8, 32, 4, 2, 27, 0, 1},
    // 32-37: radius 2-4 with the z-neighbours in registers (R + 2 slots, float)
    {4, 4, 128, 4, 8, -1, 2},  {4, 8, 64, 4, 8, -1, 2},  {4, 4, 128, 5, 8, -1, 3},  {4, 8, 64, 5, 8, -1, 3},
    {4, 4, 128, 6, 8, -1, 4},  {4, 8, 64, 6, 8, -1, 4},
    // 38: one-step 32x16 tiles (the partner of 39-40); 39-40: LEAN two-step on
    // 32x16 tiles with four consumer warps, three CTAs per SM: the y halo is
    // 4 rows per 16 instead of per 8, and 32 divides every ensemble size
    {2, 16, 32, 5, 8, -1},  {3, 16, 32, 4, 4, 38, 0, 1},  {3, 16, 32, 5, 4, 38, 0, 1},
    // 41: radius 2 with the shared z-ring on 16 x 64 tiles (4 halo rows per 16
    // instead of per 4 or 8; 6.25 against 6.79 ms/step for variant 21 at 1024^3;
    // 8 x 64 tiles measured 7.07)
    {4, 16, 64, 6, 8, -1, 2},
    // 42-45: the z-neighbours in registers with deeper rings: a register ring
    // holds the R + 1 planes still to be centres, so S = R + 2 keeps one plane
    // load in flight per CTA; these keep three (radius 2: two), at two CTAs per SM
    {4, 4, 128, 7, 8, -1, 3},  {4, 8, 64, 7, 8, -1, 3},  {4, 8, 64, 8, 8, -1, 4},  {4, 4, 128, 5, 8, -1, 2},
    // 46-47: three steps per pass (halo depth 3) on 8 x 64 and 16 x 32 tiles, two
    // CTAs of eight consumer warps per SM; an interval's last one or two steps
    // run on the two-step partner (variant 30 or 39) and its one-step partner
    {5, 8, 64, 4, 8, 30, 0, 1},  {5, 16, 32, 4, 8, 39, 0, 1},
    // 48-49: radius 2 with the z-neighbours in registers and rings of 6 and 7
    // slots (three and four plane loads in flight per CTA; the last field,
    // set, keeps the register ring although S >= 2R + 2)
    {4, 4, 128, 6, 8, -1, 2, 1},  {4, 4, 128, 7, 8, -1, 2, 1},
    // 50-55: the same deeper register rings where the slots fit two CTAs per
    // SM: radius 2 on 4 x 128 (8 slots), radius 3 on 8 x 64 (8, 9) and 16 x 32
    // (10), radius 4 on 16 x 32 (9, 10)
    {4, 4, 128, 8, 8, -1, 2, 1},  {4, 8, 64, 8, 8, -1, 3, 1},  {4, 8, 64, 9, 8, -1, 3, 1},
    {4, 16, 32, 10, 8, -1, 3, 1}, {4, 16, 32, 9, 8, -1, 4, 0}, {4, 16, 32, 10, 8, -1, 4, 1},
    // 56-57: radius 4 on 8 x 64 with 9 slots, radius 2 on 4 x 128 with 9 (at
    // the shared-memory limit of two CTAs per SM)
    {4, 8, 64, 9, 8, -1, 4, 0},   {4, 4, 128, 9, 8, -1, 2, 1},
};
static const int kNumZVariants = sizeof(kZVariants) / sizeof(kZVariants[0]);

static bool two_step(int variant) { return variant >= 0 && variant < kNumZVariants && kZVariants[variant].gen == 3; }
static bool three_step(int variant) { return variant >= 0 && variant < kNumZVariants && kZVariants[variant].gen == 5; }
// the momentum is written out of place (pih and scratch exchange after every launch)
static bool out_of_place(int variant) { return two_step(variant) || three_step(variant); }
static int steps_per_pass(int variant) { return three_step(variant) ? 3 : (two_step(variant) ? 2 : 1); }
static int radius(const ZVariant &v) { return v.r > 0 ? v.r : 1; }

std::string StepConfig::describe() const {
    char b[200];
    if (kind == 0) snprintf(b, sizeof b, "generic per-site kernel");
    else if (two_step(variant))
        snprintf(b, sizeof b, "TMA z-march variant %d (two steps per pass, halo depth 2%s; odd step on variant %d), tx=%d, zchunk=%d",
                 variant, kZVariants[variant].lean ? ", lean" : "", kZVariants[variant].partner, tx, zchunk);
    else if (three_step(variant))
        snprintf(b, sizeof b, "TMA z-march variant %d (three steps per pass, halo depth 3; last steps on variant %d), tx=%d, zchunk=%d",
                 variant, kZVariants[variant].partner, tx, zchunk);
    else if (variant >= 0 && variant < kNumZVariants && kZVariants[variant].gen == 4)
        snprintf(b, sizeof b, "TMA z-march variant %d (stencil radius %d), tx=%d, zchunk=%d", variant,
                 kZVariants[variant].r, tx, zchunk);
    else snprintf(b, sizeof b, "TMA z-march variant %d, tx=%d, zchunk=%d", variant, tx, zchunk);
    return b;
}

// Sets the kernel's shared-memory attribute and caches its occupancy. Called
// when a launch table is built, never inside a graph capture.
template <typename T, int TY, int TXMAX, int S>
static int prepare_zmarch_t() {
    typedef ZCfg<T, TY, TXMAX, S> K;
    static PerDevice occ;   // the attribute and occupancy belong to the device
    return occ.get([] {
        AXS_CUDA(cudaFuncSetAttribute(k_zmarch<T, TY, TXMAX, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM));
        int o = 0;
        AXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_zmarch<T, TY, TXMAX, S>, K::NT, K::SMEM));
        if (o < 1) fail(AXS_ERR_CUDA, "z-march kernel does not fit on an SM");
        return o;
    });
}

template <typename T, int TY, int TXMAX, int S>
static void launch_zmarch_t(const ZLat *d, int nlat, int64_t items, int *counters, int parity, int *derr,
                            cudaStream_t st, int ctas_per_sm) {
    typedef ZCfg<T, TY, TXMAX, S> K;
    int occ = prepare_zmarch_t<T, TY, TXMAX, S>();
    int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    int64_t grid = std::min<int64_t>((int64_t)per * num_sms(), items);
    k_zmarch<T, TY, TXMAX, S><<<(int)grid, K::NT, K::SMEM, st>>>(d, nlat, items, counters, parity, derr);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

template <typename T, int TY, int TXMAX, int S>
static int prepare_zmarch2_t() {
    typedef Z2Cfg<T, TY, TXMAX, S> K;
    static PerDevice occ;   // the attribute and occupancy belong to the device
    return occ.get([] {
        AXS_CUDA(cudaFuncSetAttribute(k_zmarch2<T, TY, TXMAX, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM));
        int o = 0;
        AXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_zmarch2<T, TY, TXMAX, S>, K::NT, K::SMEM));
        if (o < 1) fail(AXS_ERR_CUDA, "z-march kernel does not fit on an SM");
        return o;
    });
}

template <typename T, int TY, int TXMAX, int S>
static void launch_zmarch2_t(const ZLat *d, int nlat, int64_t items, int *counters, int parity, int *derr,
                             cudaStream_t st, int ctas_per_sm) {
    typedef Z2Cfg<T, TY, TXMAX, S> K;
    int occ = prepare_zmarch2_t<T, TY, TXMAX, S>();
    int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    int64_t grid = std::min<int64_t>((int64_t)per * num_sms(), items);
    k_zmarch2<T, TY, TXMAX, S><<<(int)grid, K::NT, K::SMEM, st>>>(d, nlat, items, counters, parity, derr);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

template <int TY, int TXMAX, int S, int NCW, int UNR, bool LEAN>
static int prepare_zmarch3_t() {
    typedef Z3Cfg<TY, TXMAX, S, NCW, LEAN ? 3 : 2> K;
    static PerDevice occ;   // the attribute and occupancy belong to the device
    return occ.get([] {
        const auto kern = zm3_kernel<TY, TXMAX, S, NCW, UNR, LEAN>();
        AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM));
        int o = 0;
        AXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, K::NT, K::SMEM));
        if (o < 1) {
            cudaFuncAttributes fa;
            AXS_CUDA(cudaFuncGetAttributes(&fa, kern));
            fail(AXS_ERR_CUDA,
                 "two-step z-march kernel <%d,%d,%d,%d,%d,%d> does not fit on an SM (%d threads x %d registers, "
                 "%d B dynamic shared memory of %d allowed, %d B static, max %d threads per block)",
                 TY, TXMAX, S, NCW, UNR, (int)LEAN, K::NT, fa.numRegs, K::SMEM, fa.maxDynamicSharedSizeBytes,
                 (int)fa.sharedSizeBytes, fa.maxThreadsPerBlock);
        }
        return o;
    });
}

template <int TY, int TXMAX, int S, int NCW, int UNR, bool LEAN>
static void launch_zmarch3_t(const ZLat *d, int nlat, int64_t items, int *counters, int parity, int *derr,
                             cudaStream_t st, int ctas_per_sm) {
    typedef Z3Cfg<TY, TXMAX, S, NCW, LEAN ? 3 : 2> K;
    int occ = prepare_zmarch3_t<TY, TXMAX, S, NCW, UNR, LEAN>();
    int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    int64_t grid = std::min<int64_t>((int64_t)per * num_sms(), items);
    zm3_kernel<TY, TXMAX, S, NCW, UNR, LEAN>()<<<(int)grid, K::NT, K::SMEM, st>>>(d, nlat, items, counters, parity, derr);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

template <int TY, int TXMAX, int S, int NCW>
static int prepare_zmarch5_t() {
    typedef Z5Cfg<TY, TXMAX, S, NCW> K;
    static PerDevice occ;   // the attribute and occupancy belong to the device
    return occ.get([] {
        const auto kern = k_zmarch_3step<TY, TXMAX, S, NCW>;
        AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM));
        int o = 0;
        AXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, K::NT, K::SMEM));
        if (o < 1) {
            cudaFuncAttributes fa;
            AXS_CUDA(cudaFuncGetAttributes(&fa, kern));
            fail(AXS_ERR_CUDA,
                 "three-step z-march kernel <%d,%d,%d,%d> does not fit on an SM (%d threads x %d registers, "
                 "%d B dynamic shared memory of %d allowed, %d B static, max %d threads per block)",
                 TY, TXMAX, S, NCW, K::NT, fa.numRegs, K::SMEM, fa.maxDynamicSharedSizeBytes, (int)fa.sharedSizeBytes,
                 fa.maxThreadsPerBlock);
        }
        return o;
    });
}

template <int TY, int TXMAX, int S, int NCW>
static void launch_zmarch5_t(const ZLat *d, int nlat, int64_t items, int *counters, int parity, int *derr,
                             cudaStream_t st, int ctas_per_sm) {
    typedef Z5Cfg<TY, TXMAX, S, NCW> K;
    int occ = prepare_zmarch5_t<TY, TXMAX, S, NCW>();
    int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    int64_t grid = std::min<int64_t>((int64_t)per * num_sms(), items);
    k_zmarch_3step<TY, TXMAX, S, NCW><<<(int)grid, K::NT, K::SMEM, st>>>(d, nlat, items, counters, parity, derr);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

static void launch_zmarch(int esz, int variant, const ZLat *d, int nlat, int64_t items, int *counters, int parity,
                          int *derr, cudaStream_t st, int ctas_per_sm) {
    if (variant >= 0 && variant < kNumZVariants && kZVariants[variant].gen == 4) {
        const ZVariant &v = kZVariants[variant];
        launch_zmarch_r(esz, v.ty, v.txmax, v.slots, v.r, v.lean, d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        return;
    }
#define AXS_ZV(I, TY, TX, S)                                                                                    \
    case I:                                                                                                     \
        if (esz == 4) launch_zmarch_t<float, TY, TX, S>(d, nlat, items, counters, parity, derr, st, ctas_per_sm); \
        else launch_zmarch_t<double, TY, TX, S>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);         \
        break;
#define AXS_ZV2(I, TY, TX, S)                                                                                    \
    case I:                                                                                                      \
        if (esz == 4) launch_zmarch2_t<float, TY, TX, S>(d, nlat, items, counters, parity, derr, st, ctas_per_sm); \
        else launch_zmarch2_t<double, TY, TX, S>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);         \
        break;
#define AXS_ZV3(I, TY, TX, S, W, U)                                                                       \
    case I:                                                                                               \
        if (esz != 4) fail(AXS_ERR_ARG, "two-step z-march variant %d needs complex float fields", variant); \
        launch_zmarch3_t<TY, TX, S, W, U, false>(d, nlat, items, counters, parity, derr, st, ctas_per_sm); \
        break;
    switch (variant) {
        AXS_ZV(0, 8, 128, 4)
        AXS_ZV(1, 8, 128, 5)
        AXS_ZV(2, 16, 128, 4)
        AXS_ZV(3, 4, 256, 4)
        AXS_ZV(4, 8, 256, 4)
        AXS_ZV2(5, 8, 128, 4)
        AXS_ZV2(6, 8, 128, 5)
        AXS_ZV2(7, 4, 256, 5)
        AXS_ZV2(8, 8, 256, 5)
        AXS_ZV2(9, 4, 128, 6)
        AXS_ZV3(10, 8, 128, 4, 8, 1)
        AXS_ZV3(11, 8, 128, 5, 8, 1)
        AXS_ZV3(12, 4, 256, 4, 8, 1)
        AXS_ZV3(13, 8, 128, 4, 8, 2)
        AXS_ZV3(14, 8, 128, 4, 8, 3)
        AXS_ZV3(15, 8, 128, 5, 8, 6)
        AXS_ZV2(16, 8, 64, 5)
        AXS_ZV3(17, 8, 64, 4, 4, 1)
        AXS_ZV3(18, 8, 64, 5, 4, 1)
        AXS_ZV3(19, 4, 128, 5, 4, 1)
        AXS_ZV2(27, 8, 32, 5)
        AXS_ZV3(28, 8, 32, 4, 2, 1)
        AXS_ZV3(29, 8, 32, 5, 2, 1)
    case 30:
        if (esz != 4) fail(AXS_ERR_ARG, "two-step z-march variant %d needs complex float fields", variant);
        launch_zmarch3_t<8, 64, 4, 4, 1, true>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;
    case 31:
        if (esz != 4) fail(AXS_ERR_ARG, "two-step z-march variant %d needs complex float fields", variant);
        launch_zmarch3_t<8, 32, 4, 2, 1, true>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;
        AXS_ZV2(38, 16, 32, 5)
    case 39:
        if (esz != 4) fail(AXS_ERR_ARG, "two-step z-march variant %d needs complex float fields", variant);
        launch_zmarch3_t<16, 32, 4, 4, 1, true>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;
    case 40:
        if (esz != 4) fail(AXS_ERR_ARG, "two-step z-march variant %d needs complex float fields", variant);
        launch_zmarch3_t<16, 32, 5, 4, 1, true>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;
    case 46:
        if (esz != 4) fail(AXS_ERR_ARG, "three-step z-march variant %d needs complex float fields", variant);
        launch_zmarch5_t<8, 64, 4, 8>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;
    case 47:
        if (esz != 4) fail(AXS_ERR_ARG, "three-step z-march variant %d needs complex float fields", variant);
        launch_zmarch5_t<16, 32, 4, 8>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);
        break;

    default: fail(AXS_ERR_ARG, "bad z-march variant %d", variant);
    }
#undef AXS_ZV
#undef AXS_ZV2
#undef AXS_ZV3
}

static void prepare_zmarch(int esz, int variant) {
    if (variant >= 0 && variant < kNumZVariants && kZVariants[variant].gen == 4) {
        const ZVariant &v = kZVariants[variant];
        prepare_zmarch_r(esz, v.ty, v.txmax, v.slots, v.r, v.lean);
        return;
    }
#define AXS_ZP(I, TY, TX, S)                                      \
    case I:                                                       \
        if (esz == 4) prepare_zmarch_t<float, TY, TX, S>();       \
        else prepare_zmarch_t<double, TY, TX, S>();               \
        break;
#define AXS_ZP2(I, TY, TX, S)                                     \
    case I:                                                       \
        if (esz == 4) prepare_zmarch2_t<float, TY, TX, S>();      \
        else prepare_zmarch2_t<double, TY, TX, S>();              \
        break;
#define AXS_ZP3(I, TY, TX, S, W, U)                               \
    case I:                                                       \
        if (esz == 4) prepare_zmarch3_t<TY, TX, S, W, U, false>(); \
        break;
    switch (variant) {
        AXS_ZP(0, 8, 128, 4)
        AXS_ZP(1, 8, 128, 5)
        AXS_ZP(2, 16, 128, 4)
        AXS_ZP(3, 4, 256, 4)
        AXS_ZP(4, 8, 256, 4)
        AXS_ZP2(5, 8, 128, 4)
        AXS_ZP2(6, 8, 128, 5)
        AXS_ZP2(7, 4, 256, 5)
        AXS_ZP2(8, 8, 256, 5)
        AXS_ZP2(9, 4, 128, 6)
        AXS_ZP3(10, 8, 128, 4, 8, 1)
        AXS_ZP3(11, 8, 128, 5, 8, 1)
        AXS_ZP3(12, 4, 256, 4, 8, 1)
        AXS_ZP3(13, 8, 128, 4, 8, 2)
        AXS_ZP3(14, 8, 128, 4, 8, 3)
        AXS_ZP3(15, 8, 128, 5, 8, 6)
        AXS_ZP2(16, 8, 64, 5)
        AXS_ZP3(17, 8, 64, 4, 4, 1)
        AXS_ZP3(18, 8, 64, 5, 4, 1)
        AXS_ZP3(19, 4, 128, 5, 4, 1)
        AXS_ZP2(27, 8, 32, 5)
        AXS_ZP3(28, 8, 32, 4, 2, 1)
        AXS_ZP3(29, 8, 32, 5, 2, 1)
    case 30:
        if (esz == 4) prepare_zmarch3_t<8, 64, 4, 4, 1, true>();
        break;
    case 31:
        if (esz == 4) prepare_zmarch3_t<8, 32, 4, 2, 1, true>();
        break;
        AXS_ZP2(38, 16, 32, 5)
    case 39:
        if (esz == 4) prepare_zmarch3_t<16, 32, 4, 4, 1, true>();
        break;
    case 40:
        if (esz == 4) prepare_zmarch3_t<16, 32, 5, 4, 1, true>();
        break;
    case 46:
        if (esz == 4) prepare_zmarch5_t<8, 64, 4, 8>();
        break;
    case 47:
        if (esz == 4) prepare_zmarch5_t<16, 32, 4, 8>();
        break;

    default: fail(AXS_ERR_ARG, "bad z-march variant %d", variant);
    }
    if (kZVariants[variant].gen == 3 || kZVariants[variant].gen == 5) prepare_zmarch(esz, kZVariants[variant].partner);
#undef AXS_ZP
#undef AXS_ZP2
#undef AXS_ZP3
}

// Dynamic shared memory of a variant (mirrors ZCfg / Z2Cfg).
// Whether the variant's kernels (and a two-step variant's partner) can be
// made resident on this device: the tuner skips a candidate that cannot
// instead of failing the whole call.
static bool variant_resident(int esz, int variant) {
    try {
        prepare_zmarch(esz, variant);
        return true;
    } catch (const Error &) {
        cudaGetLastError();   // a refused attribute or occupancy query leaves no sticky state
        clear_last_error();
        return false;
    }
}

static int variant_smem(const ZVariant &v, int esz) {
    int cs = 2 * esz;
    if (v.gen == 4) {   // mirrors ZRCfg
        int vs = 16 / cs, rp = (v.r + vs - 1) / vs * vs;
        int c = (v.ty + 2 * v.r) * v.txmax * cs, h = (v.ty * rp * cs + 127) / 128 * 128;
        return v.slots * ((c + 2 * h + v.ty * v.txmax * cs + 127) / 128 * 128) + 256;
    }
    if (v.gen == 5) {   // mirrors Z5Cfg
        int smid = (v.ty * 32 + 127) / 128 * 128, qmid = (v.ty * 16 + 127) / 128 * 128;
        int slot = (v.ty + 6) * v.txmax * cs + 2 * (256 + smid) + (v.ty + 4) * v.txmax * cs + 2 * (256 + qmid);
        int m1 = ((v.ty + 4) * v.txmax * cs + 2 * (v.ty + 2) * 16 + 127) / 128 * 128;
        int m2 = ((v.ty + 2) * v.txmax * cs + 2 * v.ty * cs + 127) / 128 * 128;
        return v.slots * slot + 3 * m1 + 3 * m2 + 256;
    }
    if (v.gen == 3) {
        int st_m = (v.ty * 16 + 127) / 128 * 128;
        int slot = (v.ty + 4) * v.txmax * cs + 2 * (256 + st_m) + (v.ty + 2) * v.txmax * cs + 2 * st_m;
        int mid = ((v.ty + 2) * v.txmax * cs + 2 * v.ty * cs + 127) / 128 * 128;
        return v.slots * slot + (v.lean ? 3 : 2) * mid + 256;
    }
    int c_bytes = (v.ty + 2) * v.txmax * cs;
    int h_pad = (v.ty * 16 + 127) / 128 * 128;
    if (v.gen == 1) return v.slots * ((c_bytes + 2 * h_pad + 127) / 128 * 128) + 128;
    return v.slots * ((c_bytes + 2 * h_pad + v.ty * v.txmax * cs + 127) / 128 * 128) + 256;
}

static int max_smem_optin() {
    static PerDevice m;
    return m.get([] {
        int v = 0;
        AXS_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, current_device()));
        return v;
    });
}

// The tx a variant would use for an N (largest admissible divisor), or 0.
static int variant_tx(const ZVariant &v, int N, int esz) {
    if (v.gen == 5) {
        // complex float, x-tiled (the kernel takes its x halo from strips), and
        // the two-step partner tiles N the same way
        if (esz != 4 || variant_smem(v, esz) > max_smem_optin() || v.ty < 3) return 0;
        const ZVariant &pv = kZVariants[v.partner];
        int tx = variant_tx(pv, N, esz);
        if (!tx || pv.ty != v.ty || tx > v.txmax || tx >= N || tx < 4) return 0;
        return tx;
    }
    if (v.gen == 3) {
        // complex float only; the partner must tile N the same way
        if (esz != 4 || variant_smem(v, esz) > max_smem_optin()) return 0;
        const ZVariant &pv = kZVariants[v.partner];
        int tx = variant_tx(pv, N, esz);
        if (!tx || pv.ty != v.ty || tx > v.txmax || N < 4) return 0;
        return tx;
    }
    int cs = 2 * esz;
    int vs = 16 / cs;
    int txmax = v.txmax;
    if (esz == 8) txmax = std::min(txmax, 128);   // box inner dim: 2*tx doubles <= 256
    if (variant_smem(v, esz) > max_smem_optin()) return 0;
    if (N % v.ty != 0 || N < 4 || v.ty < radius(v)) return 0;
    if (v.gen == 4 && (v.lean || v.slots < 2 * v.r + 2) && esz != 4) return 0;   // register z-ring: float fields only
    for (int tx = std::min(txmax, N); tx >= vs; --tx) {
        if (N % tx) continue;
        if (tx % vs) continue;
        if ((tx * cs) % 128) continue;   // shared-memory destinations stay 128-byte aligned
        return tx;
    }
    return 0;
}

// A variant serves a lattice when its stencil radius is the lattice's and it tiles N.
static bool variant_fits(const ZVariant &v, const axs_params &p, int esz) {
    return radius(v) == p.stencil_setting + 1 && variant_tx(v, p.N, esz) > 0;
}

bool zmarch_supported(const axs_params &p) {
    if (p.NDIMS != 3 || p.laplacian != 0) return false;
    int esz = p.precision == AXS_F32 ? 4 : 8;
    for (int v = 0; v < kNumZVariants; ++v)
        if (variant_fits(kZVariants[v], p, esz)) return true;
    return false;
}

typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                     const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static PFN_encodeTiled get_encode() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        AXS_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !f) fail(AXS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = (PFN_encodeTiled)f;
    }
    return fn;
}

static void encode_map(CUtensorMap *m, void *base, int N, int esz, int box_x_sites, int box_y) {
    // complex float sites as 8-byte elements; complex double as two 8-byte doubles
    int eu = esz == 4 ? 1 : 2;
    cuuint64_t dims[3] = {(cuuint64_t)N * eu, (cuuint64_t)N, (cuuint64_t)N};
    cuuint64_t strides[2] = {(cuuint64_t)N * 2 * esz, (cuuint64_t)N * N * 2 * esz};
    cuuint32_t box[3] = {(cuuint32_t)(box_x_sites * eu), (cuuint32_t)box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = get_encode()(m, esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base,
                              dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(AXS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
}

// Fill the z-march table entry of lattice L for a variant; returns items.
// a_index: the psi buffer that launch parity 0 treats as current. The entry's
// pih[b] is the momentum buffer that goes with psi[b]: L->pih for the current
// psi, and for a two-step variant L->scratch for the other one (the momentum
// is then written out of place and the host exchanges pih and scratch after
// every launch); one-step variants update the momentum in place.
static int64_t fill_zlat(ZLat &z, Lattice *L, int variant, int zchunk, int64_t item_base, int a_index) {
    const ZVariant &v = kZVariants[variant];
    int N = L->p.N;
    int tx = variant_tx(v, N, L->esz);
    if (!tx) fail(AXS_ERR_ARG, "z-march variant %d cannot tile N=%d", variant, N);
    prepare_zmarch(L->esz, variant);
    const bool oop = v.gen == 3 || v.gen == 5;
    if (oop && (!L->scratch || L->scratch == L->pih)) fail(AXS_ERR_STATE, "multi-step variant without a second momentum buffer");
    memset(&z, 0, sizeof z);
    int vs = 16 / (2 * L->esz);
    const int R = radius(v);
    const int rp = (R + vs - 1) / vs * vs;   // x-halo sites per side (16-byte multiple)
    void *pb[2];
    pb[L->cur] = L->pih;
    pb[L->cur ^ 1] = oop ? L->scratch : L->pih;
    for (int b = 0; b < 2; ++b) {
        encode_map(&z.tm_row[b], L->psi[b], N, L->esz, tx, R);     // R halo rows
        encode_map(&z.tm_main[b], L->psi[b], N, L->esz, tx, v.ty);
        encode_map(&z.tm_xh[b], L->psi[b], N, L->esz, rp, v.ty);   // x-halo strip
        encode_map(&z.tm_pih[b], pb[b], N, L->esz, tx, v.ty);
        if (oop) {   // the two-step kernel's maps (a three-step variant's partner)
            encode_map(&z.t2_row2[b], L->psi[b], N, L->esz, tx, 2);
            encode_map(&z.t2_str2[b], L->psi[b], N, L->esz, vs, 2);
            encode_map(&z.t2_prow[b], pb[b], N, L->esz, tx, 1);
            encode_map(&z.t2_pstr[b], pb[b], N, L->esz, vs, v.ty);
        }
        if (v.gen == 5) {
            encode_map(&z.t3_row3[b], L->psi[b], N, L->esz, tx, 3);
            encode_map(&z.t3_strm[b], L->psi[b], N, L->esz, 2 * vs, v.ty);
            encode_map(&z.t3_str2[b], L->psi[b], N, L->esz, 2 * vs, 2);
            encode_map(&z.t3_prow2[b], pb[b], N, L->esz, tx, 2);
            encode_map(&z.t3_pst1[b], pb[b], N, L->esz, vs, 1);
        }
        z.psi[b] = L->psi[b];
        z.pih[b] = pb[b];
    }
    z.clock = L->dclock;
    z.N = N;
    z.tx = tx;
    z.ntx = N / tx;
    z.nty = N / v.ty;
    z.nzc = std::max(1, N / std::max(1, zchunk));
    z.a_index = a_index;
    z.item_base = item_base;
    z.dt = (double)L->p.time_step;
    double dx = (double)L->p.space_step;
    z.inv_dx2 = 1.0 / (dx * dx);
    z.lambda = (double)L->p.lambda;
    double T0 = (double)L->p.T_initial;
    z.T0sq3 = (T0 * T0) / 3.0;
    z.prs = L->p.prs;
    z.form = L->p.form;
    z.debug_tx_excess = L->debug_tx_excess;
    return (int64_t)z.ntx * z.nty * z.nzc;
}

static thread_local bool t_capturing = false;
static thread_local int64_t t_captured = 0;

// The lattice's own table uses absolute parity: a launch passes L->cur.
static void ensure_single_table(Lattice *L) {
    if (t_capturing) fail(AXS_ERR_STATE, "internal: z-march table rebuilt inside a graph capture");
    ZLat z;
    int64_t items = fill_zlat(z, L, L->cfg.variant, L->cfg.zchunk, 0, 0);
    if (!L->dzlat) L->dzlat = (ZLat *)dalloc(sizeof(ZLat));
    AXS_CUDA(cudaMemcpyAsync(L->dzlat, &z, sizeof(ZLat), cudaMemcpyHostToDevice, L->stream));
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    L->zlat_variant = L->cfg.variant;
    L->zlat_zchunk = L->cfg.zchunk;
    L->zlat_pih[0] = z.pih[0];
    L->zlat_pih[1] = z.pih[1];
    L->zitems = items;
    L->cfg.tx = z.tx;
}

static bool single_table_valid(const Lattice *L) {
    if (!L->dzlat || L->zlat_variant != L->cfg.variant || L->zlat_zchunk != L->cfg.zchunk) return false;
    if (L->zlat_pih[L->cur] != L->pih) return false;
    return out_of_place(L->cfg.variant) ? L->zlat_pih[L->cur ^ 1] == L->scratch : L->zlat_pih[L->cur ^ 1] == L->pih;
}

void step_setup(Lattice *L) {
    L->cfg = StepConfig();
    L->cfg.kind = 0;
    if (zmarch_supported(L->p)) {
        // default before tuning: first variant that tiles N
        for (int v = 0; v < kNumZVariants; ++v)
            if (variant_fits(kZVariants[v], L->p, L->esz)) { L->cfg.kind = 1; L->cfg.variant = v; break; }
        L->cfg.zchunk = 64;
    }
    L->dcounter = (int *)dalloc(2 * sizeof(int));
    AXS_CUDA(cudaMemsetAsync(L->dcounter, 0, 2 * sizeof(int), L->stream));
}

void clear_graphs(std::map<GraphKey, GraphEntry> &g) {
    for (auto &e : g) cudaGraphExecDestroy(e.second.exec);
    g.clear();
}

static void spectral_release(Lattice *L);

void step_release(Lattice *L) {
    spectral_release(L);
    clear_graphs(L->graphs);
    dfree(L->dzlat);
    L->dzlat = nullptr;
    dfree(L->dcounter);
    L->dcounter = nullptr;
}

template <typename T, int ND, int R>
static void launch_generic_t(Lattice *L, const double *cin, double *cout) {
    typedef typename Cplx<T>::type C;
    const axs_params &p = L->p;
    double dx = p.space_step;
    double T0 = p.T_initial;
    k_step_generic<T, ND, R><<<grid_for(L->length), 256, 0, L->stream>>>(
        (const C *)L->psi[L->cur], (C *)L->psi[L->cur ^ 1], (C *)L->pih, cin, cout, p.N, L->length,
        (double)p.time_step, 1.0 / (dx * dx), (double)p.lambda, (T0 * T0) / 3.0, p.prs, p.stencil_setting, p.form);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

template <typename T>
static void launch_generic_dispatch(Lattice *L, const double *cin, double *cout) {
    int R = L->p.stencil_setting + 1;
    if (L->p.NDIMS == 2) {
        switch (R) {
        case 1: launch_generic_t<T, 2, 1>(L, cin, cout); break;
        case 2: launch_generic_t<T, 2, 2>(L, cin, cout); break;
        case 3: launch_generic_t<T, 2, 3>(L, cin, cout); break;
        default: launch_generic_t<T, 2, 4>(L, cin, cout); break;
        }
    } else {
        switch (R) {
        case 1: launch_generic_t<T, 3, 1>(L, cin, cout); break;
        case 2: launch_generic_t<T, 3, 2>(L, cin, cout); break;
        case 3: launch_generic_t<T, 3, 3>(L, cin, cout); break;
        default: launch_generic_t<T, 3, 4>(L, cin, cout); break;
        }
    }
}

// ---------------------------------------------------------------- spectral Laplacian
// scratch <- N^d L psi (both components): forward transform of the current psi
// into scratch, times -k^2, backward transform in place. The caller divides by
// N^d (as compute_laplacian_fft does after its backward transform).
static void spectral_laplacian(Lattice *L) {
    const int N = L->p.N;
    if (!L->have_c2c) {
        if (t_capturing) fail(AXS_ERR_STATE, "internal: transform plan created inside a graph capture");
        cufftType ty = L->esz == 4 ? CUFFT_C2C : CUFFT_Z2Z;
        if (L->p.NDIMS == 2) AXS_CUFFT(cufftPlan2d(&L->plan_c2c, N, N, ty));
        else AXS_CUFFT(cufftPlan3d(&L->plan_c2c, N, N, N, ty));
        AXS_CUFFT(cufftSetStream(L->plan_c2c, L->stream));
        // k of the reference (s_integrate.cpp:183, :193/:241): (-N/2.0f + i) * 2.0f * M_PI / L,
        // for the frequency of unshifted index j
        std::vector<unsigned char> tab((size_t)N * (sizeof(double) + sizeof(float)));
        double *kd = reinterpret_cast<double *>(tab.data());
        float *kf = reinterpret_cast<float *>(kd + N);
        const float Lf = N * L->p.space_step;
        for (int j = 0; j < N; ++j) {
            const int i = (j + N / 2) % N;   // shifted index of the same frequency
            const double k = (-N / 2.0f + i) * 2.0f * 3.14159265358979323846 / Lf;
            kd[j] = k * k;
            kf[j] = (float)kd[j];
        }
        L->dksq = dalloc(tab.size());
        AXS_CUDA(cudaMemcpyAsync(L->dksq, tab.data(), tab.size(), cudaMemcpyHostToDevice, L->stream));
        AXS_CUDA(cudaStreamSynchronize(L->stream));
        L->have_c2c = true;
    }
    const int g = grid_for(L->length);
    if (L->esz == 4) {
        AXS_CUFFT(cufftExecC2C(L->plan_c2c, (cufftComplex *)L->psi[L->cur], (cufftComplex *)L->scratch, CUFFT_FORWARD));
        k_kspace_laplacian<float><<<g, 256, 0, L->stream>>>((float2 *)L->scratch, L->dksq, N, L->p.NDIMS, L->length);
        AXS_CUDA(cudaGetLastError());
        AXS_CUFFT(cufftExecC2C(L->plan_c2c, (cufftComplex *)L->scratch, (cufftComplex *)L->scratch, CUFFT_INVERSE));
    } else {
        AXS_CUFFT(cufftExecZ2Z(L->plan_c2c, (cufftDoubleComplex *)L->psi[L->cur], (cufftDoubleComplex *)L->scratch,
                               CUFFT_FORWARD));
        k_kspace_laplacian<double><<<g, 256, 0, L->stream>>>((double2 *)L->scratch, L->dksq, N, L->p.NDIMS, L->length);
        AXS_CUDA(cudaGetLastError());
        AXS_CUFFT(cufftExecZ2Z(L->plan_c2c, (cufftDoubleComplex *)L->scratch, (cufftDoubleComplex *)L->scratch,
                               CUFFT_INVERSE));
    }
    count_launches(1);
}

template <typename T>
static void spectral_step_t(Lattice *L) {
    typedef typename Cplx<T>::type C;
    spectral_laplacian(L);
    const double T0 = L->p.T_initial;
    k_step_spectral<T><<<grid_for(L->length), 256, 0, L->stream>>>(
        (const C *)L->psi[L->cur], (C *)L->psi[L->cur ^ 1], (C *)L->pih, (const C *)L->scratch, L->dclock + L->cur,
        L->dclock + (L->cur ^ 1), L->length, (double)L->p.time_step, (double)L->p.lambda, (T0 * T0) / 3.0, L->p.prs,
        L->p.form);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

static void spectral_release(Lattice *L) {
    if (L->have_c2c) cufftDestroy(L->plan_c2c);
    L->have_c2c = false;
    dfree(L->dksq);
    L->dksq = nullptr;
}

// Advances a lattice by one launch of at most max_steps (>= 1) steps and
// returns the steps taken: two for a two-step variant when allowed, else one.
// The handle's bookkeeping advances here; the kernels may run later inside a
// graph.
int lattice_advance(Lattice *L, int max_steps) {
    const double *cin = L->dclock + L->cur;
    double *cout = L->dclock + (L->cur ^ 1);
    int k = 1;
    bool swap = false;
    if (L->fresh == 2) {   // the upload formed the drift already (launch_pack2_drift)
        L->fresh = 0;
    } else if (L->fresh) {
        if (L->esz == 4)
            k_drift0<float><<<grid_for(L->length), 256, 0, L->stream>>>((const float2 *)L->psi[L->cur],
                                                                         (float2 *)L->psi[L->cur ^ 1],
                                                                         (const float2 *)L->pih, cin, cout, L->length,
                                                                         (double)L->p.time_step, L->p.form);
        else
            k_drift0<double><<<grid_for(L->length), 256, 0, L->stream>>>((const double2 *)L->psi[L->cur],
                                                                          (double2 *)L->psi[L->cur ^ 1],
                                                                          (const double2 *)L->pih, cin, cout,
                                                                          L->length, (double)L->p.time_step, L->p.form);
        AXS_CUDA(cudaGetLastError());
        count_launches(1);
        L->fresh = 0;
    } else if (L->p.laplacian == 1) {   // the spectral step whatever the configuration says
        if (L->esz == 4) spectral_step_t<float>(L);
        else spectral_step_t<double>(L);
    } else if (L->cfg.kind == 1) {
        if (!single_table_valid(L)) ensure_single_table(L);
        int kv = L->cfg.variant;
        if (three_step(kv)) {   // an interval's last one or two steps run on the partners
            swap = true;
            if (max_steps >= 3) k = 3;
            else kv = kZVariants[kv].partner;
        }
        if (two_step(kv)) {
            swap = true;
            if (max_steps >= 2) k = 2;
            else kv = kZVariants[kv].partner;
        }
        launch_zmarch(L->esz, kv, L->dzlat, 1, L->zitems, L->dcounter, L->cur, L->derr, L->stream, L->cfg.ctas_per_sm);
        if (L->debug_tx_excess) {   // an injected stall lasts one launch: rebuild the table before the next
            L->debug_tx_excess = 0;
            L->zlat_variant = -1;
        }
    } else {
        if (L->esz == 4) launch_generic_dispatch<float>(L, cin, cout);
        else launch_generic_dispatch<double>(L, cin, cout);
    }
    L->cur ^= 1;
    if (swap) std::swap(L->pih, L->scratch);
    for (int s = 0; s < k; ++s) L->tau = L->tau + (double)L->p.time_step;
    L->steps += k;
    return k;
}

}  // namespace axs

namespace axs {

// ---------------------------------------------------------------- graphs
static int64_t g_launches = 0;
void count_launches(int64_t n) {
    if (t_capturing) t_captured += n;
    else __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED);
}
int64_t total_launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

// AXS_FORCE_CONFIG pins a configuration; it applies with AXS_AUTOTUNE=0 too.
static bool forced_config() {
    const char *f = getenv("AXS_FORCE_CONFIG");
    return f && *f;
}

static bool env_flag(const char *name, bool dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    return !(v[0] == '0' || v[0] == 'n' || v[0] == 'N' || v[0] == 'f' || v[0] == 'F');
}

static void prepare_tables(Lattice *L) {
    if (L->cfg.kind == 1 && L->p.laplacian == 0 && !single_table_valid(L)) ensure_single_table(L);
}

static uint64_t mix_state(uint64_t h, const Lattice *m) {
    h ^= (uint64_t)(uintptr_t)m->pih + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h ^= (uint64_t)m->cur + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h;
}

// Captures fn into a graph; *launches receives the kernels it launched.
template <typename StepFn>
static cudaGraphExec_t capture(cudaStream_t st, StepFn fn, int64_t *launches) {
    cudaGraph_t g = nullptr;
    AXS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    t_capturing = true;
    t_captured = 0;
    try {
        fn();
    } catch (...) {
        t_capturing = false;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    t_capturing = false;
    *launches = t_captured;
    AXS_CUDA(cudaStreamEndCapture(st, &g));
    cudaGraphExec_t ex = nullptr;
    AXS_CUDA(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    return ex;
}

void lattice_evolve(Lattice *L, int nsteps) {
    if (!L->tuned) {
        if (env_flag("AXS_AUTOTUNE", true) || forced_config()) lattice_autotune(L);
        L->tuned = true;
    }
    if (nsteps <= 0) return;
    if (L->fresh) {
        lattice_advance(L, 1);
        if (--nsteps == 0) return;
    }
    prepare_tables(L);
    if (nsteps < 2 || !env_flag("AXS_GRAPHS", true) || L->p.laplacian == 1) {   // spectral: transforms run eagerly
        while (nsteps > 0) nsteps -= lattice_advance(L, nsteps);
        return;
    }
    GraphKey key{nsteps, L->cur, mix_state(0, L)};
    auto it = L->graphs.find(key);
    if (it == L->graphs.end()) {
        const int cur0 = L->cur;
        const double tau0 = L->tau;
        const int64_t steps0 = L->steps;
        void *pih0 = L->pih, *scratch0 = L->scratch;
        GraphEntry e;
        e.exec = capture(L->stream, [&] {
            int n = nsteps;
            while (n > 0) n -= lattice_advance(L, n);
        }, &e.launches);
        e.cur_after.push_back(L->cur);
        e.swapped.push_back(L->pih != pih0);
        L->cur = cur0;
        L->tau = tau0;
        L->steps = steps0;
        L->pih = pih0;
        L->scratch = scratch0;
        it = L->graphs.insert(std::make_pair(key, e)).first;
    }
    const GraphEntry &e = it->second;
    AXS_CUDA(cudaGraphLaunch(e.exec, L->stream));
    count_launches(e.launches);
    for (int s = 0; s < nsteps; ++s) L->tau = L->tau + (double)L->p.time_step;
    L->cur = e.cur_after[0];
    if (e.swapped[0]) std::swap(L->pih, L->scratch);
    L->steps += nsteps;
}

// ---------------------------------------------------------------- autotune
// Everything that decides which kernels can run and how fast: the device,
// the shape, the precision, the stencil radius and the Laplacian (a spectral
// lattice never takes a finite-difference configuration tuned for the same
// shape).
struct TuneKey {
    int dev, n, ndims, esz, stencil, laplacian;
    bool operator<(const TuneKey &o) const {
        if (dev != o.dev) return dev < o.dev;
        if (n != o.n) return n < o.n;
        if (ndims != o.ndims) return ndims < o.ndims;
        if (esz != o.esz) return esz < o.esz;
        if (stencil != o.stencil) return stencil < o.stencil;
        return laplacian < o.laplacian;
    }
};
static std::map<TuneKey, StepConfig> g_tune_cache;
static std::mutex g_tune_mu;   // lattices may be tuned from different threads

static double time_launches(cudaStream_t st, int reps, const std::function<void()> &fn, int warm = 2) {
    cudaEvent_t a, b;
    AXS_CUDA(cudaEventCreate(&a));
    AXS_CUDA(cudaEventCreate(&b));
    for (int w = 0; w < warm; ++w) fn();
    AXS_CUDA(cudaEventRecord(a, st));
    for (int r = 0; r < reps; ++r) fn();
    AXS_CUDA(cudaEventRecord(b, st));
    AXS_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    AXS_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}

// Candidate steps run with dt = 0 on the lattice's own buffers:
// psi_out = psi + 0*pih and pih + 0*K are bit-identical copies for finite
// values (a -0.0 comes back as +0.0, which compares equal and gives the same
// decisions and sums), so the state (and tau) is unchanged. An infinite
// value would come back as NaN, so a state that is not finite is not timed
// on: the lattice keeps its untuned configuration, which is not cached.
// Candidates are
// the generic kernel and every z-march variant that tiles N (one-step
// variants, and two-step variants with halo depth 2). Every variant is first
// screened with one launch at one z-chunk; the three fastest are then timed
// at every z-chunk (32 to 256 planes) at full length, and the time per step
// decides.
void lattice_autotune(Lattice *L) {
    L->tuned = true;
    if (L->fresh == 2) L->fresh = 1;   // the trials overwrite the drift formed at upload
    // AXS_FORCE_CONFIG="kind,variant,zchunk" pins a configuration (tests use it
    // to show that every configuration gives bit-identical results).
    const char *force = getenv("AXS_FORCE_CONFIG");
    if (force && *force) {
        StepConfig c;
        int k = 0, v = 0, zc = 64;
        if (sscanf(force, "%d,%d,%d", &k, &v, &zc) >= 1) {
            c.kind = (k == 1 && zmarch_supported(L->p) && v >= 0 && v < kNumZVariants &&
                      variant_fits(kZVariants[v], L->p, L->esz)) ? 1 : 0;
            c.variant = c.kind ? v : 0;
            c.zchunk = zc > 0 ? zc : 64;
            L->cfg = c;
            L->zlat_variant = -1;
            clear_graphs(L->graphs);
            return;
        }
    }
    TuneKey key{current_device(), L->p.N, L->p.NDIMS, L->esz, L->p.stencil_setting, L->p.laplacian};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto hit = g_tune_cache.find(key);
        if (hit != g_tune_cache.end()) {
            if (hit->second.kind != L->cfg.kind || hit->second.variant != L->cfg.variant ||
                hit->second.zchunk != L->cfg.zchunk)
                clear_graphs(L->graphs);
            L->cfg = hit->second;
            L->zlat_variant = -1;
            return;
        }
        if (!zmarch_supported(L->p)) {
            L->cfg.kind = 0;
            g_tune_cache[key] = L->cfg;
            return;
        }
    }
    if (!check_finite(L)) return;
    float dt_save = L->p.time_step;
    L->p.time_step = 0.0f;
    int reps = L->length >= (1 << 27) ? 4 : 10;
    StepConfig best = L->cfg;
    double best_ms = 1e30;
    int cur_save = L->cur;
    std::vector<std::pair<StepConfig, double>> log;
    // generic kernel
    {
        StepConfig c;
        c.kind = 0;
        double ms = time_launches(L->stream, reps, [&] {
            const double *cin = L->dclock + L->cur;
            double *cout = L->dclock + (L->cur ^ 1);
            if (L->esz == 4) launch_generic_dispatch<float>(L, cin, cout);
            else launch_generic_dispatch<double>(L, cin, cout);
            L->cur ^= 1;
        });
        log.push_back({c, ms});
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    const int zchunks[] = {32, 64, 128, 256};
    auto trial = [&](int v, int zc, int nrep, int nwarm) {
        const bool two = out_of_place(v);
        StepConfig c;
        c.kind = 1;
        c.variant = v;
        c.zchunk = zc;
        L->cfg = c;
        ensure_single_table(L);   // built with dt = 0
        double ms = time_launches(L->stream, nrep, [&] {
            launch_zmarch(L->esz, v, L->dzlat, 1, L->zitems, L->dcounter, L->cur, L->derr, L->stream, 0);
            L->cur ^= 1;
            if (two) std::swap(L->pih, L->scratch);
        }, nwarm);
        ms /= steps_per_pass(v);   // per step
        c.tx = L->cfg.tx;
        log.push_back({c, ms});
        return std::make_pair(c, ms);
    };
    int zc0 = 0;   // the screening z-chunk: the largest candidate up to min(N, 128)
    for (int zc : zchunks)
        if (zc <= L->p.N && zc <= 128) zc0 = zc;
    std::vector<std::pair<double, int>> screen;
    if (zc0 > 0)
        for (int v = 0; v < kNumZVariants; ++v)
            if (variant_fits(kZVariants[v], L->p, L->esz) && variant_resident(L->esz, v))
                screen.push_back({trial(v, zc0, 1, 1).second, v});
    std::sort(screen.begin(), screen.end());
    for (size_t k = 0; k < screen.size() && k < 3; ++k)
        for (int zc : zchunks) {
            if (zc > L->p.N) continue;
            auto r = trial(screen[k].second, zc, reps, 2);
            if (r.second < best_ms) { best_ms = r.second; best = r.first; }
        }
    L->p.time_step = dt_save;
    // dt = 0 steps copied psi (and, out of place, pih) back and forth; values
    // are identical, but keep the psi buffer the caller had as current.
    if (L->cur != cur_save) {
        AXS_CUDA(cudaMemcpyAsync(L->psi[cur_save], L->psi[L->cur], (size_t)L->length * 2 * L->esz,
                                 cudaMemcpyDeviceToDevice, L->stream));
        AXS_CUDA(cudaMemcpyAsync(L->dclock + cur_save, L->dclock + L->cur, sizeof(double), cudaMemcpyDeviceToDevice,
                                 L->stream));
        L->cur = cur_save;
    }
    L->cfg = best;
    L->zlat_variant = -1;   // rebuild the table with the real dt before the next step
    clear_graphs(L->graphs);
    check_device_errors(L);   // a trial that timed out: fail here, with nothing cached
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    if (env_flag("AXS_TUNE_LOG", false)) {
        for (auto &e : log) fprintf(stderr, "[axs autotune N=%d] %-60s %.4f ms/step\n", L->p.N, e.first.describe().c_str(), e.second);
        fprintf(stderr, "[axs autotune N=%d] chose %s\n", L->p.N, best.describe().c_str());
    }
}

// ---------------------------------------------------------------- ensemble
static bool ensemble_variant_ok(Ensemble *E, int v) {
    if (three_step(v)) return false;   // single lattices only
    for (Lattice *m : E->members)
        if (m->p.NDIMS != 3 || m->p.laplacian != 0 || !variant_fits(kZVariants[v], m->p, m->esz)) return false;
    return true;
}

// One table over all members, largest first (their items are taken first).
// Parity is relative: a member's entry treats its cur at build time as
// current at launch parity 0.
static void ensemble_table(Ensemble *E, float dt_override, bool use_override) {
    const size_t nm = E->members.size();
    std::vector<int> order(nm);
    for (size_t i = 0; i < nm; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return E->members[a]->length > E->members[b]->length; });
    std::vector<ZLat> tab(nm);
    E->tab_cur.assign(nm, 0);
    E->tab_pih.assign(2 * nm, nullptr);
    int64_t base = 0;
    for (size_t k = 0; k < nm; ++k) {
        const int i = order[k];
        Lattice *m = E->members[i];
        float dt = m->p.time_step;
        if (use_override) m->p.time_step = dt_override;
        base += fill_zlat(tab[k], m, E->cfg.variant, E->cfg.zchunk, base, m->cur);
        m->p.time_step = dt;
        E->tab_cur[i] = m->cur;
        E->tab_pih[2 * i] = tab[k].pih[0];
        E->tab_pih[2 * i + 1] = tab[k].pih[1];
    }
    if (!E->dzlat) E->dzlat = (ZLat *)dalloc(sizeof(ZLat) * std::max<size_t>(1, nm));
    AXS_CUDA(cudaMemcpyAsync(E->dzlat, tab.data(), sizeof(ZLat) * nm, cudaMemcpyHostToDevice, E->stream));
    AXS_CUDA(cudaStreamSynchronize(E->stream));
    E->zitems = base;
}

void ensemble_setup(Ensemble *E) {
    E->cfg = StepConfig();
    E->cfg.kind = 0;
    for (int v = 0; v < kNumZVariants; ++v)
        if (ensemble_variant_ok(E, v)) { E->cfg.kind = 1; E->cfg.variant = v; E->cfg.zchunk = 64; break; }
    E->dcounter = (int *)dalloc(2 * sizeof(int));
    E->derr = (int *)dalloc(sizeof(int));
    AXS_CUDA(cudaMemsetAsync(E->dcounter, 0, 2 * sizeof(int), E->stream));
    AXS_CUDA(cudaMemsetAsync(E->derr, 0, sizeof(int), E->stream));
    if (E->cfg.kind == 1) ensemble_table(E, 0.f, false);
}

static int ensemble_parity(const Ensemble *E) { return E->members[0]->cur ^ E->tab_cur[0]; }

static bool ensemble_table_valid(Ensemble *E) {
    if (!E->dzlat || E->tab_cur.size() != E->members.size()) return false;
    // every member must sit at the same parity relative to its entry, with the
    // momentum buffer the entry expects
    const int d = ensemble_parity(E);
    const bool two = two_step(E->cfg.variant);
    for (size_t i = 0; i < E->members.size(); ++i) {
        const Lattice *m = E->members[i];
        if ((m->cur ^ E->tab_cur[i]) != d) return false;
        if (E->tab_pih[2 * i + m->cur] != m->pih) return false;
        if (E->tab_pih[2 * i + (m->cur ^ 1)] != (two ? m->scratch : m->pih)) return false;
    }
    return true;
}

// One launch over every member; returns the steps taken (see lattice_advance).
static int ensemble_advance(Ensemble *E, int max_steps) {
    if (E->cfg.kind != 1) {
        for (Lattice *m : E->members) lattice_advance(m, 1);
        return 1;
    }
    if (!ensemble_table_valid(E)) {
        if (t_capturing) fail(AXS_ERR_STATE, "internal: ensemble table rebuilt inside a graph capture");
        ensemble_table(E, 0.f, false);
    }
    int kv = E->cfg.variant, k = 1;
    const bool two = two_step(kv);
    if (two) {
        if (max_steps >= 2) k = 2;
        else kv = kZVariants[kv].partner;
    }
    launch_zmarch(E->members[0]->esz, kv, E->dzlat, (int)E->members.size(), E->zitems, E->dcounter, ensemble_parity(E),
                  E->derr, E->stream, E->cfg.ctas_per_sm);
    for (Lattice *m : E->members) {
        m->cur ^= 1;
        if (two) std::swap(m->pih, m->scratch);
        for (int s = 0; s < k; ++s) m->tau = m->tau + (double)m->p.time_step;
        m->steps += k;
    }
    return k;
}

void ensemble_autotune(Ensemble *E) {
    E->tuned = true;
    for (Lattice *m : E->members)
        if (m->fresh == 2) m->fresh = 1;   // the trials overwrite the drift formed at upload
    if (E->cfg.kind != 1) return;
    // AXS_FORCE_CONFIG="1,variant,zchunk" pins the ensemble's z-march
    // configuration too (when the variant tiles every member)
    const char *force = getenv("AXS_FORCE_CONFIG");
    if (force && *force) {
        int k = 0, v = 0, zc = 64;
        if (sscanf(force, "%d,%d,%d", &k, &v, &zc) >= 2 && k == 1 && v >= 0 && v < kNumZVariants &&
            ensemble_variant_ok(E, v)) {
            E->cfg.kind = 1;
            E->cfg.variant = v;
            E->cfg.zchunk = zc > 0 ? zc : 64;
            ensemble_table(E, 0.f, false);
            clear_graphs(E->graphs);
            return;
        }
    }
    // dt = 0 trials on the members' own buffers, as in lattice_autotune: not
    // on a state that is not finite (it would come back as NaN)
    for (Lattice *m : E->members)
        if (!check_finite(m)) return;
    std::vector<int> cur_save;
    for (Lattice *m : E->members) cur_save.push_back(m->cur);
    int reps = 6;
    StepConfig best = E->cfg;
    double best_ms = 1e30;
    const int zchunks[] = {32, 64, 128, 256};   // 256: whole columns of every member up to 256^3
    for (int v = 0; v < kNumZVariants; ++v) {
        if (!ensemble_variant_ok(E, v) || !variant_resident(E->members[0]->esz, v)) continue;
        const bool two = two_step(v);
        for (int zc : zchunks) {
            StepConfig c;
            c.kind = 1;
            c.variant = v;
            c.zchunk = zc;
            c.tx = variant_tx(kZVariants[v], E->members[0]->p.N, E->members[0]->esz);
            E->cfg = c;
            ensemble_table(E, 0.f, true);
            double ms = time_launches(E->stream, reps, [&] {
                launch_zmarch(E->members[0]->esz, v, E->dzlat, (int)E->members.size(), E->zitems, E->dcounter,
                              ensemble_parity(E), E->derr, E->stream, 0);
                for (Lattice *m : E->members) {
                    m->cur ^= 1;
                    if (two) std::swap(m->pih, m->scratch);
                }
            });
            if (two) ms *= 0.5;   // per step
            if (ms < best_ms) { best_ms = ms; best = c; }
            if (env_flag("AXS_TUNE_LOG", false))
                fprintf(stderr, "[axs autotune ensemble] %-60s %.4f ms/step\n", c.describe().c_str(), ms);
        }
    }
    for (size_t i = 0; i < E->members.size(); ++i) {
        Lattice *m = E->members[i];
        if (m->cur != cur_save[i]) {
            AXS_CUDA(cudaMemcpyAsync(m->psi[cur_save[i]], m->psi[m->cur], (size_t)m->length * 2 * m->esz,
                                     cudaMemcpyDeviceToDevice, E->stream));
            AXS_CUDA(cudaMemcpyAsync(m->dclock + cur_save[i], m->dclock + m->cur, sizeof(double),
                                     cudaMemcpyDeviceToDevice, E->stream));
            m->cur = cur_save[i];
        }
    }
    E->cfg = best;
    ensemble_table(E, 0.f, false);
    clear_graphs(E->graphs);
    check_device_error_flag(E->derr, E->stream);   // a trial that timed out fails here
}

std::string ensemble_describe(const Ensemble *E) {
    StepConfig c = E->cfg;
    if (c.kind == 1 && !E->members.empty()) c.tx = variant_tx(kZVariants[c.variant], E->members[0]->p.N, E->members[0]->esz);
    return c.describe();
}

void ensemble_evolve(Ensemble *E, int nsteps) {
    if (!E->tuned) {
        if (env_flag("AXS_AUTOTUNE", true) || forced_config()) ensemble_autotune(E);
        E->tuned = true;
    }
    if (nsteps <= 0) return;
    for (Lattice *m : E->members)
        if ((m->fresh != 0) != (E->members[0]->fresh != 0) || m->steps != E->members[0]->steps)
            fail(AXS_ERR_STATE, "ensemble members are not at the same step");
    if (E->members[0]->fresh) {
        for (Lattice *m : E->members) lattice_advance(m, 1);   // pure drift per member
        if (--nsteps == 0) return;
    }
    if (E->cfg.kind == 1 && !ensemble_table_valid(E)) ensemble_table(E, 0.f, false);
    if (E->cfg.kind != 1)
        for (Lattice *m : E->members) prepare_tables(m);
    if (nsteps < 2 || !env_flag("AXS_GRAPHS", true) || E->members[0]->p.laplacian == 1) {
        while (nsteps > 0) nsteps -= ensemble_advance(E, nsteps);
        return;
    }
    uint64_t h = 0;
    for (Lattice *m : E->members) h = mix_state(h, m);
    GraphKey key{nsteps, E->cfg.kind == 1 ? ensemble_parity(E) : E->members[0]->cur, h};
    auto it = E->graphs.find(key);
    if (it == E->graphs.end()) {
        std::vector<int> cur0;
        std::vector<double> tau0;
        std::vector<int64_t> st0;
        std::vector<void *> pih0, scr0;
        for (Lattice *m : E->members) {
            cur0.push_back(m->cur);
            tau0.push_back(m->tau);
            st0.push_back(m->steps);
            pih0.push_back(m->pih);
            scr0.push_back(m->scratch);
        }
        GraphEntry e;
        e.exec = capture(E->stream, [&] {
            int n = nsteps;
            while (n > 0) n -= ensemble_advance(E, n);
        }, &e.launches);
        for (size_t i = 0; i < E->members.size(); ++i) {
            Lattice *m = E->members[i];
            e.cur_after.push_back(m->cur);
            e.swapped.push_back(m->pih != pih0[i]);
            m->cur = cur0[i];
            m->tau = tau0[i];
            m->steps = st0[i];
            m->pih = pih0[i];
            m->scratch = scr0[i];
        }
        it = E->graphs.insert(std::make_pair(key, e)).first;
    }
    const GraphEntry &e = it->second;
    AXS_CUDA(cudaGraphLaunch(e.exec, E->stream));
    count_launches(e.launches);
    for (size_t i = 0; i < E->members.size(); ++i) {
        Lattice *m = E->members[i];
        for (int s = 0; s < nsteps; ++s) m->tau = m->tau + (double)m->p.time_step;
        m->cur = e.cur_after[i];
        if (e.swapped[i]) std::swap(m->pih, m->scratch);
        m->steps += nsteps;
    }
}
// ---------------------------------------------------------------- helpers
template <typename T, int ND, int R>
static void sync_pi_t(Lattice *L) {
    typedef typename Cplx<T>::type C;
    double dx = L->p.space_step, T0 = L->p.T_initial;
    k_sync_pi<T, ND, R><<<grid_for(L->length), 256, 0, L->stream>>>(
        (const C *)L->psi[L->cur], (const C *)L->pih, (C *)L->scratch, L->dclock + L->cur, L->p.N, L->length,
        (double)L->p.time_step, 1.0 / (dx * dx), (double)L->p.lambda, (T0 * T0) / 3.0, L->p.prs, L->p.stencil_setting,
        L->p.form);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}
template <typename T>
static void sync_pi_dispatch(Lattice *L) {
    int R = L->p.stencil_setting + 1;
    if (L->p.NDIMS == 2) {
        if (R == 1) sync_pi_t<T, 2, 1>(L); else if (R == 2) sync_pi_t<T, 2, 2>(L); else if (R == 3) sync_pi_t<T, 2, 3>(L); else sync_pi_t<T, 2, 4>(L);
    } else {
        if (R == 1) sync_pi_t<T, 3, 1>(L); else if (R == 2) sync_pi_t<T, 3, 2>(L); else if (R == 3) sync_pi_t<T, 3, 3>(L); else sync_pi_t<T, 3, 4>(L);
    }
}
void launch_sync_pi(Lattice *L) {
    if (L->fresh) {   // pih holds pi_0 and the reference's ker_curr is zero
        AXS_CUDA(cudaMemcpyAsync(L->scratch, L->pih, (size_t)L->length * 2 * L->esz, cudaMemcpyDeviceToDevice, L->stream));
        return;
    }
    if (L->p.laplacian == 1) {
        spectral_laplacian(L);
        const double T0 = L->p.T_initial;
        const int g = grid_for(L->length);
        if (L->esz == 4)
            k_sync_pi_spectral<float><<<g, 256, 0, L->stream>>>(
                (const float2 *)L->psi[L->cur], (const float2 *)L->pih, (float2 *)L->scratch, L->dclock + L->cur,
                L->length, (double)L->p.time_step, (double)L->p.lambda, (T0 * T0) / 3.0, L->p.prs, L->p.form);
        else
            k_sync_pi_spectral<double><<<g, 256, 0, L->stream>>>(
                (const double2 *)L->psi[L->cur], (const double2 *)L->pih, (double2 *)L->scratch, L->dclock + L->cur,
                L->length, (double)L->p.time_step, (double)L->p.lambda, (T0 * T0) / 3.0, L->p.prs, L->p.form);
        AXS_CUDA(cudaGetLastError());
        count_launches(1);
        return;
    }
    if (L->esz == 4) sync_pi_dispatch<float>(L);
    else sync_pi_dispatch<double>(L);
}

template <typename T, int ND, int R>
static void lap_t(Lattice *L, int comp, double *dout) {
    typedef typename Cplx<T>::type C;
    double dx = L->p.space_step;
    k_laplacian<T, ND, R><<<grid_for(L->length), 256, 0, L->stream>>>((const C *)L->psi[L->cur], dout, comp, L->p.N,
                                                                       L->length, 1.0 / (dx * dx), L->p.stencil_setting);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}
template <typename T>
static void lap_dispatch(Lattice *L, int comp, double *dout) {
    int R = L->p.stencil_setting + 1;
    if (L->p.NDIMS == 2) {
        if (R == 1) lap_t<T, 2, 1>(L, comp, dout); else if (R == 2) lap_t<T, 2, 2>(L, comp, dout); else if (R == 3) lap_t<T, 2, 3>(L, comp, dout); else lap_t<T, 2, 4>(L, comp, dout);
    } else {
        if (R == 1) lap_t<T, 3, 1>(L, comp, dout); else if (R == 2) lap_t<T, 3, 2>(L, comp, dout); else if (R == 3) lap_t<T, 3, 3>(L, comp, dout); else lap_t<T, 3, 4>(L, comp, dout);
    }
}
void launch_laplacian(Lattice *L, int comp, double *dout) {
    if (L->p.laplacian == 1) {   // the spectral Laplacian itself (already in physical units)
        spectral_laplacian(L);
        const int g = grid_for(L->length);
        if (L->esz == 4) k_laplacian_spectral<float><<<g, 256, 0, L->stream>>>((const float2 *)L->scratch, dout, comp, L->length);
        else k_laplacian_spectral<double><<<g, 256, 0, L->stream>>>((const double2 *)L->scratch, dout, comp, L->length);
        AXS_CUDA(cudaGetLastError());
        count_launches(1);
        return;
    }
    if (L->esz == 4) lap_dispatch<float>(L, comp, dout);
    else lap_dispatch<double>(L, comp, dout);
}

// which: 0 = current psi, 1 = pih
void launch_pack(Lattice *L, const void *src_real, int src_is_double, int which, int comp) {
    void *dst = which == 0 ? L->psi[L->cur] : L->pih;
    int g = grid_for(L->length);
    if (L->esz == 4) {
        if (src_is_double) k_pack<float, double><<<g, 256, 0, L->stream>>>((const double *)src_real, (float *)dst, comp, L->length);
        else k_pack<float, float><<<g, 256, 0, L->stream>>>((const float *)src_real, (float *)dst, comp, L->length);
    } else {
        if (src_is_double) k_pack<double, double><<<g, 256, 0, L->stream>>>((const double *)src_real, (double *)dst, comp, L->length);
        else k_pack<double, float><<<g, 256, 0, L->stream>>>((const float *)src_real, (double *)dst, comp, L->length);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

void launch_unpack(Lattice *L, const void *src, int which, int comp, void *dst_real, int dst_is_double) {
    (void)which;
    int g = grid_for(L->length);
    if (L->esz == 4) {
        if (dst_is_double) k_unpack<float, double><<<g, 256, 0, L->stream>>>((const float *)src, (double *)dst_real, comp, L->length);
        else k_unpack<float, float><<<g, 256, 0, L->stream>>>((const float *)src, (float *)dst_real, comp, L->length);
    } else {
        if (dst_is_double) k_unpack<double, double><<<g, 256, 0, L->stream>>>((const double *)src, (double *)dst_real, comp, L->length);
        else k_unpack<double, float><<<g, 256, 0, L->stream>>>((const double *)src, (float *)dst_real, comp, L->length);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

// Pair transfers: dst/src complex array <-> (a, b) real arrays reachable by
// the device (device pointers or device aliases of page-locked host memory).
static bool quad_ok(const void *a, const void *b, const void *c, int64_t n) {
    return ((((uintptr_t)a | (uintptr_t)b | (uintptr_t)c) & 15) == 0) && (n & 3) == 0;
}
void launch_pack2(Lattice *L, const void *a, const void *b, int src_is_double, void *dst_cplx, int64_t n,
                  cudaStream_t st) {
    if (quad_ok(a, b, dst_cplx, n)) {
        const int g = grid_for(n / 4);
        if (L->esz == 4) {
            if (src_is_double) k_pack2_x4<float, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (float *)dst_cplx, n / 4);
            else k_pack2_x4<float, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (float *)dst_cplx, n / 4);
        } else {
            if (src_is_double) k_pack2_x4<double, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (double *)dst_cplx, n / 4);
            else k_pack2_x4<double, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (double *)dst_cplx, n / 4);
        }
        AXS_CUDA(cudaGetLastError());
        count_launches(1);
        return;
    }
    int g = grid_for(n);
    if (L->esz == 4) {
        if (src_is_double) k_pack2<float, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (float2 *)dst_cplx, n);
        else k_pack2<float, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (float2 *)dst_cplx, n);
    } else {
        if (src_is_double) k_pack2<double, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (double2 *)dst_cplx, n);
        else k_pack2<double, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (double2 *)dst_cplx, n);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}
void launch_pack2_drift(Lattice *L, const void *a, const void *b, int src_is_double, int64_t off, int64_t n,
                        cudaStream_t st) {
    const size_t cs = (size_t)2 * L->esz;
    char *pih = (char *)L->pih + (size_t)off * cs;
    const char *psi = (const char *)L->psi[L->cur] + (size_t)off * cs;
    char *nxt = (char *)L->psi[L->cur ^ 1] + (size_t)off * cs;
    const double *cin = L->dclock + L->cur;
    double *cout = L->dclock + (L->cur ^ 1);
    const double dt = L->p.time_step;
    const int form = L->p.form;
    if (quad_ok(a, b, pih, n) && quad_ok(a, b, nxt, n) && quad_ok(a, b, psi, n)) {
        const int g = grid_for(n / 4);
        if (L->esz == 4) {
            if (src_is_double)
                k_pack2_drift_x4<float, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (float *)pih,
                                                                  (const float *)psi, (float *)nxt, n / 4, cin, cout, dt, form);
            else
                k_pack2_drift_x4<float, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (float *)pih,
                                                                 (const float *)psi, (float *)nxt, n / 4, cin, cout, dt, form);
        } else {
            if (src_is_double)
                k_pack2_drift_x4<double, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (double *)pih,
                                                                   (const double *)psi, (double *)nxt, n / 4, cin, cout, dt, form);
            else
                k_pack2_drift_x4<double, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (double *)pih,
                                                                  (const double *)psi, (double *)nxt, n / 4, cin, cout, dt, form);
        }
    } else {
        const int g = grid_for(n);
        if (L->esz == 4) {
            if (src_is_double)
                k_pack2_drift<float, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (float2 *)pih,
                                                               (const float2 *)psi, (float2 *)nxt, n, cin, cout, dt, form);
            else
                k_pack2_drift<float, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (float2 *)pih,
                                                              (const float2 *)psi, (float2 *)nxt, n, cin, cout, dt, form);
        } else {
            if (src_is_double)
                k_pack2_drift<double, double><<<g, 256, 0, st>>>((const double *)a, (const double *)b, (double2 *)pih,
                                                                (const double2 *)psi, (double2 *)nxt, n, cin, cout, dt, form);
            else
                k_pack2_drift<double, float><<<g, 256, 0, st>>>((const float *)a, (const float *)b, (double2 *)pih,
                                                               (const double2 *)psi, (double2 *)nxt, n, cin, cout, dt, form);
        }
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}
void launch_unpack2(Lattice *L, const void *src_cplx, void *a, void *b, int dst_is_double, int64_t n, cudaStream_t st) {
    if (quad_ok(a, b, src_cplx, n)) {
        const int g = grid_for(n / 4);
        if (L->esz == 4) {
            if (dst_is_double) k_unpack2_x4<float, double><<<g, 256, 0, st>>>((const float *)src_cplx, (double *)a, (double *)b, n / 4);
            else k_unpack2_x4<float, float><<<g, 256, 0, st>>>((const float *)src_cplx, (float *)a, (float *)b, n / 4);
        } else {
            if (dst_is_double) k_unpack2_x4<double, double><<<g, 256, 0, st>>>((const double *)src_cplx, (double *)a, (double *)b, n / 4);
            else k_unpack2_x4<double, float><<<g, 256, 0, st>>>((const double *)src_cplx, (float *)a, (float *)b, n / 4);
        }
        AXS_CUDA(cudaGetLastError());
        count_launches(1);
        return;
    }
    int g = grid_for(n);
    if (L->esz == 4) {
        if (dst_is_double) k_unpack2<float, double><<<g, 256, 0, st>>>((const float2 *)src_cplx, (double *)a, (double *)b, n);
        else k_unpack2<float, float><<<g, 256, 0, st>>>((const float2 *)src_cplx, (float *)a, (float *)b, n);
    } else {
        if (dst_is_double) k_unpack2<double, double><<<g, 256, 0, st>>>((const double2 *)src_cplx, (double *)a, (double *)b, n);
        else k_unpack2<double, float><<<g, 256, 0, st>>>((const double2 *)src_cplx, (float *)a, (float *)b, n);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

void check_device_error_flag(int *derr, cudaStream_t s) {
    int h = 0;
    AXS_CUDA(cudaMemcpyAsync(&h, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    AXS_CUDA(cudaStreamSynchronize(s));
    if (h & DEVERR_TIMEOUT) {
        AXS_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), s));
        fail(AXS_ERR_TIMEOUT, "a step kernel gave up waiting for a TMA load; the step was not completed");
    }
}
void check_device_errors(Lattice *L) { check_device_error_flag(L->derr, L->stream); }

}  // namespace axs
