// Per-output analysis on the device: plaquette string finder, power spectra
// after cuFFT, background means, energies and the finiteness check.
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#include <mutex>

#include "axs_internal.h"
#include "axs_tma.cuh"

namespace axs {

static int grid_cap(int64_t work, int threads, int per_sm) {
    int64_t want = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)num_sms() * per_sm));
}

// ============================================================== string finder
//
// cores2 / cores3 (src/common/string_finding.cpp:3-86) flag a cell when the sum
// of min(|dn|, 1-|dn|) over three edges of a plaquette exceeds
// accept = (double)(0.5f*(1-thr/100.0f)), with n = (theta+pi)/(2 pi) and
// theta = atan2(phi1, phi2). The decision is taken in two stages:
//  1. FP32: n from fast_atan2 (below), edges and sums in float. The error of
//     each float sum against the exact double sum is below 2e-6 (theta within
//     5e-7 rad, n within 1.5e-7, each edge within 4e-7, plus the rounding of
//     two additions), so a float sum farther than kMargin = 1e-5 from accept
//     decides the cell.
//  2. Otherwise the cell is recomputed with the reference's double
//     expressions in the reference's order (no contraction, IEEE division),
//     which makes the decision bit-exact to the reference on a given theta.
static constexpr float kMargin = 1e-5f;

// atan2(y, x) in float within 5e-7 rad (the background means' float angle):
// octant reduction to a = min(|x|,|y|) / max(|x|,|y|) in [0, 1] (a fast
// division, within 2 ulp), atan(a) = a P(a^2) with P of degree 7 fitted to
// atan on [0, 1] (weighted least squares iterated to equal ripple, Lawson's
// method; tests/atan_fit.py regenerates the table), then the octant undone.
// Exact zeros and magnitudes outside [1e-30, 1e30] take atan2f (the signed
// results on the axes).
__device__ constexpr float kAtanC[8] = {9.999993443e-01f, -3.332986236e-01f, 1.994658262e-01f, -1.390872002e-01f,
                                        9.642439336e-02f, -5.591578037e-02f, 2.186544798e-02f, -4.055280238e-03f};
// The string finder's angle in turns, atan2(y, x) / (2 pi): the same
// reduction with P of degree 5 fitted to atan(a) / (2 pi) (tests/atan_fit.py),
// within 2.8e-7 turns (1.7e-6 rad) evaluated in float, and the octant undone
// in turns (1/4, 1/2). Only |x| + |y| outside [2e-30, 1e30] (so max(|x|, |y|)
// within [1e-30, 1e30] otherwise) and a NaN component take atan2f: with one
// zero component the reduced argument is 0 and the fix-ups give atan2's
// signed axis values. turns_core is the polynomial path; it clears `ok` when
// the pair needs atan2f, so a caller can test several angles at once.
__device__ constexpr float kTurnC[6] = {1.591513157e-01f, -5.293861777e-02f, 3.080324642e-02f,
                                        -1.853073202e-02f, 8.380074054e-03f, -1.865555299e-03f};
__device__ __forceinline__ float turns_core(float y, float x, bool &ok) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float sum = ax + ay;   // NaN when either component is
    ok = ok && sum >= 2e-30f && sum <= 1e30f;
    const float a = __fdividef(mn, mx);   // within 2 ulp for 2^-126 <= mx <= 2^126
    const float s = a * a;
    float p = kTurnC[5];
#pragma unroll
    for (int k = 4; k >= 0; --k) p = fmaf(p, s, kTurnC[k]);
    float r = p * a;
    if (ay > ax) r = 0.25f - r;
    if (x < 0.0f) r = 0.5f - r;
    return copysignf(r, y);
}
__device__ __forceinline__ float fast_turns(float y, float x) {
    bool ok = true;
    const float r = turns_core(y, x, ok);
    return ok ? r : atan2f(y, x) * 0.15915494309189535f;
}
__device__ __forceinline__ float fast_atan2(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    if (mn == 0.0f || mx < 1e-30f || mx > 1e30f) return atan2f(y, x);
    const float a = __fdividef(mn, mx);   // within 2 ulp for 2^-126 <= mx <= 2^126
    const float s = a * a;
    float p = kAtanC[7];
#pragma unroll
    for (int k = 6; k >= 0; --k) p = fmaf(p, s, kAtanC[k]);
    float r = p * a;
    if (ay > ax) r = 1.5707963267948966f - r;
    if (x < 0.0f) r = 3.1415926535897932f - r;
    return copysignf(r, y);
}

template <typename T, bool FROM_THETA>
struct Corner {
    const typename Cplx<T>::type *psi;
    const double *theta;
    __device__ __forceinline__ float nf(int64_t m) const {
        float th;
        if (FROM_THETA) th = (float)theta[m];
        else { auto v = psi[m]; th = fast_atan2((float)v.x, (float)v.y); }
        return fmaf(th, 0.15915494309189535f, 0.5f);
    }
    __device__ __forceinline__ double nd(int64_t m) const {
        double th;
        if (FROM_THETA) th = theta[m];
        else { auto v = psi[m]; th = atan2((double)v.x, (double)v.y); }
        return __ddiv_rn(__dadd_rn(th, 3.14159265358979323846), 6.28318530717958647692);   // (theta + M_PI)/(2*M_PI)
    }
};

__device__ __forceinline__ float circf(float a, float b) {
    float d = fabsf(b - a);
    return fminf(d, 1.0f - d);
}
// std::min(abs(d), 1 - abs(d)) of string_finding.cpp:22-24 in double
__device__ __forceinline__ double circd(double a, double b) {
    double d = fabs(__dsub_rn(b, a));
    double e = __dsub_rn(1.0, d);
    return (e < d) ? e : d;
}
__device__ __forceinline__ double sum3(double a, double b, double c) { return __dadd_rn(__dadd_rn(a, b), c); }

// The reference's double decision for the 3D cell whose (i,j,k) corner is
// site (x, y, z) (reference (i,j,k) = (z,y,x)). Out of line: it runs only for
// cells within the float margin, and inlined its double registers would
// lower the occupancy of the float path.
template <typename T, bool FROM_THETA>
__device__ __noinline__ int cell3_exact(Corner<T, FROM_THETA> cn, int64_t x, int64_t y, int64_t z, int N,
                                        double accept) {
    const int64_t NN = (int64_t)N * N;
    const int64_t xp = x + 1 == N ? 0 : x + 1, yp = y + 1 == N ? 0 : y + 1, zp = z + 1 == N ? 0 : z + 1;
    const double d000 = cn.nd(z * NN + y * N + x), d100 = cn.nd(zp * NN + y * N + x), d110 = cn.nd(zp * NN + yp * N + x),
                 d010 = cn.nd(z * NN + yp * N + x), d011 = cn.nd(z * NN + yp * N + xp), d001 = cn.nd(z * NN + y * N + xp);
    const double ta = sum3(circd(d000, d100), circd(d100, d110), circd(d110, d010));
    const double tb = sum3(circd(d000, d100), circd(d100, d011), circd(d011, d001));
    const double tc = sum3(circd(d000, d010), circd(d010, d011), circd(d011, d001));
    return (ta > accept || tb > accept || tc > accept) ? 1 : 0;
}

template <typename T, int ND, bool FROM_THETA>
__global__ void __launch_bounds__(256) k_cores(const typename Cplx<T>::type *__restrict__ psi,
                                               const double *__restrict__ theta, uint8_t *__restrict__ mask, int N,
                                               int64_t len, double accept, unsigned long long *count) {
    Corner<T, FROM_THETA> cn{psi, theta};
    const float acc_f = (float)accept;
    unsigned long long local = 0;
    const int64_t NN = (int64_t)N * N;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        int flag;
        if (ND == 2) {
            int64_t i = m % N, j = m / N;
            int64_t ip = i + 1 == N ? 0 : i + 1, jp = j + 1 == N ? 0 : j + 1;
            int64_t o1 = m, o2 = ip + N * j, o3 = ip + N * jp, o4 = i + N * jp;
            float s = circf(cn.nf(o1), cn.nf(o2)) + circf(cn.nf(o2), cn.nf(o3)) + circf(cn.nf(o3), cn.nf(o4));
            if (s > acc_f + kMargin) flag = 1;
            else if (s < acc_f - kMargin) flag = 0;
            else {
                double n1 = cn.nd(o1), n2 = cn.nd(o2), n3 = cn.nd(o3), n4 = cn.nd(o4);
                flag = sum3(circd(n1, n2), circd(n2, n3), circd(n3, n4)) > accept;
            }
        } else {
            // reference (i,j,k) = (z,y,x) here: i slowest, k fastest
            int64_t x = m % N, y = (m / N) % N, z = m / NN;
            int64_t xp = x + 1 == N ? 0 : x + 1, yp = y + 1 == N ? 0 : y + 1, zp = z + 1 == N ? 0 : z + 1;
            int64_t o000 = m;                       // (i,j,k)
            int64_t o100 = zp * NN + y * N + x;     // (i+1,j,k)
            int64_t o110 = zp * NN + yp * N + x;    // (i+1,j+1,k)
            int64_t o010 = z * NN + yp * N + x;     // (i,j+1,k)
            int64_t o011 = z * NN + yp * N + xp;    // (i,j+1,k+1)
            int64_t o001 = z * NN + y * N + xp;     // (i,j,k+1)
            float f000 = cn.nf(o000), f100 = cn.nf(o100), f110 = cn.nf(o110), f010 = cn.nf(o010), f011 = cn.nf(o011),
                  f001 = cn.nf(o001);
            float e_000_100 = circf(f000, f100);
            float e_011_001 = circf(f011, f001);
            float sa = e_000_100 + circf(f100, f110) + circf(f110, f010);
            float sb = e_000_100 + circf(f100, f011) + e_011_001;    // plaquette b, string_finding.cpp:54-57
            float sc = circf(f000, f010) + circf(f010, f011) + e_011_001;
            float mx = fmaxf(sa, fmaxf(sb, sc));
            if (mx > acc_f + kMargin) flag = 1;
            else if (mx < acc_f - kMargin) flag = 0;
            else flag = cell3_exact<T, FROM_THETA>(cn, x, y, z, N, accept);
        }
        mask[m] = (uint8_t)flag;
        local += flag;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// 3D finder from psi, tiled: a block owns a CX x CY tile of cells and marches a
// z-chunk. Each thread owns a run of four cells along x in one row and loads
// the four sites at their (i,j,k) corners (in FP32 two 16-byte loads when N is
// a multiple of 4); threads 0-80 load one more site each, the tile's +y row
// and +x column. The angles, in turns theta/(2 pi) (fast_turns; n of the
// reference minus 1/2, which no difference sees), are computed once per site
// into a two-plane shared ring (k_cores evaluates them once per corner, six
// times per site), one range test for a thread's four. A thread keeps its own
// four angles in registers and per plane reads six of plane z+1 from the ring
// (one 16-byte and two 4-byte shared loads: row y+1 and the +x neighbours);
// it carries the angles of plane z and the edge values of their y-edges, and
// forms 21 edge values for its four cells. The four mask bytes go out as one
// 32-bit store when N is a multiple of 4.
// An edge is kept as t = 1/2 - |d| (d the difference of its angles, |d| < 1):
// the reference's min(|d|, 1 - |d|) is 1/2 - |t|, so a plaquette's sum is
// 3/2 - (|t1| + |t2| + |t3|) and the three sums of a cell exceed accept when
// the least sum of |t| is below 3/2 - accept. Plaquettes a and b share their
// z-edge e, so the cell's least sum is min(e + min(sa', sb'), sc) with sa',
// sb' the sums of their other two edges. The float stage decides at a margin
// of kMargin from that bound (its error: angles within 3.2e-7 turns with the
// division and the octant roundings, edges within 7e-7, a sum of |t| within
// 2.3e-6); the other cells take the double replay after the march. A thread
// whose twelve sums all lie above the margin (nearly every thread: flagged
// cells are rare) writes four zero bytes without forming the flag bits.
static constexpr int kCX = 64, kCY = 16, kCZ = 32;   // cells per block tile; 256 threads x 4 cells
static constexpr int kHalo = kCX + kCY + 1;          // the tile's +y row and +x column (with the corner)

// 1/2 - |b - a| for angles in turns (see above)
__device__ __forceinline__ float half_gap(float a, float b) { return 0.5f - fabsf(b - a); }
static_assert(kCZ * 4 <= 128, "two 64-bit words of margin bits per thread");
static constexpr int kRS = kCX + 4;                   // shared row stride: 16-byte aligned rows, +x halo at kCX

// VEC: N is a multiple of 4, so a thread's four cells are all in the lattice
// or all outside it and its four sites are contiguous and 16-byte aligned.
// FP32: four CTAs per SM (64 registers); the march is issue-bound, and 32
// warps per SM ran 3.12 against 3.36 ms at 1024^3 for 24. FP64 holds twice
// the prefetched field in registers: three CTAs.
template <typename T, bool VEC>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3)
    k_cores3_tiled(const typename Cplx<T>::type *__restrict__ psi, uint8_t *__restrict__ mask, int N, double accept,
                   unsigned long long *count) {
    typedef typename Cplx<T>::type C;
    __shared__ __align__(16) float nsm[2][kCY + 1][kRS];
    Corner<T, false> cn{psi, nullptr};
    const float acc_f = (float)accept;
    // least sum of |t| of a certainly flagged cell, greatest of an undecided one
    const float t_flag = 1.5f - acc_f - kMargin, t_undecided = 1.5f - acc_f + kMargin;
    const int64_t NN = (int64_t)N * N;
    const int x0 = blockIdx.x * kCX, y0 = blockIdx.y * kCY, z0 = blockIdx.z * kCZ;
    const int z1 = min(N, z0 + kCZ);
    const int tid = threadIdx.x;
    const int lx = 4 * (tid & 15), ly = tid >> 4;   // the thread's cells: (lx .. lx+3, ly) of the tile
    const int gx = x0 + lx, gy = y0 + ly;
    unsigned local = 0;   // flagged cells of this thread (at most 4 kCZ)
    // bit 4 (z - z0 - 8 w) + j of unc[w][tid]: cell (gx + j, gy, z) lies within
    // the float margin (in shared memory: set rarely, read once at the end)
    __shared__ unsigned unc[kCZ / 8][256];
#pragma unroll
    for (int w = 0; w < kCZ / 8; ++w) unc[w][tid] = 0;
    // The sites this thread loads, as in-plane offsets that do not depend on z.
    // A site at x = N or y = N is site 0 of that axis (periodic); sites past
    // that are corners of no cell in the lattice and are not loaded.
    const int wy = gy < N ? gy : (gy == N ? 0 : -1);
    int own = -1;   // VEC: the first of the four sites
    int xs[4];      // general N: each site's x, -1 when not loaded
    if (VEC) {
        const int wx = gx < N ? gx : (gx == N ? 0 : -1);   // gx < N: gx + 3 < N
        if (wy >= 0 && wx >= 0) own = wy * N + wx;
    } else {
        own = wy >= 0 ? wy * N : -1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int x = gx + j;
            xs[j] = (wy < 0 || x > N) ? -1 : (x == N ? 0 : x);
        }
    }
    int hso = -1, hsi = 0;   // threads 0-80: the +y row (x0 .. x0+63), then the +x column (y0 .. y0+16)
    if (tid < kHalo) {
        const bool row = tid < kCX;
        const int hx = row ? x0 + tid : x0 + kCX, hy = row ? y0 + kCY : y0 + (tid - kCX);
        hsi = row ? kCY * kRS + tid : (tid - kCX) * kRS + kCX;
        if (hx <= N && hy <= N) hso = (hy == N ? 0 : hy) * N + (hx == N ? 0 : hx);
    }
    const bool row_ok = gy < N;
    unsigned vmask = 0, vbytes = 0;   // bit / byte j: cell (gx + j, gy) is in the lattice
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (row_ok && gx + j < N) {
            vmask |= 1u << j;
            vbytes |= 1u << (8 * j);
        }
    // psi of the next plane's sites, loaded one plane ahead; sites not loaded
    // keep (0, 1), a valid angle that only cells outside the lattice see
    C pre[4], ph;
#pragma unroll
    for (int j = 0; j < 4; ++j) pre[j] = C{T(0), T(1)};
    ph = C{T(0), T(1)};
    auto load = [&](int z) {
        const C *pl = psi + (int64_t)(z >= N ? z - N : z) * NN;
        if (VEC) {
            if (own >= 0) {
                if constexpr (sizeof(T) == 4) {
                    const float4 *q = reinterpret_cast<const float4 *>(pl + own);
                    const float4 u = q[0], v = q[1];
                    pre[0] = C{u.x, u.y};
                    pre[1] = C{u.z, u.w};
                    pre[2] = C{v.x, v.y};
                    pre[3] = C{v.z, v.w};
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) pre[j] = pl[own + j];
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (xs[j] >= 0) pre[j] = pl[own + xs[j]];
        }
        if (hso >= 0) ph = pl[hso];
    };
    // the angles of the prefetched plane: the thread's four into c[0..3] and
    // the ring's row ly, the halo site into the ring
    auto angles = [&](int buf, float (&c)[5]) {
        bool ok = true;
#pragma unroll
        for (int j = 0; j < 4; ++j) c[j] = turns_core((float)pre[j].x, (float)pre[j].y, ok);
        if (!ok) {
#pragma unroll
            for (int j = 0; j < 4; ++j) c[j] = fast_turns((float)pre[j].x, (float)pre[j].y);
        }
        *reinterpret_cast<float4 *>(&nsm[buf][ly][lx]) = make_float4(c[0], c[1], c[2], c[3]);
        if (hso >= 0) (&nsm[buf][0][0])[hsi] = fast_turns((float)ph.x, (float)ph.y);
    };
    // after the barrier: the +x neighbour of row ly and row ly+1 at x = lx .. lx+4
    auto read = [&](int buf, float (&r0)[5], float (&r1)[5]) {
        const float4 v = *reinterpret_cast<const float4 *>(&nsm[buf][ly + 1][lx]);
        r0[4] = nsm[buf][ly][lx + 4];
        r1[0] = v.x; r1[1] = v.y; r1[2] = v.z; r1[3] = v.w; r1[4] = nsm[buf][ly + 1][lx + 4];
    };
    float a0[5], a1[5], ya[5];   // plane z: rows y, y+1 and their y-edge values t
    load(z0);
    angles(0, a0);
    load(z0 + 1);
    __syncthreads();
    read(0, a0, a1);
#pragma unroll
    for (int i = 0; i < 5; ++i) ya[i] = half_gap(a0[i], a1[i]);
    // One plane: plane z+1 goes into buffer nb, the one last read two planes
    // ago (every thread is past the previous barrier, so done with it).
    int64_t mo = (int64_t)z0 * NN + (int64_t)gy * N + gx;   // mask offset of cell (gx, gy, z)
    auto plane_step = [&](const int z, const int nb) {
        float b0[5], b1[5], yb[5];
        angles(nb, b0);
        if (z + 2 <= z1) load(z + 2);   // in flight while plane z is evaluated
        __syncthreads();
        read(nb, b0, b1);
#pragma unroll
        for (int i = 0; i < 5; ++i) yb[i] = half_gap(b0[i], b1[i]);
        float tm[4];   // each cell's least sum of |t|
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // f000 = a0[j], f001 = a0[j+1], f010 = a1[j], f011 = a1[j+1],
            // f100 = b0[j], f110 = b1[j]; plaquettes a, b, c of string_finding.cpp:49-82
            const float e_000_100 = fabsf(half_gap(a0[j], b0[j]));
            const float sa = fabsf(yb[j]) + fabsf(half_gap(b1[j], a1[j]));
            const float sb = fabsf(half_gap(b0[j], a1[j + 1])) + fabsf(ya[j + 1]);   // the (i,j+1,k+1) corner
            const float tc = fabsf(ya[j]) + fabsf(half_gap(a1[j], a1[j + 1])) + fabsf(ya[j + 1]);
            tm[j] = fminf(e_000_100 + fminf(sa, sb), tc);
        }
        unsigned word = 0;
        if (fminf(fminf(tm[0], tm[1]), fminf(tm[2], tm[3])) <= t_undecided) {
            unsigned und = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const bool flag = tm[j] < t_flag;
                word |= (flag ? 1u : 0u) << (8 * j);
                und |= (!flag && tm[j] <= t_undecided ? 1u : 0u) << j;   // the double replay, after the march
            }
            word &= vbytes;   // cells past the lattice's edge
            und &= vmask;
            local += __popc(word);
            if (und) unc[(z - z0) >> 3][tid] |= und << (4 * ((z - z0) & 7));
        }
        if (VEC) {
            if (vbytes) *reinterpret_cast<unsigned *>(mask + mo) = word;   // 4-byte aligned: N, gx multiples of 4
        } else if (row_ok) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (gx + j < N) mask[mo + j] = (uint8_t)(word >> (8 * j));
        }
        mo += NN;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            a0[i] = b0[i];
            a1[i] = b1[i];
            ya[i] = yb[i];
        }
    };
    // two planes per trip (a chunk has an even number of planes: N and kCZ
    // are even), so the buffer indices are constants and the carried
    // registers alternate instead of moving
    for (int z = z0; z < z1; z += 2) {
        plane_step(z, 1);
        plane_step(z + 1, 0);
    }
    // The cells within the float margin (written 0 above) take the exact
    // double decision here, where little else is live across the call.
#pragma unroll 1
    for (int w = 0; w < kCZ / 8; ++w) {
        unsigned u = unc[w][tid];
        while (u) {
            const int b = __ffs((int)u) - 1 + 32 * w;
            u &= u - 1;
            const int zz = z0 + (b >> 2), j = b & 3;
            if (cell3_exact<T, false>(cn, gx + j, gy, zz, N, accept)) {
                mask[(int64_t)zz * NN + (int64_t)gy * N + gx + j] = 1;
                ++local;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, (unsigned long long)local);
}

// ---- ordered compaction of the mask: chunk counts, scan, ordered write
static constexpr int kChunk = 4096;   // cells per block

__global__ void k_chunk_counts(const uint8_t *__restrict__ mask, int64_t len, int64_t *__restrict__ counts) {
    int64_t base = (int64_t)blockIdx.x * kChunk;
    int c = 0;
    for (int q = threadIdx.x; q < kChunk; q += blockDim.x) {
        int64_t m = base + q;
        if (m < len) c += mask[m];
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t s = 0;
        for (int w = 0; w < 8; ++w) s += ws[w];
        counts[blockIdx.x] = s;
    }
}

// Exclusive scan of n counts by one block of 1024 threads.
__global__ void k_scan(int64_t *__restrict__ counts, int64_t n, int64_t *__restrict__ total) {
    __shared__ int64_t part[1024];
    int64_t per = (n + 1023) / 1024;
    int64_t b = threadIdx.x * per, e = b + per < n ? b + per : n;
    int64_t s = 0;
    for (int64_t i = b; i < e; ++i) s += counts[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (int i = 0; i < 1024; ++i) { int64_t v = part[i]; part[i] = run; run += v; }
        *total = run;
    }
    __syncthreads();
    int64_t run = part[threadIdx.x];
    for (int64_t i = b; i < e; ++i) { int64_t v = counts[i]; counts[i] = run; run += v; }
}

__global__ void k_chunk_write(const uint8_t *__restrict__ mask, int64_t len, const int64_t *__restrict__ offsets,
                              int64_t *__restrict__ list) {
    __shared__ int wsum[8];
    int64_t base = (int64_t)blockIdx.x * kChunk;
    int64_t out = offsets[blockIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q0 = 0; q0 < kChunk; q0 += blockDim.x) {
        int64_t m = base + q0 + threadIdx.x;
        int f = (m < len) ? mask[m] : 0;
        unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wsum[w] = __popc(bal);
        __syncthreads();
        int before = 0, tot = 0;
        for (int i = 0; i < 8; ++i) { if (i < w) before += wsum[i]; tot += wsum[i]; }
        if (f) list[out + before + __popc(bal & ((1u << lane) - 1))] = m;
        out += tot;
        __syncthreads();
    }
}

// Neighbouring-plaquette pairs of s_run.cpp:101-109 over the ascending list.
__global__ void k_pairs2(const int64_t *__restrict__ list, int64_t n, int N, unsigned long long *pairs) {
    unsigned long long local = 0;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q + 1 < n; q += stride) {
        int64_t a = list[q], b = list[q + 1];
        int64_t dx = (b % N) - (a % N), dy = (b / N) - (a / N);
        local += (dy == 0 && dx == 1) || (dy == 1 && dx == 0);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(pairs, local);
}

__global__ void k_positions(const int64_t *__restrict__ list, int64_t n, int N, int ndims, int32_t *__restrict__ pos) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t NN = (int64_t)N * N;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        int64_t m = list[q];
        if (ndims == 2) { pos[2 * q] = (int32_t)(m % N); pos[2 * q + 1] = (int32_t)(m / N); }
        else { pos[3 * q] = (int32_t)(m / NN); pos[3 * q + 1] = (int32_t)((m / N) % N); pos[3 * q + 2] = (int32_t)(m % N); }
    }
}

static void ensure_mask(Lattice *L) {
    if (!L->dmask) L->dmask = (uint8_t *)dalloc((size_t)L->length);
    if (!L->dcount) L->dcount = (int64_t *)dalloc(4 * sizeof(int64_t));
}

// A work buffer of at least `bytes` in the lattice's slot (allocated once, grown
// when a call needs more), so repeated analysis calls do not allocate.
static void *lattice_tmp(Lattice *L, int slot, size_t bytes) {
    if (L->tmp_cap[slot] < bytes) {
        dfree(L->tmp[slot]);
        L->tmp[slot] = nullptr;
        L->tmp_cap[slot] = 0;
        L->tmp[slot] = dalloc(bytes);
        L->tmp_cap[slot] = bytes;
    }
    return L->tmp[slot];
}

// Build the ascending list of flagged offsets from the device mask.
static int64_t compact(Lattice *L) {
    int64_t nch = (L->length + kChunk - 1) / kChunk;
    int64_t *counts = (int64_t *)lattice_tmp(L, 0, (size_t)nch * sizeof(int64_t));
    int64_t total = 0;
    {
        k_chunk_counts<<<(unsigned)nch, 256, 0, L->stream>>>(L->dmask, L->length, counts);
        k_scan<<<1, 1024, 0, L->stream>>>(counts, nch, L->dcount + 2);
        count_launches(2);
        AXS_CUDA(cudaGetLastError());
        AXS_CUDA(cudaMemcpyAsync(&total, L->dcount + 2, sizeof(int64_t), cudaMemcpyDeviceToHost, L->stream));
        AXS_CUDA(cudaStreamSynchronize(L->stream));
        if (total > L->list_cap) {
            dfree(L->dlist);
            L->dlist = nullptr;
            L->list_cap = std::max<int64_t>(total, 1024);
            L->dlist = (int32_t *)dalloc((size_t)L->list_cap * sizeof(int64_t));
        }
        k_chunk_write<<<(unsigned)nch, 256, 0, L->stream>>>(L->dmask, L->length, counts, (int64_t *)L->dlist);
        count_launches(1);
        AXS_CUDA(cudaGetLastError());
        AXS_CUDA(cudaStreamSynchronize(L->stream));
    }
    L->list_valid = true;
    return total;
}

template <typename T>
static void launch_cores(Lattice *L, bool from_theta, double accept, unsigned long long *cnt) {
    typedef typename Cplx<T>::type C;
    const C *psi = (const C *)L->psi[L->cur];
    int g = grid_cap(L->length, 256, 8);
    int N = L->p.N;
    if (L->p.NDIMS == 2) {
        if (from_theta) k_cores<T, 2, true><<<g, 256, 0, L->stream>>>(psi, L->dtheta, L->dmask, N, L->length, accept, cnt);
        else k_cores<T, 2, false><<<g, 256, 0, L->stream>>>(psi, nullptr, L->dmask, N, L->length, accept, cnt);
    } else {
        if (from_theta) k_cores<T, 3, true><<<g, 256, 0, L->stream>>>(psi, L->dtheta, L->dmask, N, L->length, accept, cnt);
        else {
            dim3 grid((N + kCX - 1) / kCX, (N + kCY - 1) / kCY, (N + kCZ - 1) / kCZ);
            if ((N & 3) == 0) k_cores3_tiled<T, true><<<grid, 256, 0, L->stream>>>(psi, L->dmask, N, accept, cnt);
            else k_cores3_tiled<T, false><<<grid, 256, 0, L->stream>>>(psi, L->dmask, N, accept, cnt);
        }
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

void find_strings(Lattice *L, const double *theta_host, uint8_t *mask_host, int64_t *nplaq, int64_t *ncores) {
    ensure_mask(L);
    bool from_theta = theta_host != nullptr;
    if (from_theta) {
        if (!L->dtheta) L->dtheta = (double *)dalloc((size_t)L->length * sizeof(double));
        AXS_CUDA(cudaMemcpyAsync(L->dtheta, theta_host, (size_t)L->length * sizeof(double), cudaMemcpyHostToDevice,
                                 L->stream));
    }
    int thr = L->p.thr;
    double accept = (double)(0.5f * (1.0f - thr / 100.0f));   // string_finding.cpp:8,40
    AXS_CUDA(cudaMemsetAsync(L->dcount, 0, 2 * sizeof(int64_t), L->stream));
    unsigned long long *cnt = (unsigned long long *)L->dcount;
    if (L->esz == 4) launch_cores<float>(L, from_theta, accept, cnt);
    else launch_cores<double>(L, from_theta, accept, cnt);
    int64_t n = 0;
    AXS_CUDA(cudaMemcpyAsync(&n, L->dcount, sizeof(int64_t), cudaMemcpyDeviceToHost, L->stream));
    if (mask_host) AXS_CUDA(cudaMemcpyAsync(mask_host, L->dmask, (size_t)L->length, cudaMemcpyDeviceToHost, L->stream));
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    L->last_nplaq = n;
    L->list_valid = false;
    int64_t cores = n;
    if (L->p.NDIMS == 2) {
        int64_t total = compact(L);
        AXS_CUDA(cudaMemsetAsync(L->dcount + 1, 0, sizeof(int64_t), L->stream));
        k_pairs2<<<grid_cap(std::max<int64_t>(total, 1), 256, 4), 256, 0, L->stream>>>(
            (const int64_t *)L->dlist, total, L->p.N, (unsigned long long *)(L->dcount + 1));
        count_launches(1);
        AXS_CUDA(cudaGetLastError());
        int64_t pairs = 0;
        AXS_CUDA(cudaMemcpyAsync(&pairs, L->dcount + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, L->stream));
        AXS_CUDA(cudaStreamSynchronize(L->stream));
        cores = n - pairs;
    }
    if (nplaq) *nplaq = n;
    if (ncores) *ncores = cores;
}

void string_positions(Lattice *L, int32_t *pos, int64_t cap, int64_t *n) {
    if (L->last_nplaq < 0) fail(AXS_ERR_STATE, "axs_string_positions needs a preceding axs_find_strings");
    int64_t total = L->list_valid ? L->last_nplaq : compact(L);
    if (n) *n = total;
    int64_t w = std::min<int64_t>(cap, total);
    if (w <= 0 || !pos) return;
    int nd = L->p.NDIMS;
    int32_t *dpos = (int32_t *)dalloc((size_t)w * nd * sizeof(int32_t));
    try {
        k_positions<<<grid_cap(w, 256, 4), 256, 0, L->stream>>>((const int64_t *)L->dlist, w, L->p.N, nd, dpos);
        count_launches(1);
        AXS_CUDA(cudaGetLastError());
        AXS_CUDA(cudaMemcpyAsync(pos, dpos, (size_t)w * nd * sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
        AXS_CUDA(cudaStreamSynchronize(L->stream));
    } catch (...) {
        dfree(dpos);
        throw;
    }
    dfree(dpos);
}

// ============================================================== spectra
//
// Real field -> R2C cuFFT -> binning. The half spectrum stands for the full
// one: a mode with 0 < kx < N/2 represents itself and its mirror (weight 2);
// kx = 0 is its own mirror set (weight 1); kx = N/2 lies at |n| >= N/2, which
// both spectra drop or place in the last bin like any other mode.
//
// Binning is deterministic: each warp owns a shared-memory histogram it alone
// updates; lanes holding the same bin are summed by a fixed shuffle tree; the
// block adds its warps' histograms in order and writes one partial row; a
// final kernel adds the rows in block order.

struct RefBins {     // pk_estimation.cpp:92-100: floor(|n|) - 1 for 0 < |n| < N/2
    int half;
    __device__ __forceinline__ RefBins staged(double *) const { return *this; }
    static constexpr int kSmemTable = 0;
    __device__ __forceinline__ int bin(int64_t n2) const {
        double kmag = sqrt((double)n2);
        if (kmag == 0.0 || kmag >= half) return -1;
        return (int)floor(kmag) - 1;
    }
};
struct LogBins {     // nbins log-spaced in |n| between 1 and sqrt(d) N/2
    const double *edge2;   // edge2[b] = t_b^2, b = 1..nbins-1
    int nbins;
    // copy of the edge table in shared memory (s: nbins doubles)
    __device__ __forceinline__ LogBins staged(double *s) const {
        for (int i = threadIdx.x; i < nbins; i += blockDim.x) s[i] = edge2[i];
        return LogBins{s, nbins};
    }
    static constexpr int kSmemTable = 1;
    __device__ __forceinline__ int bin(int64_t n2) const {
        if (n2 == 0) return -1;
        double v = (double)n2;
        int lo = 0, hi = nbins - 1;    // largest b with edge2[b] <= v (edge2[0] = 0)
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (edge2[mid] <= v) lo = mid; else hi = mid - 1;
        }
        return lo;
    }
};

// ROWS = 2: per-bin counts by global integer atomics (the allocation-free
// binner's layout); ROWS = 3: counts accumulated like the sums, as a third
// per-warp row (exact: integer-valued doubles), one partial row each.
template <typename T, typename B, int ROWS = 2>
__global__ void __launch_bounds__(128) k_bin(const typename Cplx<T>::type *__restrict__ F, int N, int ndims, B binner,
                                             int nbins, double *__restrict__ partials, unsigned long long *__restrict__ counts) {
    extern __shared__ double hist[];   // [4 warps][ROWS][nbins], then the bin table if the binner has one
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 4 * ROWS * nbins; i += blockDim.x) hist[i] = 0.0;
    const B bins = binner.staged(hist + 4 * ROWS * nbins);
    __syncthreads();
    double *hp = hist + (size_t)w * ROWS * nbins;
    double *hk = hp + nbins;
    double *hc = hk + nbins;   // ROWS == 3 only
    const int nh = N / 2 + 1;
    const int64_t rows = ndims == 2 ? (int64_t)N : (int64_t)N * N;
    const int64_t total = rows * nh;
    const int64_t wstride = (int64_t)gridDim.x * 4 * 32;
    const int64_t start = ((int64_t)blockIdx.x * 4 + w) * 32;
    for (int64_t base = start; base < total; base += wstride) {
        int64_t q = base + lane;
        int b = -1;
        double v = 0.0, kk = 0.0, wt = 0.0;
        if (q < total) {
            int ix = (int)(q % nh);
            int64_t r = q / nh;
            int64_t fx = ix;
            int64_t n2;
            if (ndims == 2) {
                int64_t iy = r, fy = iy < N / 2 ? iy : iy - N;
                n2 = fx * fx + fy * fy;
            } else {
                int64_t iz = r / N, iy = r % N;
                int64_t fz = iz < N / 2 ? iz : iz - N, fy = iy < N / 2 ? iy : iy - N;
                n2 = fx * fx + fy * fy + fz * fz;
            }
            b = bins.bin(n2);
            if (b >= 0) {
                auto f = F[q];
                wt = (ix == 0 || 2 * ix == N) ? 1.0 : 2.0;
                double re = (double)f.x, im = (double)f.y;
                v = wt * (re * re + im * im);
                kk = wt * sqrt((double)n2);
            }
        }
        unsigned active = __ballot_sync(0xffffffffu, b >= 0);
        while (active) {
            const int leader = __ffs(active) - 1;
            const int bl = __shfl_sync(0xffffffffu, b, leader);
            const unsigned same = __ballot_sync(0xffffffffu, b == bl) & active;
            const bool mine = (same >> lane) & 1u;
            double sv = mine ? v : 0.0, sk = mine ? kk : 0.0;
            unsigned long long sc = mine ? (unsigned long long)wt : 0ull;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sv += __shfl_xor_sync(0xffffffffu, sv, o);
                sk += __shfl_xor_sync(0xffffffffu, sk, o);
                sc += __shfl_xor_sync(0xffffffffu, sc, o);
            }
            if (lane == 0) {
                hp[bl] += sv;
                hk[bl] += sk;
                if (ROWS == 3) hc[bl] += (double)sc;
                else atomicAdd(&counts[bl], sc);
            }
            active &= ~same;
        }
    }
    __syncthreads();
    for (int bn = threadIdx.x; bn < nbins; bn += blockDim.x) {
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            double acc = 0.0;
            for (int ww = 0; ww < 4; ++ww) acc += hist[(size_t)ww * ROWS * nbins + (size_t)r * nbins + bn];
            partials[((int64_t)blockIdx.x * ROWS + r) * nbins + bn] = acc;
        }
    }
}

// One block per bin: strided partial sums over the blocks in a fixed order,
// then a fixed shuffle tree; out = [pk | |n| | count] rows of nbins.
__global__ void k_bin_final3(const double *__restrict__ partials, int nblocks, int nbins, double *__restrict__ out) {
    const int bn = blockIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int r = 0; r < 3; ++r) v[r] += partials[((int64_t)b * 3 + r) * nbins + bn];
    __shared__ double red[8][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        for (int o = 16; o > 0; o >>= 1) v[r] += __shfl_down_sync(0xffffffffu, v[r], o);
    if ((threadIdx.x & 31) == 0)
        for (int r = 0; r < 3; ++r) red[threadIdx.x >> 5][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int r = 0; r < 3; ++r) {
            double acc = 0.0;
            for (int w = 0; w < 8; ++w) acc += red[w][r];
            out[(int64_t)r * nbins + bn] = acc;
        }
}

// ---- row-based binner (the allocating spectra)
//
// Integer bin rules (n2 = |n|^2 is an integer):
//   RefBinsI: floor(|n|) - 1 for 0 < n2 < (N/2)^2, floor(|n|) = isqrt(n2) (equal
//             to floor(sqrt((double)n2)) of pk_estimation.cpp:92-95 for n2 < 2^52)
//   LogBinsI: b = #{ b' in 1..nbins-1 : n2 >= thr[b'] }, thr = ceil(edge^2),
//             the same test as n2 >= edge^2 for integer n2.
struct RefBinsI {
    int half;
    __device__ __forceinline__ RefBinsI staged(double *) const { return *this; }
    static constexpr int kSmemTable = 0;
    __device__ __forceinline__ int bin(int n2) const {
        if (n2 == 0 || n2 >= half * half) return -1;
        const float fn = (float)n2;
        int s = (int)(fn * rsqrtf(fn));   // within 0.02 of sqrt(n2), as in ceil_isqrt
        while (s * s > n2) --s;
        while ((s + 1) * (s + 1) <= n2) ++s;
        return s - 1;
    }
    // bin of n2 >= the n2 that gave b (bins only grow along a row)
    __device__ __forceinline__ int next(int b, int n2) const {
        if (b < 0 || n2 >= half * half) return bin(n2);
        while ((b + 2) * (b + 2) <= n2) ++b;
        return b;
    }
    // the least n2' > n2 whose bin may differ from b = bin(n2)
    __device__ __forceinline__ int upper(int b, int n2) const {
        if (b >= 0) return min((b + 2) * (b + 2), half * half);
        return n2 == 0 ? 1 : INT_MAX;   // the origin, or past the last bin for good
    }
};
struct LogBinsI {
    const int *thr;   // thr[b] for b = 1..nbins-1 (thr[0] = 0)
    int nbins;
    float lscale;     // nbins / log2(ratio^2): thr[b] ~ ratio^(2b/nbins), so b ~ log2(n2) * lscale
    __device__ __forceinline__ LogBinsI staged(double *s) const {
        int *t = reinterpret_cast<int *>(s);
        for (int i = threadIdx.x; i < nbins; i += blockDim.x) t[i] = thr[i];
        return LogBinsI{t, nbins, lscale};
    }
    static constexpr int kSmemTable = 1;   // nbins ints fit in nbins doubles
    // The bin from the logarithm's estimate (off by at most a step or two),
    // then moved to the largest b with thr[b] <= n2: the table decides.
    __device__ __forceinline__ int bin(int n2) const {
        if (n2 == 0) return -1;
        int b = min(nbins - 1, max(0, (int)(__log2f((float)n2) * lscale)));
        while (b + 1 < nbins && thr[b + 1] <= n2) ++b;
        while (b > 0 && thr[b] > n2) --b;
        return b;
    }
    // bin of n2 >= the n2 that gave b (bins only grow along a row)
    __device__ __forceinline__ int next(int b, int n2) const {
        if (b < 0) return bin(n2);
        while (b + 1 < nbins && thr[b + 1] <= n2) ++b;
        return b;
    }
    // the least n2' > n2 whose bin may differ from b = bin(n2)
    __device__ __forceinline__ int upper(int b, int) const {
        if (b >= 0) return b + 1 < nbins ? thr[b + 1] : INT_MAX;
        return 1;   // b < 0 only at the origin (n2 = 0)
    }
};

// Float-float values (hi + lo, about 48 significant bits): the warp-level sums
// run in FP32, where GB300 issues ~60x more operations per cycle than in FP64.
// Sums use Knuth's error-free two-sum (TAOCP vol. 2, 4.2.2) in a fixed order.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    err = __fadd_rn(err, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, err);
    return FF{hi, __fsub_rn(err, __fsub_rn(hi, s))};
}
__device__ __forceinline__ FF ff_shfl_up(FF a, int o) {
    return FF{__shfl_up_sync(0xffffffffu, a.hi, o), __shfl_up_sync(0xffffffffu, a.lo, o)};
}
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }

// Add x to a float-float histogram slot (a double-sized slot holding hi, lo):
// the per-warp histograms stay in FP32 arithmetic, off GB300's FP64 pipe, and
// are widened to double once per block. All values added are non-negative.
__device__ __forceinline__ void ff_acc(double *slot, FF x) {
    float2 *s = reinterpret_cast<float2 *>(slot);
    const float2 h = *s;
    const FF r = ff_add(FF{h.x, h.y}, x);
    *s = make_float2(r.hi, r.lo);
}

// w * a for w = 1 or 2 (exact in float-float)
__device__ __forceinline__ FF ff_scale(FF a, float w) { return FF{w * a.hi, w * a.lo}; }

// |n| = sqrt(n2) as float-float. Below 2^24, n2 is exact in float: hi = sqrtf
// (correctly rounded), the residual n2 - hi^2 is exact in float (that of a
// correctly rounded square root always is) and lo = residual / (2 hi). Above
// (large 2D lattices), from the double square root (used by a binning's first
// call only).
__device__ __forceinline__ FF mode_norm(int n2) {
    if (n2 < (1 << 24)) {
        const float n2f = (float)n2;
        const float shi = sqrtf(n2f);
        return FF{shi, shi > 0.0f ? __fdiv_rn(fmaf(-shi, shi, n2f), 2.0f * shi) : 0.0f};
    }
    const double rd = sqrt((double)n2);
    const float shi = (float)rd;
    return FF{shi, (float)(rd - (double)shi)};
}

// The least s >= 0 with s^2 >= m (m < 2^31). The estimate m * rsqrt(m) is
// within a few 1e-7 of sqrt(m) relatively (the approximate reciprocal square
// root and the rounding of m to float), so within 0.02 of it for m < 2^31; the
// corrections are exact in 32-bit unsigned arithmetic (s <= 46341).
__device__ __forceinline__ int ceil_isqrt(int m) {
    if (m <= 0) return 0;
    const float fm = (float)m;
    unsigned s = (unsigned)(fm * rsqrtf(fm));
    const unsigned um = (unsigned)m;
    while (s * s < um) ++s;
    while (s > 0 && (s - 1) * (s - 1) >= um) --s;
    return (int)s;
}

// Weighted power of the modes ix in [a, e) of one bin's run, added to v:
// weight 2 (the mode and its conjugate of the half spectrum), 1 for the row's
// first (ix = 0) and last (ix = N/2 = nh - 1) mode. Summed in FP32 in blocks
// of at most 16 modes (relative error below 16 ulp of a block's sum, all terms
// being non-negative), a full block of 16 unrolled in four chains (modes k
// mod 4, then chains 0+2 and 1+3), a shorter one in two (even and odd modes),
// each block added to v in float-float. s: the staged row segment that starts
// at mode s0.
__device__ __forceinline__ FF run_power(const float2 *s, int s0, int a, int e, int nh, FF v) {
    if (a == 0) {
        const float2 f = s[-s0];
        v = ff_add(v, FF{fmaf(f.x, f.x, f.y * f.y), 0.f});
        a = 1;
    }
    const int eh = e == nh ? nh - 1 : e;
    while (a < eh) {
        const int ce = min(eh, a + 16);
        float t0 = 0.f, t1 = 0.f;
        if (ce - a == 16) {
            const float2 *q = s + (a - s0);
            float t2 = 0.f, t3 = 0.f;
#pragma unroll
            for (int k = 0; k < 16; k += 4) {
                const float2 f0 = q[k], f1 = q[k + 1], f2 = q[k + 2], f3 = q[k + 3];
                t0 = fmaf(f0.x, f0.x, fmaf(f0.y, f0.y, t0));
                t1 = fmaf(f1.x, f1.x, fmaf(f1.y, f1.y, t1));
                t2 = fmaf(f2.x, f2.x, fmaf(f2.y, f2.y, t2));
                t3 = fmaf(f3.x, f3.x, fmaf(f3.y, f3.y, t3));
            }
            t0 += t2;
            t1 += t3;
            a = ce;
        } else {
            for (; a + 1 < ce; a += 2) {
                const float2 f = s[a - s0], g = s[a + 1 - s0];
                t0 = fmaf(f.x, f.x, fmaf(f.y, f.y, t0));
                t1 = fmaf(g.x, g.x, fmaf(g.y, g.y, t1));
            }
            if (a < ce) {
                const float2 f = s[a - s0];
                t0 = fmaf(f.x, f.x, fmaf(f.y, f.y, t0));
                ++a;
            }
        }
        v = ff_add(v, FF{2.f * (t0 + t1), 0.f});
    }
    if (e == nh) {
        const float2 f = s[nh - 1 - s0];
        v = ff_add(v, FF{fmaf(f.x, f.x, f.y * f.y), 0.f});
    }
    return v;
}

template <typename T> __device__ __forceinline__ FF mode_power(const typename Cplx<T>::type &f);
template <> __device__ __forceinline__ FF mode_power<float>(const float2 &f) { return FF{fmaf(f.x, f.x, f.y * f.y), 0.0f}; }
template <> __device__ __forceinline__ FF mode_power<double>(const double2 &f) {
    const double v = f.x * f.x + f.y * f.y;
    const float hi = __double2float_rn(v);
    return FF{hi, __double2float_rn(v - (double)hi)};
}

// Run-length binner over the rows of the half spectrum. Along a row |n|^2 =
// ix^2 + c only grows, so the bins do too: each lane takes a contiguous slice
// of the (shared-memory staged) row and sums runs of one bin in registers
// (float-float). A run strictly inside a lane's slice belongs to that lane
// alone and goes straight into the warp's histogram; a lane's first run may
// continue runs of the lanes before it (equal bins sit in consecutive lanes:
// one segmented scan of 5 shuffle steps), and its last run has a bin no other
// lane's last run has. Every bin thus receives its sums in an order fixed by
// the data: results are the same run to run and for an ensemble member alone.
// Rows are taken in groups that share every bin boundary (see the unit loop).
// Per-warp histograms (float-float slots), block partial rows in double and
// k_bin_final3 (three rows: power, |n|, count). With KS false only the power
// row is summed and held (the |n| and count rows, which depend on N and the
// bin edges alone, come out zero; the power sums are the same bits either
// way: the host gives both kinds of call the same segments, passes and grid).
// Large spectra run in pieces that fit shared memory: a row of the half
// spectrum is taken in segments of `seg` modes (each segment is binned like a
// row: bins still only grow along it), and the bins in passes of `nbp`, this
// launch summing bins b0 .. b0+nbp-1 only (modes of other bins are skipped).
// One segment per row and one pass is the common case.
template <typename T, typename B, bool KS>
__global__ void __launch_bounds__(128, 8) k_bin_runs(const typename Cplx<T>::type *__restrict__ F, int N, int ndims,
                                                  B binner, int nbins, int seg, int b0, int nbp,
                                                  double *__restrict__ partials, int *derr) {
    typedef typename Cplx<T>::type C;
    constexpr bool kRuns = sizeof(T) == 4;   // FP32 modes: whole runs per bin lookup
    // [4 warps][HR][nbp] histograms, bin table, [4 warps][2][sbuf] staging buffers, [4 warps][2] mbarriers
    extern __shared__ double hist[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nh = N / 2 + 1;
    const int nseg = (nh + seg - 1) / seg;
    const int b1 = b0 + nbp;
    constexpr int HR = KS ? 3 : 1;   // histogram rows: power (and |n|, count on a binning's first call)
    for (int i = threadIdx.x; i < 4 * HR * nbp; i += blockDim.x) hist[i] = 0.0;
    const B bins = binner.staged(hist + 4 * HR * nbp);
    // Row segments arrive by bulk copies into two staging buffers per warp: the
    // next unit's copy is in flight while this one is binned. A buffer holds a
    // segment and up to one mode either side (the copy starts and ends on 16
    // bytes); buffers start 16-byte aligned, the warp's two mbarriers follow.
    const int sbuf = (seg + 3) & ~1;
    C *stg = reinterpret_cast<C *>(hist + ((4 * HR * nbp + B::kSmemTable * nbins + 1) & ~1)) + (size_t)w * 2 * sbuf;
    uint64_t *bars = reinterpret_cast<uint64_t *>(reinterpret_cast<C *>(hist + ((4 * HR * nbp + B::kSmemTable * nbins + 1) & ~1)) +
                                                  (size_t)4 * 2 * sbuf) + 2 * w;
    if (lane == 0) {
        mbar_init(smem_u32(&bars[0]), 1);
        mbar_init(smem_u32(&bars[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    double *hp = hist + (size_t)w * HR * nbp;   // indexed by bin - b0
    double *hk = hp + nbp;
    double *hc = hk + nbp;
    auto in_pass = [&](int bb) { return bb >= b0 && bb < b1; };
    // A unit is (group, segment si). A group holds the rows whose frequencies
    // are (+-gz, +-gy), gz and gy in 0 .. N/2 (2D: +-gy): up to four rows with
    // the same c = fy^2 + fz^2, hence the same bin at every x. A lane's slice
    // has the same runs in each of them, so its first and last runs are summed
    // over the group's rows in registers, and the segmented scan and the
    // histogram updates run once per group instead of once per row. There are
    // (N/2 + 1)^2 nseg < 2^31 units (3D N <= 4096; 2D far fewer): int.
    const int gh = N / 2 + 1;
    const int units = (ndims == 3 ? gh * gh : gh) * nseg;
    const int nwarps = gridDim.x * 4;
    // The mode offset of unit uu's copy below its first mode (FP32 modes are 8
    // bytes; the array and every row-segment copy start on 16 bytes), and the
    // copy itself (lane 0). The copy ends on 16 bytes too: at most one mode
    // past the segment, which exists (the array holds an even number of modes,
    // so the last segment's copy ends exactly at its end).
    auto unit_off = [&](int rr, int ssi) -> int {
        return sizeof(C) == 8 ? (int)(((unsigned)rr * (unsigned)nh + (unsigned)(ssi * seg)) & 1u) : 0;
    };
    auto issue = [&](int rr, int ssi, int buf) {
        const int ss0 = ssi * seg, ssl = min(seg, nh - ss0);
        const int off = unit_off(rr, ssi);
        const uint32_t bytes = (uint32_t)(((size_t)(ssl + off) * sizeof(C) + 15) & ~(size_t)15);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // after this warp's reads of the buffer
        mbar_expect_tx(smem_u32(&bars[buf]), bytes);
        bulk_load(smem_u32(stg + (size_t)buf * sbuf), F + (int64_t)rr * nh + ss0 - off, bytes, smem_u32(&bars[buf]));
    };
    struct Unit {
        int gz, gy, si, ny, cnt;   // ny: 1 or 2 values of y; cnt: rows in the group
    };
    auto unit_at = [&](int uu) {
        const int g = uu / nseg;
        Unit q;
        q.si = uu - g * nseg;
        q.gz = ndims == 3 ? g / gh : 0;
        q.gy = ndims == 3 ? g - q.gz * gh : g;
        q.ny = (q.gy == 0 || 2 * q.gy == N) ? 1 : 2;
        q.cnt = q.ny * ((ndims == 2 || q.gz == 0 || 2 * q.gz == N) ? 1 : 2);
        return q;
    };
    // row m of a group: y = gy, then N - gy; z = gz, then N - gz
    auto row_of = [&](const Unit &q, int m) {
        const int jz = m >= q.ny ? 1 : 0, jy = m - jz * q.ny;
        const int iy = jy ? N - q.gy : q.gy;
        return ndims == 2 ? iy : (jz ? N - q.gz : q.gz) * N + iy;
    };
    const int ufirst = blockIdx.x * 4 + w;
    if (lane == 0 && ufirst < units) {
        const Unit q0 = unit_at(ufirst);
        issue(row_of(q0, 0), q0.si, 0);
    }
    int it = 0;            // row copies taken by this warp: buffer it & 1, phase (it >> 1) & 1
    bool ok = true;
    bool more = false;     // a copy after the current one is in flight
    for (int u = ufirst; u < units; u += nwarps) {
        const Unit q = unit_at(u);
        const int s0 = q.si * seg, sl = min(seg, nh - s0);
        // Lane slices of an odd number of modes: lanes reading mode k of their
        // slices at once are 2 * chunk words apart, which spreads them over the
        // 32 banks (an even chunk such as 16 put every lane on one bank).
        const int chunk = ((sl + 31) / 32) | 1;
        const int lo = s0 + min(sl, lane * chunk), hi = s0 + min(sl, lane * chunk + chunk);
        // |n|^2 = ix^2 + fy^2 (+ fz^2) <= 2 (N/2)^2 < 2^31 in 2D (N <= 32768), 3 (N/2)^2 in 3D (N <= 4096): int
        const int c2 = q.gy * q.gy + q.gz * q.gz;
        int fb = -1, lb = -1;   // the slice's first and last runs' bins, the same in every row of the group
        int nr = 0, r1b = -1, r1e = 0, r2b = -1;   // FP32: the slice's runs in the group's first row (count, bins, first end)
        FF fv{0.f, 0.f}, fk{0.f, 0.f}, lv{0.f, 0.f}, lk{0.f, 0.f};
        int fc = 0, lc = 0;
        for (int m = 0; m < q.cnt; ++m, ++it) {
            const int cur = it & 1;
            __syncwarp();   // every lane is done with the other buffer (the previous row)
            more = m + 1 < q.cnt || u + nwarps < units;
            if (lane == 0 && more) {
                if (m + 1 < q.cnt) {
                    issue(row_of(q, m + 1), q.si, cur ^ 1);
                } else {
                    const Unit qn = unit_at(u + nwarps);
                    issue(row_of(qn, 0), qn.si, cur ^ 1);
                }
            }
            ok = __all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[cur]), (uint32_t)((it >> 1) & 1)));
            if (!ok) break;
            const C *stage = stg + (size_t)cur * sbuf + unit_off(row_of(q, m), q.si);
            int b = -1;
            int up = 0;          // the bin is looked up again once n2 reaches this
            bool inp = false;    // in_pass(b)
            bool first = true;   // no run of this row has ended yet
            FF v{0.f, 0.f}, kk{0.f, 0.f};
            int c = 0;
            // a run of bin b ended inside the slice: the row's first (summed over
            // the group's rows), or one strictly inside, straight to the histogram
            auto close_run = [&]() {
                if (b < 0) return;
                if (first) {
                    fb = b;
                    fv = ff_add(fv, v);
                    if constexpr (KS) {
                        fk = ff_add(fk, kk);
                        fc += c;
                    }
                    first = false;
                } else if (in_pass(b)) {
                    ff_acc(hp + (b - b0), v);
                    if constexpr (KS) {
                        ff_acc(hk + (b - b0), kk);
                        ff_acc(hc + (b - b0), FF{(float)c, 0.f});
                    }
                }
            };
            if constexpr (kRuns) {
                // FP32: jump from run to run. A run ends where n2 reaches `up`, at
                // ix = ceil(sqrt(up - c2)); its power is summed by run_power, so a
                // binning's first call (KS: also |n| and the mode count, per mode)
                // and its later calls give the same power sums. The group's later
                // rows have the first row's runs: a slice of one or two runs
                // replays them without the bin lookups.
                const float2 *sf = reinterpret_cast<const float2 *>(stage);
                if (m > 0 && nr <= 2) {
                    if (nr > 0) {
                        b = r1b;
                        if (b >= 0 && in_pass(b)) v = run_power(sf, s0, lo, r1e, nh, v);
                    }
                    if (nr == 2) {
                        close_run();
                        b = r2b;
                        v = FF{0.f, 0.f};
                        if (b >= 0 && in_pass(b)) v = run_power(sf, s0, r1e, hi, nh, v);
                    }
                } else
                for (int ix = lo; ix < hi;) {
                    const int n2 = ix * ix + c2;
                    if (n2 >= up) {   // every pass but the first: n2 reached the bound of b's run
                        const int nb = bins.next(b, n2);
                        up = bins.upper(nb, n2);
                        close_run();
                        b = nb;
                        v = kk = FF{0.f, 0.f};
                        c = 0;
                    }
                    const int e = up == INT_MAX ? hi : min(hi, ceil_isqrt(up - c2));
                    if (m == 0) {   // the slice's runs, for the group's later rows
                        if (nr == 0) {
                            r1b = b;
                            r1e = e;
                        } else if (nr == 1) {
                            r2b = b;
                        }
                        ++nr;
                    }
                    if (b >= 0 && in_pass(b)) {
                        v = run_power(sf, s0, ix, e, nh, v);
                        // the |n| sums and mode counts are the same in every row of
                        // the group: the first row's, times the rows (1, 2 or 4: exact)
                        if constexpr (KS)
                            if (m == 0)
                                for (int a = ix; a < e; ++a) {
                                    const int wt = ((a == 0 || 2 * a == N) ? 1 : 2) * q.cnt;
                                    kk = ff_add(kk, ff_scale(mode_norm(a * a + c2), (float)wt));
                                    c += wt;
                                }
                    }
                    ix = e;
                }
            } else
            for (int ix = lo; ix < hi; ++ix) {
                const int n2 = ix * ix + c2;
                int nb = b;
                if (n2 >= up) {
                    nb = bins.next(b, n2);
                    up = bins.upper(nb, n2);
                }
                if (nb != b) {
                    close_run();
                    b = nb;
                    inp = in_pass(b);
                    v = kk = FF{0.f, 0.f};
                    c = 0;
                }
                if (inp) {
                    const int wt = (ix == 0 || 2 * ix == N) ? 1 : 2;
                    const float fw = (float)wt;   // x1 or x2: exact in float-float
                    const FF p = mode_power<T>(stage[ix - s0]);
                    v = ff_add(v, FF{fw * p.hi, fw * p.lo});
                    if constexpr (KS) {
                        if (m == 0) {   // as above: the first row's |n| and count, times the rows
                            kk = ff_add(kk, ff_scale(mode_norm(n2), fw * (float)q.cnt));
                            c += wt * q.cnt;
                        }
                    }
                }
            }
            if (b >= 0) {   // the open run: the row's first if none ended, else the slice's last
                if (first) {
                    fb = b;
                    fv = ff_add(fv, v);
                    if constexpr (KS) {
                        fk = ff_add(fk, kk);
                        fc += c;
                    }
                } else {
                    lb = b;
                    lv = ff_add(lv, v);
                    if constexpr (KS) {
                        lk = ff_add(lk, kk);
                        lc += c;
                    }
                }
            }
        }
        if (!ok) break;
        __syncwarp();   // inside runs are in; the staged rows are no longer read
        // first runs: inclusive segmented scan over lanes with equal bins
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int ob = __shfl_up_sync(0xffffffffu, fb, o);
            const FF ov = ff_shfl_up(fv, o);
            FF ok{0.f, 0.f};
            int oc = 0;
            if constexpr (KS) {
                ok = ff_shfl_up(fk, o);
                oc = __shfl_up_sync(0xffffffffu, fc, o);
            }
            if (lane >= o && fb >= 0 && ob == fb) {
                fv = ff_add(ov, fv);
                if constexpr (KS) {
                    fk = ff_add(ok, fk);
                    fc += oc;
                }
            }
        }
        const int nextb = __shfl_down_sync(0xffffffffu, fb, 1);
        if (in_pass(fb) && (lane == 31 || nextb != fb)) {
            ff_acc(hp + (fb - b0), fv);
            if constexpr (KS) {
                ff_acc(hk + (fb - b0), fk);
                ff_acc(hc + (fb - b0), FF{(float)fc, 0.f});
            }
        }
        __syncwarp();
        if (in_pass(lb)) {
            ff_acc(hp + (lb - b0), lv);
            if constexpr (KS) {
                ff_acc(hk + (lb - b0), lk);
                ff_acc(hc + (lb - b0), FF{(float)lc, 0.f});
            }
        }
        __syncwarp();
    }
    if (!ok) {   // a copy never completed: flag it, then wait (bounded) for this warp's copies in flight
        if (lane == 0) {
            atomicOr(derr, DEVERR_TIMEOUT);
            mbar_wait_bounded(smem_u32(&bars[it & 1]), (uint32_t)((it >> 1) & 1));
            if (more) mbar_wait_bounded(smem_u32(&bars[(it + 1) & 1]), (uint32_t)(((it + 1) >> 1) & 1));
        }
        __syncwarp();
    }
    __syncthreads();
    for (int bn = threadIdx.x; bn < nbp; bn += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double acc = 0.0;
            for (int ww = 0; ww < 4 && q < HR; ++ww) {
                const float2 h = reinterpret_cast<const float2 *>(hist)[(size_t)ww * HR * nbp + (size_t)q * nbp + bn];
                acc += (double)h.x + (double)h.y;
            }
            partials[((int64_t)blockIdx.x * 3 + q) * nbp + bn] = acc;
        }
    }
}

// gather a real field into fft_in: src = complex array, component comp
template <typename T>
__global__ void k_gather_real(const T *__restrict__ src_cplx, int comp, T *__restrict__ dst, int64_t len) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) dst[m] = src_cplx[2 * m + comp];
}

// f = |phi| dtheta/dtau = (psi2 pi1 - psi1 pi2) / (tau |psi|)
template <typename T>
__global__ void k_gather_axion(const typename Cplx<T>::type *__restrict__ psi, const typename Cplx<T>::type *__restrict__ pi,
                               T *__restrict__ dst, int64_t len, double tau) {
    const T itau = (T)(1.0 / tau);
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        auto a = psi[m];
        auto p = pi[m];
        dst[m] = axion_f<T>(a.x, a.y, p.x, p.y, itau);
    }
}

// ---- staged z-column kernels (the axion field for every stencil radius,
// the energies for radius 2..4)
//
// f = |phi| dtheta/dtau = (psi2 pi1 - psi1 pi2) / (tau |psi|) and the energies
// need pi_n = pih + dt/2 K(psi), formed per site with k_sync_pi's arithmetic
// (stencil_at's order) and never stored. A block marches 32 x 8 columns
// through z with every load from DRAM staged by cp.async into shared memory,
// so the loads in flight hold no registers:
// per plane, the block's psi tile with an R-wide periodic halo (the in-plane
// neighbours) and its own pih values, in rings of S = A + 1 slots issued A
// planes ahead, with one block barrier per site. Each thread keeps its
// column's psi in a register ring for the z-neighbours, filled from the
// staged tiles R + 1 planes ahead. Reading the 4R in-plane neighbours from
// global memory left the warps waiting on L1/L2 latency, and register-held
// column loads could keep too few bytes in flight for the DRAM rate.

__device__ __forceinline__ void cp_async_ca(uint32_t dst, const void *src, int bytes) {
    if (bytes == 16) asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int P>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(P) : "memory"); }

// Geometry of the radius-R march. A plane tile is TH = 8 + 2R rows of
// TW = 32 + 2RX elements (the block's columns and their periodic halo);
// float tiles are copied in 16-byte pairs, so their x halo RX is R rounded
// up to even (N is even, so a pair never straddles the periodic edge).
template <typename T, int R>
struct ZMarch {
    typedef typename Cplx<T>::type C;
    static constexpr int VEC = sizeof(T) == 4 ? 2 : 1;           // elements per copy
    static constexpr int RX = VEC == 2 ? (R + 1) & ~1 : R;
    static constexpr int TW = 32 + 2 * RX, TH = 8 + 2 * R, E = TW * TH, NCP = E / VEC, PER = (NCP + 255) / 256;
    static constexpr int A = R + 2 + (sizeof(T) == 4 ? 2 : 0);   // planes staged ahead
    static constexpr int S = A + 1;                               // ring slots
    static constexpr int W = 2 * R + 2;                           // register ring (planes z-R-1 .. z+R)
    static constexpr size_t SMEM = (size_t)S * (E + 256) * sizeof(C);
    static constexpr int MINB = sizeof(T) == 8 ? 2 : (R == 4 ? 3 : 4);   // blocks per SM the smem allows
};

// The copies one thread makes of each plane: tile copies t, t + 256, ...
// (offsets within a plane, -1 past the tile) and its own pih value.
template <typename T, int R>
struct ZStage {
    typedef ZMarch<T, R> M;
    typedef typename M::C C;
    int goff[M::PER];
    __device__ __forceinline__ ZStage(int bx0, int by0, int N) {
#pragma unroll
        for (int k = 0; k < M::PER; ++k) {
            const int q = (int)threadIdx.x + 256 * k, e = q * M::VEC;
            goff[k] = -1;
            if (q < M::NCP) {
                int gx = (bx0 - M::RX + e % M::TW) % N, gy = (by0 - R + e / M::TW) % N;
                if (gx < 0) gx += N;
                if (gy < 0) gy += N;
                goff[k] = gy * N + gx;
            }
        }
    }
    // stage the plane at element offset po into ring slot s
    __device__ __forceinline__ void issue(const C *psi, const C *pih, int64_t po, int s, C *tiles, C *pown,
                                          bool active, int col) const {
        C *slot = tiles + s * M::E;
#pragma unroll
        for (int k = 0; k < M::PER; ++k)
            if (goff[k] >= 0)
                cp_async_ca(smem_u32(slot + ((int)threadIdx.x + 256 * k) * M::VEC), psi + po + goff[k],
                            (int)(M::VEC * sizeof(C)));
        if (active) cp_async_ca(smem_u32(pown + s * 256 + threadIdx.x), pih + po + col, (int)sizeof(C));
    }
};

// The radius-R stencil sums of a column's site in plane z, in stencil_at's
// order (coefficient 0 times the centre; per distance l the x pair plus the y
// pair, plus the z pair, added with one fma), so pi_n keeps k_sync_pi's bits.
// t points at the site in its plane tile (row length TW); the column's plane
// z + d is zr[(g + d) % W].
template <typename T, int R, int W, int TW>
__device__ __forceinline__ void tile_stencil(const typename Cplx<T>::type *t, const typename Cplx<T>::type (&zr)[W],
                                             int g, T &L1, T &L2) {
    const auto &ctr = zr[g % W];
    if constexpr (R == 1) {   // lap7's order, as stencil_at forms radius 1
        const auto xm = t[-1], xp = t[1], ym = t[-TW], yp = t[TW];
        const auto &zm = zr[(g + W - 1) % W], &zp = zr[(g + 1) % W];
        L1 = lap7<T>(ctr.x, xm.x, xp.x, ym.x, yp.x, zm.x, zp.x);
        L2 = lap7<T>(ctr.y, xm.y, xp.y, ym.y, yp.y, zm.y, zp.y);
        return;
    }
    T a1 = (T)stencil_coef(R - 1, 3, 0) * ctr.x, a2 = (T)stencil_coef(R - 1, 3, 0) * ctr.y;
#pragma unroll
    for (int l = 1; l <= R; ++l) {
        const auto xm = t[-l], xp = t[l], ym = t[-l * TW], yp = t[l * TW];
        const auto &zm = zr[(g + W - l) % W], &zp = zr[(g + l) % W];
        T s1 = (xm.x + xp.x) + (ym.x + yp.x), s2 = (xm.y + xp.y) + (ym.y + yp.y);
        s1 = s1 + (zm.x + zp.x);
        s2 = s2 + (zm.y + zp.y);
        const T cl = (T)stencil_coef(R - 1, 3, l);
        a1 = fma(cl, s1, a1);
        a2 = fma(cl, s2, a2);
    }
    L1 = a1;
    L2 = a2;
}

// The march itself, shared by the radius-R axion field and energies: for
// each site of the thread's column (threads past the lattice's edge take part
// in the staging and barriers only) it forms pi_n with k_sync_pi's
// arithmetic and calls site(h, z, zc, zp, p, t): the site's psi, psi of plane
// z + 1, pi_n and its place in the staged tile. The register ring holds
// planes z-R-1 .. z+R at site z; plane z+R+1 replaces plane z-R-1 from the
// staged tile, so the ring has period W and the march runs W sites per trip
// (no register moves). N > 2R and A <= 2R + 2 <= N, so a plane index past
// the end wraps with one subtraction.
template <typename T, int R, class Site>
__device__ __forceinline__ void zcol_march(const typename Cplx<T>::type *__restrict__ psi,
                                           const typename Cplx<T>::type *__restrict__ pih, int N, int fresh,
                                           const StepCoefs<T> &c, Site &&site) {
    typedef ZMarch<T, R> M;
    typedef typename M::C C;
    constexpr int W = M::W, A = M::A, S = M::S;
    extern __shared__ __align__(16) unsigned char zsm[];
    C *tiles = reinterpret_cast<C *>(zsm), *pown = tiles + S * M::E;
    const int nbx = (N + 31) / 32, bx0 = (int)(blockIdx.x % nbx) * 32, by0 = (int)(blockIdx.x / nbx) * 8;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, x = bx0 + tx, y = by0 + ty;
    const bool active = x < N && y < N;
    const int col = active ? y * N + x : 0;
    const ZStage<T, R> st(bx0, by0, N);
    const int64_t NN = (int64_t)N * N, len = NN * N;
#pragma unroll
    for (int a = 0; a < A; ++a) {
        st.issue(psi, pih, a * NN, a, tiles, pown, active, col);
        cp_async_commit();
    }
    C zr[W];   // at a trip's start z0: zr[j] = plane z0 - R - 1 + j
#pragma unroll
    for (int j = 1; j < W; ++j) zr[j] = psi[(int64_t)(j <= R ? j - R - 1 + N : j - R - 1) * NN + col];
    zr[0] = zr[1];   // plane -R-1 is never read
    const int cidx = (ty + R) * M::TW + tx + M::RX;
    int slot = 0, rslot = R + 1;   // ring slots of planes z and z + R + 1
    int64_t pa = A * NN;
    for (int z0 = 0; z0 < N; z0 += W) {
#pragma unroll
        for (int h = 0; h < W; ++h) {
            const int z = z0 + h;
            if (z < N) {   // uniform over the block
                cp_async_wait<A - R - 2>();   // this thread's copies of planes <= z + R + 1 are in
                __syncthreads();              // everyone's are; slot (z - 1) is no longer read
                st.issue(psi, pih, z + A < N ? pa : pa - len, slot == 0 ? A : slot - 1, tiles, pown, active, col);
                cp_async_commit();
                pa += NN;
                if (active) {
                    const C *ts = tiles + slot * M::E + cidx;
                    zr[h] = tiles[rslot * M::E + cidx];   // plane z + R + 1 over plane z - R - 1
                    C p = pown[slot * 256 + threadIdx.x];
                    const C zc = zr[(h + R + 1) % W], zp = zr[(h + R + 2) % W];
                    if (!fresh) {   // a fresh state holds pi_0 itself (the reference's ker is zero)
                        T L1, L2;
                        tile_stencil<T, R, W, M::TW>(ts, zr, h + R + 1, L1, L2);
                        sync_pi_site<T>(zc.x, zc.y, L1, L2, p.x, p.y, c);
                    }
                    site(h, z, zc, zp, p, ts);
                }
                slot = slot == A ? 0 : slot + 1;
                rslot = rslot == A ? 0 : rslot + 1;
            }
        }
    }
    cp_async_wait<0>();
}

// The axion field of the kinetic spectrum for a stencil of radius R = 1..4:
// 20 B per site from DRAM (psi, pih in, f out), against 44 B and per-site
// 64-bit index arithmetic through k_sync_pi and scratch. (At radius 1 a
// march with the column's psi and pih loaded into registers two planes ahead
// and the in-plane neighbours read from global memory ran 3.7 against 3.5 ms
// at 1024^3.)
template <typename T, int R>
__global__ void __launch_bounds__(256, (ZMarch<T, R>::MINB)) k_axion_zcol_r(const typename Cplx<T>::type *__restrict__ psi,
                                                                 const typename Cplx<T>::type *__restrict__ pih,
                                                                 T *__restrict__ dst, const double *clock, int N,
                                                                 double dt, double inv_dx2, double lambda,
                                                                 double T0sq3, int prs, int fresh, double tau) {
    typedef typename Cplx<T>::type C;
    const StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, inv_dx2, lambda, T0sq3, prs, 0);
    const T itau = (T)(1.0 / tau);
    const int nbx = (N + 31) / 32;
    const int x = (int)(blockIdx.x % nbx) * 32 + (threadIdx.x & 31), y = (int)(blockIdx.x / nbx) * 8 + (threadIdx.x >> 5);
    const int64_t NN = (int64_t)N * N;
    T *out = dst + (x < N && y < N ? y * N + x : 0);
    zcol_march<T, R>(psi, pih, N, fresh, c, [&](int, int z, const C &zc, const C &, const C &p, const C *) {
        out[z * NN] = axion_f<T>(zc.x, zc.y, p.x, p.y, itau);
    });
}

// The axion field of a 3D finite-difference lattice into fft_in, by the
// z-column kernel of its stencil radius.
template <typename T>
static void axion_zcol_t(Lattice *L) {
    typedef typename Cplx<T>::type C;
    const axs_params &p = L->p;
    const int N = p.N;
    const double dx = p.space_step, T0 = p.T_initial;
    const C *f = (const C *)L->psi[L->cur], *q = (const C *)L->pih;
    T *dst = (T *)L->fft_in;
    const double *clk = L->dclock + L->cur;
    const double dt = p.time_step, idx2 = 1.0 / (dx * dx), la = p.lambda, t3 = (T0 * T0) / 3.0;
    const int g = ((N + 31) / 32) * ((N + 7) / 8);   // blocks of 32 x 8 columns
    auto radius = [&](auto kern, size_t smem) {
        AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<g, 256, smem, L->stream>>>(f, q, dst, clk, N, dt, idx2, la, t3, p.prs, L->fresh, L->tau);
    };
    switch (p.stencil_setting) {
    case 0: radius(k_axion_zcol_r<T, 1>, ZMarch<T, 1>::SMEM); break;
    case 1: radius(k_axion_zcol_r<T, 2>, ZMarch<T, 2>::SMEM); break;
    case 2: radius(k_axion_zcol_r<T, 3>, ZMarch<T, 3>::SMEM); break;
    default: radius(k_axion_zcol_r<T, 4>, ZMarch<T, 4>::SMEM); break;
    }
}

static void ensure_fft(Lattice *L) {
    if (L->have_plan) return;
    int N = L->p.N;
    int64_t half = (L->p.NDIMS == 2 ? (int64_t)N : (int64_t)N * N) * (N / 2 + 1);
    L->fft_in = dalloc((size_t)L->length * L->esz);
    L->fft_out = dalloc((size_t)half * 2 * L->esz);
    cufftType ty = L->esz == 4 ? CUFFT_R2C : CUFFT_D2Z;
    if (L->p.NDIMS == 2) AXS_CUFFT(cufftPlan2d(&L->plan_r2c, N, N, ty));
    else AXS_CUFFT(cufftPlan3d(&L->plan_r2c, N, N, N, ty));
    AXS_CUFFT(cufftSetStream(L->plan_r2c, L->stream));
    L->have_plan = true;
}

static void exec_r2c(Lattice *L) {
    AXS_CUFFT(cufftSetStream(L->plan_r2c, L->stream));   // the stream of this call (batched calls use a pool)
    if (L->esz == 4) AXS_CUFFT(cufftExecR2C(L->plan_r2c, (cufftReal *)L->fft_in, (cufftComplex *)L->fft_out));
    else AXS_CUFFT(cufftExecD2Z(L->plan_r2c, (cufftDoubleReal *)L->fft_in, (cufftDoubleComplex *)L->fft_out));
}

// A binning in flight: its result rows land in `host` (3 x nbins doubles,
// pass by pass) when the stream reaches them. The |n| sums and counts of a
// binning (kind, edges) are computed by its first call and reused
// afterwards, when the kernel sums the power alone.
struct BinPending {
    int nbins = 0, nbp = 0, kind = 0;
    bool ks = false;
    std::vector<int> edges;
    const double *host = nullptr;
};

template <typename B>
static BinPending bin_spectrum_enqueue(Lattice *L, const B &binner, int kind, const std::vector<int> &edges, int nbins,
                                       double *host) {
    const Lattice::BinGeom *geom = nullptr;
    for (const Lattice::BinGeom &g : L->bin_geom)
        if (g.kind == kind && g.edges == edges) geom = &g;
    const bool ks = geom == nullptr;
    const int N = L->p.N;
    const int nh = N / 2 + 1;
    // shared memory of one block: 4 warp histograms of nbp bins x 3 rows (1 row
    // when only the power is summed), the bin table, two staging buffers of a
    // segment of seg modes per warp. Whole rows and every bin in one pass when
    // they fit (up to N ~ 1500); else segments of 2048 modes, then passes over
    // the bins.
    // k_bin_runs' layout: histograms (hr rows), table, 4 x 2 buffers, 8 mbarriers
    auto smem_of = [&](int nbp, int seg, int hr) {
        return (size_t)((4 * hr * nbp + B::kSmemTable * nbins + 1) & ~1) * sizeof(double) +
               (size_t)4 * 2 * ((seg + 3) & ~1) * 2 * L->esz + 8 * sizeof(uint64_t);
    };
    // The segments, the bin passes and the grid fix which modes each lane and
    // each warp sums, hence the bits: they follow from the first call's layout
    // (three histogram rows) for every call, so later calls (one row) give the
    // first call's power sums exactly.
    const size_t cap = 200 * 1024;
    int nbp = nbins, seg = nh;
    while (smem_of(nbp, seg, 3) > cap) {
        if (seg > 2048) seg = 2048;
        else if (nbp > 512) nbp = (nbp + 1) / 2;
        else if (seg > 256) seg /= 2;
        else fail(AXS_ERR_ARG, "spectrum binning with %d bins does not fit shared memory", nbins);
    }
    const size_t sm = smem_of(nbp, seg, ks ? 3 : 1);
    // as many 4-warp blocks as the later calls' layout fits on the SMs (up to 16
    // per SM): the per-warp histograms leave this kernel latency-bound at low
    // occupancy; the first call runs the same grid in more waves
    int per_sm = (int)std::max<size_t>(1, std::min<size_t>(16, cap / std::max<size_t>(smem_of(nbp, seg, 1), 1)));
    // k_bin_runs' units: groups of up to four rows (+-gz, +-gy) times segments
    const int64_t groups = L->p.NDIMS == 2 ? (int64_t)nh : (int64_t)nh * nh;
    const int64_t units = groups * ((nh + seg - 1) / seg);
    if (units >= ((int64_t)1 << 31)) fail(AXS_ERR_ARG, "spectrum of N = %d: too many row groups", N);
    int nblk = (int)std::min<int64_t>((int64_t)num_sms() * per_sm, (units + 3) / 4);   // whole units per warp
    double *part = (double *)lattice_tmp(L, 1, (size_t)nblk * 3 * nbp * sizeof(double) + (size_t)3 * nbp * sizeof(double));
    double *out = part + (size_t)nblk * 3 * nbp;
    auto kern = L->esz == 4 ? (ks ? (const void *)k_bin_runs<float, B, true> : (const void *)k_bin_runs<float, B, false>)
                            : (ks ? (const void *)k_bin_runs<double, B, true> : (const void *)k_bin_runs<double, B, false>);
    if (sm > 48 * 1024) AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    for (int b0 = 0; b0 < nbins; b0 += nbp) {
        const int nb = std::min(nbp, nbins - b0);
        if (L->esz == 4) {
            if (ks) k_bin_runs<float, B, true><<<nblk, 128, sm, L->stream>>>((const float2 *)L->fft_out, N, L->p.NDIMS, binner, nbins, seg, b0, nb, part, L->derr);
            else k_bin_runs<float, B, false><<<nblk, 128, sm, L->stream>>>((const float2 *)L->fft_out, N, L->p.NDIMS, binner, nbins, seg, b0, nb, part, L->derr);
        } else {
            if (ks) k_bin_runs<double, B, true><<<nblk, 128, sm, L->stream>>>((const double2 *)L->fft_out, N, L->p.NDIMS, binner, nbins, seg, b0, nb, part, L->derr);
            else k_bin_runs<double, B, false><<<nblk, 128, sm, L->stream>>>((const double2 *)L->fft_out, N, L->p.NDIMS, binner, nbins, seg, b0, nb, part, L->derr);
        }
        AXS_CUDA(cudaGetLastError());
        k_bin_final3<<<nb, 256, 0, L->stream>>>(part, nblk, nb, out);
        AXS_CUDA(cudaGetLastError());
        count_launches(2);
        // rows (power, |n|, count) of this pass at host[3 b0 ..]; the next pass
        // overwrites `out` only after this copy (stream order)
        AXS_CUDA(cudaMemcpyAsync(host + 3 * (size_t)b0, out, 3 * (size_t)nb * sizeof(double), cudaMemcpyDeviceToHost,
                                 L->stream));
    }
    // the lattice's error flag into the slot after the rows (host holds 3 nbins + 1 doubles)
    AXS_CUDA(cudaMemcpyAsync(host + 3 * (size_t)nbins, L->derr, sizeof(int), cudaMemcpyDeviceToHost, L->stream));
    BinPending pd;
    pd.nbins = nbins;
    pd.nbp = nbp;
    pd.kind = kind;
    pd.ks = ks;
    pd.edges = edges;
    pd.host = host;
    return pd;
}

// After the stream reached the copies: per-bin power sums, |n| sums and
// counts (the latter two from the lattice's cache of this binning, filled by
// its first call).
static void bin_spectrum_finish(Lattice *L, const BinPending &pd, std::vector<double> &psum, std::vector<double> &nsum,
                                std::vector<unsigned long long> &cnt) {
    const int nbins = pd.nbins;
    int flag = 0;   // the error flag copied after the rows (k_bin_runs' row copies complete on bounded waits)
    memcpy(&flag, pd.host + 3 * (size_t)nbins, sizeof(int));
    if (flag & DEVERR_TIMEOUT) {
        AXS_CUDA(cudaMemsetAsync(L->derr, 0, sizeof(int), L->stream));
        fail(AXS_ERR_TIMEOUT, "the spectrum binner gave up waiting for a row copy; the spectrum was not computed");
    }
    psum.assign(nbins, 0.0);
    std::vector<double> nk(pd.ks ? nbins : 0, 0.0), cc(pd.ks ? nbins : 0, 0.0);
    for (int b0 = 0; b0 < nbins; b0 += pd.nbp) {
        const int nb = std::min(pd.nbp, nbins - b0);
        const double *h = pd.host + 3 * (size_t)b0;
        for (int b = 0; b < nb; ++b) {
            psum[b0 + b] = h[b];
            if (pd.ks) {
                nk[b0 + b] = h[(size_t)nb + b];
                cc[b0 + b] = h[2 * (size_t)nb + b];
            }
        }
    }
    const Lattice::BinGeom *geom = nullptr;
    for (const Lattice::BinGeom &g : L->bin_geom)
        if (g.kind == pd.kind && g.edges == pd.edges) geom = &g;
    if (!geom) {
        if (!pd.ks) fail(AXS_ERR_STATE, "internal: spectrum binning geometry missing");
        Lattice::BinGeom g;
        g.kind = pd.kind;
        g.edges = pd.edges;
        g.nsum = nk;
        g.cnt.resize(nbins);
        for (int b = 0; b < nbins; ++b) g.cnt[b] = (unsigned long long)cc[b];
        if (L->bin_geom.size() >= 8) L->bin_geom.erase(L->bin_geom.begin());
        L->bin_geom.push_back(std::move(g));
        geom = &L->bin_geom.back();
    }
    nsum = geom->nsum;
    cnt = geom->cnt;
}

// Bin the current fft_out; returns per-bin sums (pk, |n|) and weighted counts.
// A pageable destination makes each copy complete before the call returns.
template <typename B>
static void bin_spectrum(Lattice *L, const B &binner, int kind, const std::vector<int> &edges, int nbins,
                         std::vector<double> &psum, std::vector<double> &nsum, std::vector<unsigned long long> &cnt) {
    std::vector<double> h(3 * (size_t)nbins + 1);   // rows, then the error flag
    const BinPending pd = bin_spectrum_enqueue(L, binner, kind, edges, nbins, h.data());
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    bin_spectrum_finish(L, pd, psum, nsum, cnt);
}

void powerspec(Lattice *L, int field, double *pk, double *ks, int *count) {
    ensure_fft(L);
    const void *src;
    int comp = field & 1;
    if (field <= AXS_PHI2) src = L->psi[L->cur];
    else { launch_sync_pi(L); src = L->scratch; }
    int g = grid_cap(L->length, 256, 16);
    if (L->esz == 4) k_gather_real<float><<<g, 256, 0, L->stream>>>((const float *)src, comp, (float *)L->fft_in, L->length);
    else k_gather_real<double><<<g, 256, 0, L->stream>>>((const double *)src, comp, (double *)L->fft_in, L->length);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
    exec_r2c(L);
    int N = L->p.N;
    int nb = N / 2;
    std::vector<double> ps, ns;
    std::vector<unsigned long long> c;
    bin_spectrum(L, RefBinsI{N / 2}, 0, std::vector<int>{nb}, nb, ps, ns, c);
    float Lf = N * L->p.space_step;                     // pk_estimation.cpp:41
    for (int b = 0; b < nb; ++b) {                      // pk_estimation.cpp:117-121 / 195-199
        double k = ns[b] / (double)(int)c[b];
        double p = ps[b];
        if (L->p.NDIMS == 2) p /= 2.0f * M_PI * k;
        else p /= 4.0f * M_PI * (k * k);
        k *= 2.0f * M_PI / Lf;
        pk[b] = p;
        ks[b] = k;
        count[b] = (int)c[b];
    }
}

// The axion spectrum of one lattice in flight: the field, the transform and
// the binning are enqueued; thresholds travel from `thr_host` (page-locked
// for a truly asynchronous copy, or nullptr for the lattice's own pageable
// copy) and the result rows land in `host` (3 x nbins doubles).
struct AxionPending {
    BinPending bin;
    std::vector<int> thr;
};

static AxionPending axion_spectrum_enqueue(Lattice *L, int nbins, double *host, int *thr_host) {
    if (nbins < 1) fail(AXS_ERR_ARG, "nbins must be >= 1");
    if (L->p.form != 0) fail(AXS_ERR_STATE, "the axion kinetic spectrum is defined on the field-rescaled variables (form 0)");
    ensure_fft(L);
    if (L->p.NDIMS == 3 && L->p.laplacian == 0) {
        if (L->esz == 4) axion_zcol_t<float>(L);
        else axion_zcol_t<double>(L);
    } else {
        launch_sync_pi(L);
        int g = grid_cap(L->length, 256, 16);
        if (L->esz == 4)
            k_gather_axion<float><<<g, 256, 0, L->stream>>>((const float2 *)L->psi[L->cur], (const float2 *)L->scratch,
                                                            (float *)L->fft_in, L->length, L->tau);
        else
            k_gather_axion<double><<<g, 256, 0, L->stream>>>((const double2 *)L->psi[L->cur],
                                                             (const double2 *)L->scratch, (double *)L->fft_in, L->length,
                                                             L->tau);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
    exec_r2c(L);
    const int d = L->p.NDIMS, N = L->p.N;
    const double ratio = sqrt((double)d) * (double)N / 2.0;
    // bin b starts at |n| = t_b = ratio^(b/nbins); for integer n2 the test
    // n2 >= t_b^2 is n2 >= ceil(t_b^2)
    AxionPending pd;
    pd.thr.assign(nbins, 0);
    for (int b = 1; b < nbins; ++b) { double t = exp(log(ratio) * (double)b / (double)nbins); pd.thr[b] = (int)ceil(t * t); }
    int *de2 = (int *)lattice_tmp(L, 2, nbins * sizeof(int));
    const int *src = pd.thr.data();
    if (thr_host) {
        memcpy(thr_host, pd.thr.data(), nbins * sizeof(int));
        src = thr_host;
    }
    AXS_CUDA(cudaMemcpyAsync(de2, src, nbins * sizeof(int), cudaMemcpyHostToDevice, L->stream));
    pd.bin = bin_spectrum_enqueue(L, LogBinsI{de2, nbins, (float)((double)nbins / log2(ratio * ratio))}, 1, pd.thr,
                                  nbins, host);
    return pd;
}

static void axion_spectrum_finish(Lattice *L, const AxionPending &pd, double *kmean, double *pk, int64_t *count) {
    const int nbins = pd.bin.nbins, d = L->p.NDIMS, N = L->p.N;
    std::vector<double> ps, ns;
    std::vector<unsigned long long> c;
    bin_spectrum_finish(L, pd.bin, ps, ns, c);
    const double Ld = (double)N * (double)L->p.space_step;
    const double norm = pow(Ld, d) / pow((double)L->length, 2.0);
    for (int b = 0; b < nbins; ++b) {
        count[b] = (int64_t)c[b];
        if (c[b]) {
            kmean[b] = 2.0 * M_PI * (ns[b] / (double)c[b]) / Ld;
            pk[b] = norm * ps[b] / (double)c[b];
        } else {
            kmean[b] = 0.0;
            pk[b] = 0.0;
        }
    }
}

void axion_spectrum(Lattice *L, int nbins, double *kmean, double *pk, int64_t *count) {
    std::vector<double> h(3 * (size_t)std::max(nbins, 1) + 1);   // rows, then the error flag
    const AxionPending pd = axion_spectrum_enqueue(L, nbins, h.data(), nullptr);
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    axion_spectrum_finish(L, pd, kmean, pk, count);
}

// ---------------------------------------------------------------- batched over an ensemble
//
// Per member the same kernels as the single-lattice calls, enqueued back to
// back on the ensemble's stream with the results copied into one page-locked
// buffer, and a single synchronisation: the members' results are the bits of
// the per-member calls.

static void *ensemble_pinned(Ensemble *E, size_t bytes) {
    if (E->hpin_cap < bytes) {
        if (E->hpin) AXS_CUDA(cudaFreeHost(E->hpin));
        E->hpin = nullptr;
        E->hpin_cap = 0;
        AXS_CUDA(cudaHostAlloc(&E->hpin, bytes, cudaHostAllocDefault));
        E->hpin_cap = bytes;
    }
    return E->hpin;
}

// Members run on a pool of streams forked from and joined back into the
// ensemble's stream; `fn(L)` enqueues one member's work on L->stream.
template <typename Fn>
static void ensemble_fan_out(Ensemble *E, Fn fn) {
    const size_t n = E->members.size(), k = std::min<size_t>(8, n);
    while (E->pool.size() < k) {
        cudaStream_t s;
        cudaEvent_t ev;
        AXS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        E->pool.push_back(s);
        AXS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        E->pool_ev.push_back(ev);
    }
    if (!E->ev_fork) AXS_CUDA(cudaEventCreateWithFlags(&E->ev_fork, cudaEventDisableTiming));
    AXS_CUDA(cudaEventRecord(E->ev_fork, E->stream));
    for (size_t j = 0; j < k; ++j) AXS_CUDA(cudaStreamWaitEvent(E->pool[j], E->ev_fork, 0));
    auto join = [&] {   // the ensemble's stream waits for everything enqueued on the pool
        for (size_t j = 0; j < k; ++j) {
            cudaEventRecord(E->pool_ev[j], E->pool[j]);
            cudaStreamWaitEvent(E->stream, E->pool_ev[j], 0);
        }
    };
    for (size_t i = 0; i < n; ++i) {
        Lattice *L = E->members[i];
        cudaStream_t own = L->stream;
        L->stream = E->pool[i % k];
        try {
            fn(L, i);
        } catch (...) {
            L->stream = own;
            join();   // later work on the ensemble stays ordered after what did get enqueued
            throw;
        }
        L->stream = own;
    }
    join();
    AXS_CUDA(cudaGetLastError());
}

void ensemble_release_pool(Ensemble *E) {
    for (cudaStream_t s : E->pool) cudaStreamDestroy(s);
    for (cudaEvent_t e : E->pool_ev) cudaEventDestroy(e);
    if (E->ev_fork) cudaEventDestroy(E->ev_fork);
    E->pool.clear();
    E->pool_ev.clear();
    E->ev_fork = nullptr;
}

void ensemble_find_strings(Ensemble *E, int64_t *nplaq, int64_t *ncores) {
    const size_t n = E->members.size();
    if (E->members[0]->p.NDIMS == 2) {   // 2D: the neighbouring-pair count needs each member's list
        for (size_t i = 0; i < n; ++i) find_strings(E->members[i], nullptr, nullptr, &nplaq[i], &ncores[i]);
        return;
    }
    int64_t *hc = (int64_t *)ensemble_pinned(E, n * sizeof(int64_t));
    ensemble_fan_out(E, [&](Lattice *L, size_t i) {
        ensure_mask(L);
        const double accept = (double)(0.5f * (1.0f - L->p.thr / 100.0f));   // string_finding.cpp:8,40
        AXS_CUDA(cudaMemsetAsync(L->dcount, 0, 2 * sizeof(int64_t), L->stream));
        unsigned long long *cnt = (unsigned long long *)L->dcount;
        if (L->esz == 4) launch_cores<float>(L, false, accept, cnt);
        else launch_cores<double>(L, false, accept, cnt);
        AXS_CUDA(cudaMemcpyAsync(&hc[i], L->dcount, sizeof(int64_t), cudaMemcpyDeviceToHost, L->stream));
    });
    AXS_CUDA(cudaStreamSynchronize(E->stream));
    for (size_t i = 0; i < n; ++i) {
        Lattice *L = E->members[i];
        L->last_nplaq = hc[i];
        L->list_valid = false;
        nplaq[i] = hc[i];
        ncores[i] = hc[i];   // 3D: every flagged plaquette counts (s_run.cpp:112-131)
    }
}

void ensemble_axion_spectrum(Ensemble *E, int nbins, double *kmean, double *pk, int64_t *count) {
    if (nbins < 1) fail(AXS_ERR_ARG, "nbins must be >= 1");
    const size_t n = E->members.size();
    // per member: the rows and the error flag (3 nbins + 1 doubles), then the bin thresholds
    const size_t per = (3 * (size_t)nbins + 2) * sizeof(double) + (((size_t)nbins * sizeof(int) + 15) & ~(size_t)15);
    char *base = (char *)ensemble_pinned(E, n * per);
    std::vector<AxionPending> pend(n);
    ensemble_fan_out(E, [&](Lattice *L, size_t i) {
        double *h = (double *)(base + i * per);
        int *t = (int *)(base + i * per + (3 * (size_t)nbins + 2) * sizeof(double));
        pend[i] = axion_spectrum_enqueue(L, nbins, h, t);
    });
    AXS_CUDA(cudaStreamSynchronize(E->stream));
    for (size_t i = 0; i < n; ++i)
        axion_spectrum_finish(E->members[i], pend[i], kmean + i * nbins, pk + i * nbins, count + i * nbins);
}

// ============================================================== reductions

// Kahan-compensated accumulator for the FP32 path; plain double for FP64.
template <typename T> struct Acc;
template <> struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <> struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};

// |theta| = |atan2(phi1, phi2)| for the background mean: float fields take
// fast_atan2 (within 5e-7 rad, a tenth of the float means' 2e-6 tolerance
// relative to a mean |theta| near pi/2), FP64 fields abs_phi_theta (below).
__device__ __forceinline__ float abs_theta(float a, float b) { return fabsf(fast_atan2(a, b)); }
// FP64 fields: |atan2(a, b)| and |(a, b)| to double precision at a fraction
// of the library's FP64 cost (GB300's FP64 pipe bounds the FP64 means). The
// float angle picks the nearest of the angles k pi/128 (k = -128 .. 128); the
// vector (b, a) is rotated by -k pi/128 with that angle's double cosine and
// sine (formed on the host) to (x, y), a small angle from the x axis. With
// u = y/x (the reciprocal from the float one by two Newton-Raphson steps,
// within an ulp), |u| < 0.0125: the remainder angle atan(u) is the Taylor
// series to u^7 and |(a, b)| = x sqrt(1 + u^2) the binomial series to u^6
// (truncations below 3e-17). Vectors outside that (a zero, tiny, huge or
// non-finite component) take the library's atan2 and square root. The angle
// is brought back to [-pi, pi] before its magnitude.
__device__ double2 g_theta_rot[257];   // (cos, sin) of k pi/128 at index k + 128
__device__ __forceinline__ void abs_phi_theta(double a, double b, double &aphi, double &ath) {
    const float t0 = fast_atan2((float)a, (float)b);
    const int k = __float2int_rn(t0 * 40.743665431525205f);   // 128 / pi
    const double2 cs = g_theta_rot[k + 128];
    const double x = fma(b, cs.x, a * cs.y), y = fma(a, cs.x, -(b * cs.y));
    if (x > 1e-30 && x < 1e30) {
        double r = (double)__frcp_rn((float)x);
        r = fma(r, fma(-x, r, 1.0), r);
        r = fma(r, fma(-x, r, 1.0), r);
        const double u = y * r;
        if (fabs(u) < 0.0125) {
            const double u2 = u * u;
            double q = fma(u2, -1.0 / 7.0, 1.0 / 5.0);
            q = fma(u2, q, -1.0 / 3.0);
            double t = fma(u * u2, q, u) + (double)k * (3.141592653589793 / 128.0);
            if (t > 3.141592653589793) t -= 6.283185307179586;
            else if (t < -3.141592653589793) t += 6.283185307179586;
            ath = fabs(t);
            double w = fma(u2, 1.0 / 16.0, -1.0 / 8.0);
            w = fma(u2, w, 0.5);
            aphi = x * fma(u2, w, 1.0);
            return;
        }
    }
    ath = fabs(atan2(a, b));
    aphi = sqrt(a * a + b * b);
}
// the rotation table of abs_phi_theta, once per device
static void ensure_theta_table() {
    static PerDevice done;
    done.get([] {
        double2 tab[257];
        for (int k = -128; k <= 128; ++k) {
            const double t = (double)k * (3.141592653589793 / 128.0);
            tab[k + 128] = make_double2(cos(t), sin(t));
        }
        AXS_CUDA(cudaMemcpyToSymbol(g_theta_rot, tab, sizeof(tab)));
        return 1;
    });
}

// Two neighbouring sites q = 2i, 2i+1 (one 16-byte load for float fields).
__device__ __forceinline__ void load_pair(const float2 *__restrict__ a, int64_t i, float2 (&v)[2]) {
    const float4 w = reinterpret_cast<const float4 *>(a)[i];
    v[0] = make_float2(w.x, w.y);
    v[1] = make_float2(w.z, w.w);
}
__device__ __forceinline__ void load_pair(const double2 *__restrict__ a, int64_t i, double2 (&v)[2]) {
    v[0] = a[2 * i];
    v[1] = a[2 * i + 1];
}

// Background means (s_run.cpp:135-150) of psi and pi_n in one streaming pass
// over psi and pih, for every lattice kind. pi_n = pih + dt/2 K(psi) needs no
// neighbours for its mean: on a periodic lattice every site is the neighbour
// of as many sites as the stencil has points, so the Laplacian part of K sums
// to W sum(psi), W the sum of the stencil's weights (zero for the 5- and
// 7-point stencils, ~1e-7 for the reference's float weights of radius 2-4;
// the spectral operator has no k = 0 mode). The kernel sums the mean of pih
// plus the local part of the half kick and the host adds dt/2 W/dx^2 mean(psi).
// That equals the mean of the per-site pi_n up to rounding (FP64: within
// 1e-12 of the oracle's per-site sums) and reads 16 B per site instead of
// k_sync_pi's 24 B plus 16 B. Two sites per trip
// (N^d is even), their terms added before one compensated add; the grid is
// one wave of resident blocks.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) k_background(const typename Cplx<T>::type *__restrict__ psi,
                                                       const typename Cplx<T>::type *__restrict__ pih,
                                                       const double *clock, int64_t len, double dt, double lambda,
                                                       double T0sq3, int prs, int form, int fresh,
                                                       double *__restrict__ partials) {
    typedef typename Cplx<T>::type C;
    const StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, 0.0, lambda, T0sq3, prs, form);
    Acc<T> a[6];
    const int64_t npair = len >> 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    auto trip = [&](C (&f)[2], C (&p)[2]) {
        T t[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) t[k] = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!fresh) sync_pi_site<T>(f[h].x, f[h].y, (T)0, (T)0, p[h].x, p[h].y, c);   // a fresh pih is pi_0
            t[0] += f[h].x;
            t[1] += f[h].y;
            t[2] += p[h].x;
            t[3] += p[h].y;
            if constexpr (sizeof(T) == 8) {
                double ap, at;
                abs_phi_theta(f[h].x, f[h].y, ap, at);
                t[4] += at;
                t[5] += ap;
            } else {
                t[4] += abs_theta(f[h].x, f[h].y);
                t[5] += sqrt(f[h].x * f[h].x + f[h].y * f[h].y);
            }
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) a[k].add(t[k]);
    };
    // the loads of two trips are in flight before either is summed (the same
    // trips in the same order as one at a time: the same sums)
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < npair; i += 2 * stride) {
        C f0[2], p0[2], f1[2], p1[2];
        load_pair(psi, i, f0);
        load_pair(pih, i, p0);
        load_pair(psi, i + stride, f1);
        load_pair(pih, i + stride, p1);
        trip(f0, p0);
        trip(f1, p1);
    }
    if (i < npair) {
        C f[2], p[2];
        load_pair(psi, i, f);
        load_pair(pih, i, p);
        trip(f, p);
    }
    double v[6];
    for (int k = 0; k < 6; ++k) v[k] = a[k].value();
    block_reduce_store<6>(v, partials);
}

template <typename T, int ND>
__global__ void __launch_bounds__(256) k_energies(const typename Cplx<T>::type *__restrict__ psi,
                                                  const typename Cplx<T>::type *__restrict__ pi, int N, int64_t len,
                                                  double tau, double dx, double lam_eff, double *__restrict__ partials) {
    Acc<T> a[3];
    const T it = (T)(1.0 / tau), idx = (T)(1.0 / dx), q = (T)(0.25 * lam_eff);
    const int64_t NN = (int64_t)N * N;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        auto s = psi[m];
        auto p = pi[m];
        T f1 = s.x * it, f2 = s.y * it;
        T d1 = (p.x - f1) * it, d2 = (p.y - f2) * it;
        a[0].add((T)0.5 * (d1 * d1 + d2 * d2));
        int64_t x = m % N, nb[3];
        int nn;
        if (ND == 2) {
            int64_t y = m / N;
            nb[0] = m - x + (x + 1 == N ? 0 : x + 1);
            nb[1] = (y + 1 == N ? 0 : y + 1) * N + x;
            nn = 2;
        } else {
            int64_t y = (m / N) % N, z = m / NN;
            nb[0] = m - x + (x + 1 == N ? 0 : x + 1);
            nb[1] = z * NN + (y + 1 == N ? 0 : y + 1) * N + x;
            nb[2] = (z + 1 == N ? 0 : z + 1) * NN + y * N + x;
            nn = 3;
        }
        T g = 0;
        for (int k = 0; k < nn; ++k) {
            auto o = psi[nb[k]];
            T g1 = (o.x * it - f1) * idx, g2 = (o.y * it - f2) * idx;
            g += g1 * g1 + g2 * g2;
        }
        a[1].add((T)0.5 * g);
        T r = f1 * f1 + f2 * f2 - (T)1;
        a[2].add(q * r * r);
    }
    double v[3];
    for (int k = 0; k < 3; ++k) v[k] = a[k].value();
    block_reduce_store<3>(v, partials);
}

// Energy densities of a 3D radius-1 lattice in one pass over psi and pih
// (the kinetic term is quadratic in pi_n, so unlike the background means it
// needs the full half kick per site). pi_n is formed per site with
// k_sync_pi's arithmetic and never stored, and each thread marches one (x, y)
// column through z: psi's z-neighbours stay in registers
// and the in-plane neighbours (also the x+1, y+1 forward differences of the
// gradient energy; z+1 is the next plane in registers) come from the
// neighbouring threads' loads of the same plane. 16 B from DRAM per site
// instead of 40 B through scratch. Blocks are 256 threads over 32 x 8 columns
// (threads past the edge add nothing); each block writes its partial sums at
// its index, so the totals are deterministic.
//
// The kernel is issue-bound, so the march is arranged for few instructions per
// site: three column pointers advance a plane per site (wrapping once, near the
// end), two sites per trip (N is even) so the register rotation is renaming,
// the two sites' terms are added in plain T before one compensated add, and
// the constant factors (1/2 tau^-2, 1/2 (tau dx)^-2, lambda/4) are applied to
// the column sums: the sums are of (pi - psi/tau)^2, of the squared
// differences of psi and of (|psi|^2/tau^2 - 1)^2. Float fields fit 64
// registers (4 CTAs per SM). N >= 4.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) k_energies_zcol(const typename Cplx<T>::type *__restrict__ psi,
                                                         const typename Cplx<T>::type *__restrict__ pih,
                                                         double *__restrict__ partials, const double *clock, int N,
                                                         double dt, double inv_dx2, double lambda, double T0sq3,
                                                         int prs, int form, int fresh, double tau, double dx,
                                                         double lam_eff) {
    typedef typename Cplx<T>::type C;
    constexpr int K = 3;
    Acc<T> acc[K];
    const int bx = (N + 31) / 32;
    const int x = (int)(blockIdx.x % bx) * 32 + (threadIdx.x & 31), y = (int)(blockIdx.x / bx) * 8 + (threadIdx.x >> 5);
    if (x < N && y < N) {
        const StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, inv_dx2, lambda, T0sq3, prs, form);
        const T it = (T)(1.0 / tau), it2 = (T)(1.0 / (tau * tau));
        const int64_t NN = (int64_t)N * N, len = NN * N;
        const int col = y * N + x;
        const int xm = y * N + (x == 0 ? N - 1 : x - 1) - col, xp = y * N + (x == N - 1 ? 0 : x + 1) - col;
        const int ym = (y == 0 ? N - 1 : y - 1) * N + x - col, yp = (y == N - 1 ? 0 : y + 1) * N + x - col;
        // column values: psi planes z-1, z, z+1 in use, z+2 and z+3 in flight;
        // pih plane z in use, z+1 and z+2 in flight; neighbours of plane z in
        // use (loaded a site earlier), those of z+1 in flight
        C zm = psi[(N - 1) * NN + col], zc = psi[col];
        C zp = psi[NN + col], zq = psi[2 * NN + col];
        C pc = pih[col], pq = pih[NN + col];
        C a, b, d, e;
        { a = psi[col + xm]; b = psi[col + xp]; d = psi[col + ym]; e = psi[col + yp]; }
        const C *s3 = psi + 3 * NN + col, *p2 = pih + 2 * NN + col, *s1 = psi + NN + col;   // planes z+3, z+2, z+1
        for (int z = 0; z < N; z += 2) {
            T t[K];
#pragma unroll
            for (int k = 0; k < K; ++k) t[k] = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int zz = z + h;
                const C zr = *(zz + 3 < N ? s3 : s3 - len);
                const C pr = *(zz + 2 < N ? p2 : p2 - len);
                const C *q1 = zz + 1 < N ? s1 : s1 - len;
                s3 += NN;
                p2 += NN;
                s1 += NN;
                C na, nb, nd, ne;
                { na = q1[xm]; nb = q1[xp]; nd = q1[ym]; ne = q1[yp]; }
                C p = pc;
                if (!fresh) {   // a fresh state holds pi_0 itself (the reference's ker is zero)
                    const T L1 = lap7<T>(zc.x, a.x, b.x, d.x, e.x, zm.x, zp.x);
                    const T L2 = lap7<T>(zc.y, a.y, b.y, d.y, e.y, zm.y, zp.y);
                    sync_pi_site<T>(zc.x, zc.y, L1, L2, p.x, p.y, c);
                }
                {   // differences in the order x, y, z
                    const T e1 = fma(-zc.x, it, p.x), e2 = fma(-zc.y, it, p.y);
                    t[0] += fma(e1, e1, e2 * e2);
                    T g1 = b.x - zc.x, g2 = b.y - zc.y;
                    T g = fma(g1, g1, g2 * g2);
                    g1 = e.x - zc.x;
                    g2 = e.y - zc.y;
                    g = fma(g1, g1, fma(g2, g2, g));
                    g1 = zp.x - zc.x;
                    g2 = zp.y - zc.y;
                    t[1] += fma(g1, g1, fma(g2, g2, g));
                    const T r = fma(it2, fma(zc.x, zc.x, zc.y * zc.y), (T)-1);
                    t[2] += r * r;
                }
                a = na; b = nb; d = nd; e = ne;
                zm = zc;
                zc = zp;
                zp = zq;
                zq = zr;
                pc = pq;
                pq = pr;
            }
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k].add(t[k]);
        }
    }
    double v[K];
    for (int k = 0; k < K; ++k) v[k] = acc[k].value();
    v[0] *= 0.5 / (tau * tau);
    v[1] *= 0.5 / (tau * tau * dx * dx);
    v[2] *= 0.25 * lam_eff;
    block_reduce_store<K>(v, partials);
}

// k_energies_zcol for the radius-R stencils (R = 2..4), on k_axion_zcol_r's
// march: x+1 and y+1 of the gradient are the stencil's distance-1 neighbours
// in the staged tile, z+1 the next ring plane. Two sites' terms go into one
// compensated add, as in k_energies_zcol. 16 B from DRAM per site.
template <typename T, int R>
__global__ void __launch_bounds__(256, (ZMarch<T, R>::MINB)) k_energies_zcol_r(const typename Cplx<T>::type *__restrict__ psi,
                                                                    const typename Cplx<T>::type *__restrict__ pih,
                                                                    double *__restrict__ partials, const double *clock,
                                                                    int N, double dt, double inv_dx2, double lambda,
                                                                    double T0sq3, int prs, int form, int fresh,
                                                                    double tau, double dx, double lam_eff) {
    typedef typename Cplx<T>::type C;
    constexpr int K = 3, TW = ZMarch<T, R>::TW;
    Acc<T> acc[K];
    T t[K] = {0, 0, 0};
    const StepCoefs<T> c = make_coefs<T>(*clock, dt, 0.5 * dt, inv_dx2, lambda, T0sq3, prs, form);
    const T it = (T)(1.0 / tau), it2 = (T)(1.0 / (tau * tau));
    zcol_march<T, R>(psi, pih, N, fresh, c, [&](int h, int, const C &zc, const C &zp, const C &p, const C *ts) {
        const C b = ts[1], e = ts[TW];   // differences in the order x, y, z
        const T e1 = fma(-zc.x, it, p.x), e2 = fma(-zc.y, it, p.y);
        t[0] += fma(e1, e1, e2 * e2);
        T g1 = b.x - zc.x, g2 = b.y - zc.y;
        T g = fma(g1, g1, g2 * g2);
        g1 = e.x - zc.x;
        g2 = e.y - zc.y;
        g = fma(g1, g1, fma(g2, g2, g));
        g1 = zp.x - zc.x;
        g2 = zp.y - zc.y;
        t[1] += fma(g1, g1, fma(g2, g2, g));
        const T r = fma(it2, fma(zc.x, zc.x, zc.y * zc.y), (T)-1);
        t[2] += r * r;
        if (h & 1) {   // W is even, so sites pair up within a trip
#pragma unroll
            for (int k = 0; k < K; ++k) {
                acc[k].add(t[k]);
                t[k] = 0;
            }
        }
    });
    double v[K];
    for (int k = 0; k < K; ++k) v[k] = acc[k].value();
    v[0] *= 0.5 / (tau * tau);
    v[1] *= 0.5 / (tau * tau * dx * dx);
    v[2] *= 0.25 * lam_eff;
    block_reduce_store<K>(v, partials);
}

template <typename T>
__global__ void k_finite(const T *__restrict__ a, int64_t n, int *flag) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) bad |= !isfinite(a[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

static double *ensure_partials(Lattice *L, int nblocks, int K) {
    size_t need = (size_t)nblocks * K;
    if (!L->dpartials || L->partials_cap < need) {
        dfree(L->dpartials);
        L->dpartials = nullptr;
        L->partials_cap = std::max<size_t>(need, 4096);
        L->dpartials = (double *)dalloc(L->partials_cap * sizeof(double));
    }
    return L->dpartials;
}

// The z-column energies serve 3D lattices with a finite-difference Laplacian
// (any radius); 2D and the spectral Laplacian form pi_n in scratch first.
static bool energies_zcol(const Lattice *L) { return L->p.NDIMS == 3 && L->p.laplacian == 0; }

template <typename T>
static void energies_zcol_t(Lattice *L, double *part, int g, double lam) {
    typedef typename Cplx<T>::type C;
    const axs_params &p = L->p;
    const double dx = p.space_step, T0 = p.T_initial;
    const C *f = (const C *)L->psi[L->cur], *q = (const C *)L->pih;
    const double *clk = L->dclock + L->cur;
    const double dt = p.time_step, idx2 = 1.0 / (dx * dx), la = p.lambda, t3 = (T0 * T0) / 3.0;
    auto radius = [&](auto kern, size_t smem) {
        AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<g, 256, smem, L->stream>>>(f, q, part, clk, p.N, dt, idx2, la, t3, p.prs, p.form, L->fresh, L->tau, dx, lam);
    };
    switch (p.stencil_setting) {
    case 0: k_energies_zcol<T><<<g, 256, 0, L->stream>>>(f, q, part, clk, p.N, dt, idx2, la, t3, p.prs, p.form, L->fresh, L->tau, dx, lam); break;
    case 1: radius(k_energies_zcol_r<T, 2>, ZMarch<T, 2>::SMEM); break;
    case 2: radius(k_energies_zcol_r<T, 3>, ZMarch<T, 3>::SMEM); break;
    default: radius(k_energies_zcol_r<T, 4>, ZMarch<T, 4>::SMEM); break;
    }
}
static int zcol_blocks(int N) { return ((N + 31) / 32) * ((N + 7) / 8); }

void background(Lattice *L, double out[6]) {
    const axs_params &p = L->p;
    if (L->esz == 8) ensure_theta_table();
    const double T0 = p.T_initial;
    const int resident = L->esz == 4 ? 4 : 2;   // k_background's blocks per SM
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((L->length / 2 + 255) / 256, (int64_t)num_sms() * resident));
    double *part = ensure_partials(L, g, 6);
    if (L->esz == 4)
        k_background<float><<<g, 256, 0, L->stream>>>((const float2 *)L->psi[L->cur], (const float2 *)L->pih,
                                                       L->dclock + L->cur, L->length, (double)p.time_step,
                                                       (double)p.lambda, (T0 * T0) / 3.0, p.prs, p.form, L->fresh, part);
    else
        k_background<double><<<g, 256, 0, L->stream>>>((const double2 *)L->psi[L->cur], (const double2 *)L->pih,
                                                        L->dclock + L->cur, L->length, (double)p.time_step,
                                                        (double)p.lambda, (T0 * T0) / 3.0, p.prs, p.form, L->fresh, part);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
    double s[6];
    sum_partials(part, g, 6, s, L->stream);
    for (int k = 0; k < 6; ++k) out[k] = s[k] / (double)L->length;   // s_run.cpp:149
    if (!L->fresh && p.laplacian == 0) {   // the stencil's share of the half kick: W mean(psi)
        double W = (double)stencil_coef(p.stencil_setting, p.NDIMS, 0);
        for (int l = 1; l <= p.stencil_setting + 1; ++l)
            W += 2.0 * p.NDIMS * (double)stencil_coef(p.stencil_setting, p.NDIMS, l);
        const double dx = p.space_step;
        const double kidx2 = 0.5 * (double)p.time_step / (dx * dx) * (p.form == 1 ? L->tau * L->tau : 1.0);
        out[2] += kidx2 * W * out[0];
        out[3] += kidx2 * W * out[1];
    }
}

void energies(Lattice *L, double out[3]) {
    if (L->p.form != 0) fail(AXS_ERR_STATE, "the energies are defined on the field-rescaled variables (form 0)");
    double lam = (double)L->p.lambda * (L->p.prs ? 1.0 : L->tau * L->tau);
    double dx = L->p.space_step;
    int g;
    double *part;
    if (energies_zcol(L)) {
        g = zcol_blocks(L->p.N);
        part = ensure_partials(L, g, 3);
        if (L->esz == 4) energies_zcol_t<float>(L, part, g, lam);
        else energies_zcol_t<double>(L, part, g, lam);
    } else {
        launch_sync_pi(L);
        g = reduce_grid(L->length);
        part = ensure_partials(L, g, 3);
        const int N = L->p.N;
        const int64_t n = L->length;
        if (L->esz == 4) {
            const float2 *f = (const float2 *)L->psi[L->cur], *q = (const float2 *)L->scratch;
            if (L->p.NDIMS == 2) k_energies<float, 2><<<g, 256, 0, L->stream>>>(f, q, N, n, L->tau, dx, lam, part);
            else k_energies<float, 3><<<g, 256, 0, L->stream>>>(f, q, N, n, L->tau, dx, lam, part);
        } else {
            const double2 *f = (const double2 *)L->psi[L->cur], *q = (const double2 *)L->scratch;
            if (L->p.NDIMS == 2) k_energies<double, 2><<<g, 256, 0, L->stream>>>(f, q, N, n, L->tau, dx, lam, part);
            else k_energies<double, 3><<<g, 256, 0, L->stream>>>(f, q, N, n, L->tau, dx, lam, part);
        }
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
    double s[3];
    sum_partials(part, g, 3, s, L->stream);
    for (int k = 0; k < 3; ++k) out[k] = s[k] / (double)L->length;
}

int check_finite(Lattice *L) {
    int *flag = (int *)(L->dcount ? L->dcount : (L->dcount = (int64_t *)dalloc(4 * sizeof(int64_t)))) + 6;
    AXS_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), L->stream));
    int64_t n = L->length * 2;
    int g = grid_cap(n, 256, 8);
    if (L->esz == 4) {
        k_finite<float><<<g, 256, 0, L->stream>>>((const float *)L->psi[L->cur], n, flag);
        k_finite<float><<<g, 256, 0, L->stream>>>((const float *)L->pih, n, flag);
    } else {
        k_finite<double><<<g, 256, 0, L->stream>>>((const double *)L->psi[L->cur], n, flag);
        k_finite<double><<<g, 256, 0, L->stream>>>((const double *)L->pih, n, flag);
    }
    AXS_CUDA(cudaGetLastError());
    count_launches(2);
    int h = 0;
    AXS_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, L->stream));
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    return h == 0;
}

void analysis_release(Lattice *L) {
    dfree(L->dmask); L->dmask = nullptr;
    dfree(L->dcount); L->dcount = nullptr;
    dfree(L->dlist); L->dlist = nullptr;
    dfree(L->dtheta); L->dtheta = nullptr;
    dfree(L->fft_in); L->fft_in = nullptr;
    dfree(L->fft_out); L->fft_out = nullptr;
    if (L->have_plan) cufftDestroy(L->plan_r2c);
    L->have_plan = false;
    dfree(L->dpartials); L->dpartials = nullptr;
    for (int i = 0; i < 3; ++i) {
        dfree(L->tmp[i]);
        L->tmp[i] = nullptr;
        L->tmp_cap[i] = 0;
    }
}

}  // namespace axs

// ============================================================== allocation-free binner
//
// axs_powerspec_noalloc serves callers that own all device memory themselves
// and cannot let a library call cudaMalloc/cudaFree while they run: hosts that
// budget the whole device up front, frameworks whose caching allocator must
// be the only one handing out device memory, and applications that cannot
// afford the device-wide synchronisation a cudaFree implies. They run their
// own R2C FFT into their own buffer and ask only for the binning.
//
// Its scratch is one file-scope __device__ array (below), held by every GPU
// that loads this library until the process exits. All calls share it and it
// keeps the last call's contents: the per-bin counts are cleared at the start
// of every call and everything else is overwritten, so calls that follow one
// another on a stream are independent, but calls whose kernels overlap on the
// GPU (different streams, no ordering) race on the array and give wrong
// results.

namespace axs {

static constexpr int kNoAllocMaxBins = 1024;   // N/2 bins, so N <= 2048
static constexpr int kNoAllocBlocks = 128;     // binning grid (partials rows)
static constexpr int kNoAllocScratchDoubles = kNoAllocBlocks * 2 * kNoAllocMaxBins   // block partials
                                              + kNoAllocMaxBins;                      // counts (as u64)
// 2 MiB + 8 KiB per device.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

__global__ void k_noalloc_clear(unsigned long long *counts, int nbins) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbins) counts[b] = 0ull;
}

// Sum the block partials in block order and normalise as output_powerspec
// does (pk_estimation.cpp:117-121 / 195-199).
__global__ void k_noalloc_final(const double *__restrict__ partials, int nblocks, int nbins,
                                const unsigned long long *__restrict__ counts, int ndims, float Lf,
                                double *__restrict__ pk, double *__restrict__ ks, int *__restrict__ count) {
    int bn = blockIdx.x * blockDim.x + threadIdx.x;
    if (bn >= nbins) return;
    double sp = 0.0, sk = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        sp += partials[((int64_t)b * 2 + 0) * nbins + bn];
        sk += partials[((int64_t)b * 2 + 1) * nbins + bn];
    }
    int c = (int)counts[bn];
    double k = sk / (double)c;
    double p = sp;
    if (ndims == 2) p /= 2.0f * M_PI * k;
    else p /= 4.0f * M_PI * (k * k);
    k *= 2.0f * M_PI / Lf;
    pk[bn] = p;
    ks[bn] = k;
    count[bn] = c;
}

// Device address of the scratch array on each device, looked up once per
// device by the first call made with that device current.
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[128] = {nullptr};

static double *noalloc_scratch() {
    int dev = 0;
    AXS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) fail(AXS_ERR_ARG, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            fail(AXS_ERR_CUDA, "cudaGetSymbolAddress of the binner scratch failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    return (double *)g_noalloc_ptr[dev];
}

template <typename T>
static void noalloc_bin(const void *spectrum, int ndims, int N, float Lf, double *pk, double *ks, int *count,
                        cudaStream_t st) {
    int nbins = N / 2;
    double *scratch = noalloc_scratch();
    double *partials = scratch;
    unsigned long long *counts = (unsigned long long *)(scratch + (size_t)kNoAllocBlocks * 2 * kNoAllocMaxBins);
    size_t sm = (size_t)4 * 2 * nbins * sizeof(double);
    // Raise the kernel's dynamic shared-memory limit only above the 48 KiB
    // default (never lower it: the allocating binner launches the same kernel).
    if (sm > 48 * 1024)
        AXS_CUDA(cudaFuncSetAttribute(k_bin<T, RefBins>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_noalloc_clear<<<(nbins + 127) / 128, 128, 0, st>>>(counts, nbins);
    k_bin<T, RefBins><<<kNoAllocBlocks, 128, sm, st>>>((const typename Cplx<T>::type *)spectrum, N, ndims,
                                                       RefBins{N / 2}, nbins, partials, counts);
    k_noalloc_final<<<(nbins + 127) / 128, 128, 0, st>>>(partials, kNoAllocBlocks, nbins, counts, ndims, Lf, pk, ks,
                                                         count);
    AXS_CUDA(cudaGetLastError());
    count_launches(3);
}

}  // namespace axs

extern "C" int axs_powerspec_noalloc(const void *spectrum, int NDIMS, int N, int precision, float space_step,
                                     double *pk, double *ks, int *count, void *stream) {
    try {
        if (!spectrum || !pk || !ks || !count) axs::fail(AXS_ERR_ARG, "null pointer argument");
        if (NDIMS != 2 && NDIMS != 3) axs::fail(AXS_ERR_ARG, "NDIMS must be 2 or 3 (got %d)", NDIMS);
        if (N < 4 || (N % 2) != 0) axs::fail(AXS_ERR_ARG, "N must be even and >= 4 (got %d)", N);
        if (N / 2 > axs::kNoAllocMaxBins)
            axs::fail(AXS_ERR_ARG, "N=%d needs %d bins; the allocation-free binner holds at most %d (N <= %d)", N,
                      N / 2, axs::kNoAllocMaxBins, 2 * axs::kNoAllocMaxBins);
        if (precision != AXS_F32 && precision != AXS_F64) axs::fail(AXS_ERR_ARG, "precision must be 32 or 64");
        if (!(space_step > 0.0f)) axs::fail(AXS_ERR_ARG, "space_step must be positive");
        float Lf = N * space_step;
        cudaStream_t st = (cudaStream_t)stream;
        if (precision == AXS_F32) axs::noalloc_bin<float>(spectrum, NDIMS, N, Lf, pk, ks, count, st);
        else axs::noalloc_bin<double>(spectrum, NDIMS, N, Lf, pk, ks, count, st);
    } catch (const axs::Error &e) {
        axs::set_last_error(e.code, e.msg);
        return e.code;
    } catch (...) {
        axs::set_last_error(AXS_ERR_CUDA, "unexpected internal error");
        return AXS_ERR_CUDA;
    }
    return AXS_OK;
}

namespace axs {

// ============================================================== lattice distance
//
// Per field f of (phi1, phi2, phidot1, phidot2): sum (a_f - b_f)^2 and sum b_f^2
// over the lattice, both in FP64 with a fixed reduction order. a and b are the
// synchronised states (psi and pi_n) of two lattices of the same shape, any
// precision each.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_distance(const typename Cplx<TA>::type *__restrict__ pa,
                                                  const typename Cplx<TA>::type *__restrict__ qa,
                                                  const typename Cplx<TB>::type *__restrict__ pb,
                                                  const typename Cplx<TB>::type *__restrict__ qb, int64_t len,
                                                  double *__restrict__ partials) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < len; m += stride) {
        auto a0 = pa[m], a1 = qa[m];
        auto b0 = pb[m], b1 = qb[m];
        double av[4] = {(double)a0.x, (double)a0.y, (double)a1.x, (double)a1.y};
        double bv[4] = {(double)b0.x, (double)b0.y, (double)b1.x, (double)b1.y};
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            double d = av[f] - bv[f];
            acc[2 * f] += d * d;
            acc[2 * f + 1] += bv[f] * bv[f];
        }
    }
    block_reduce_store<8>(acc, partials);
}

void field_distance(Lattice *A, Lattice *B, double out[8]) {
    if (A->p.NDIMS != B->p.NDIMS || A->p.N != B->p.N) fail(AXS_ERR_ARG, "lattices differ in shape");
    launch_sync_pi(A);
    launch_sync_pi(B);
    AXS_CUDA(cudaStreamSynchronize(A->stream));   // B's kernels below run on B's stream
    int g = reduce_grid(A->length);
    double *part = ensure_partials(B, g, 8);
    const void *pa = A->psi[A->cur], *qa = A->scratch, *pb = B->psi[B->cur], *qb = B->scratch;
    if (A->esz == 4 && B->esz == 4) k_distance<float, float><<<g, 256, 0, B->stream>>>((const float2 *)pa, (const float2 *)qa, (const float2 *)pb, (const float2 *)qb, A->length, part);
    else if (A->esz == 4) k_distance<float, double><<<g, 256, 0, B->stream>>>((const float2 *)pa, (const float2 *)qa, (const double2 *)pb, (const double2 *)qb, A->length, part);
    else if (B->esz == 4) k_distance<double, float><<<g, 256, 0, B->stream>>>((const double2 *)pa, (const double2 *)qa, (const float2 *)pb, (const float2 *)qb, A->length, part);
    else k_distance<double, double><<<g, 256, 0, B->stream>>>((const double2 *)pa, (const double2 *)qa, (const double2 *)pb, (const double2 *)qb, A->length, part);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
    sum_partials(part, g, 8, out, B->stream);
}

}  // namespace axs
