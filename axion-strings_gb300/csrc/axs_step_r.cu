// TMA z-march step for the higher-order stencils: stencil_setting 1..3, i.e.
// radius R = 2..4 of build_coefficient_matrix (src/standard/s_integrate.cpp:9-14,
// 5-149). Same organisation as k_zmarch2 (one TMA producer warp, eight
// consumer warps, full/empty mbarriers per ring slot, persistent CTAs taking
// work items from a counter), with
//  * per plane: the psi tile with an R-row periodic y halo (three boxes of R,
//    TY and R rows that never wrap, TY >= R) and x strips of RP sites on both
//    sides (R rounded up to 16 bytes, so strip coordinates stay 16-byte
//    aligned; only the tile rows need them: the stencil is a cross), plus the
//    pih tile;
//  * a ring of S >= 2R + 2 slots holding the planes z-R .. z+R and one in flight;
//    or (ZREG, float fields, one vector per thread: with fewer slots, or with
//    any number when ZR is set) each thread carries psi of its vector at
//    planes z-R .. z+R in registers (radius 4: z-R .. z-1, the rest read from
//    the ring) and the ring holds only the planes z .. z+R still to be centres
//    (S >= R + 2), so S - R - 1 plane loads are in flight per CTA and more
//    CTAs share an SM;
//  * the stencil sum formed exactly as stencil_at forms it for R > 1
//    (c0 * psi, then per l: ((x- + x+) + (y- + y+)) + (z- + z+), fused into the
//    sum with c_l), so every configuration is bit-identical to k_step_generic.
// One pass per step: 32 B (FP32) / 64 B (FP64) per site-update, as for radius 1.
#include <algorithm>
#include <atomic>

#include "axs_internal.h"
#include "axs_tma.cuh"

namespace axs {

template <typename T, int TY, int TXMAX, int S, int R, int ZR = 0>
struct ZRCfg {
    static constexpr int CS = 2 * (int)sizeof(T);
    static constexpr int VS = 16 / CS;                         // sites per 16-byte vector
    static constexpr int EU = CS / 8;                          // tensor-map elements per site
    static constexpr int RP = (R + VS - 1) / VS * VS;          // x-halo sites per side
    static constexpr int NCW = 8;
    static constexpr int NT = (NCW + 1) * 32;
    static constexpr int NC = NCW * 32;
    static constexpr int MAXV = (TXMAX * TY / VS + NC - 1) / NC;
    static constexpr int C_BYTES = (TY + 2 * R) * TXMAX * CS;  // psi rows y0-R .. y0+TY+R-1
    static constexpr int H_PAD = (TY * RP * CS + 127) / 128 * 128;
    static constexpr int P_OFF = C_BYTES + 2 * H_PAD;          // pih tile
    static constexpr int SLOT = (P_OFF + TY * TXMAX * CS + 127) / 128 * 128;
    static constexpr int BAR_OFF = S * SLOT;
    static constexpr int SMEM = BAR_OFF + 256;
    static constexpr bool ZREG = ZR || S < 2 * R + 2;          // z-neighbours in registers (ZR: also with a deeper ring)
    // radius 4: only the planes below the centre in registers, those above read
    // from the ring (where they wait to be centres): 16 registers, not 36
    static constexpr bool ZHALF = ZREG && R >= 4;
    static_assert(S >= (ZREG ? R + 2 : 2 * R + 2), "the ring holds the planes in use and one in flight");
    static_assert(!ZREG || (sizeof(T) == 4 && MAXV == 1), "register z-ring: float fields, one vector per thread");
    static_assert(TY >= R, "halo bands must not wrap inside a box");
};

template <typename T, int TY, int TXMAX, int S, int R, int ZR>
__device__ __forceinline__ void zmarch2r_body(const ZLat *__restrict__ lats, int nlat, int64_t total_items,
                                              int *counters, int parity, int *derr) {
    typedef ZRCfg<T, TY, TXMAX, S, R, ZR> K;
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
                const int nload = zb - za + 2 * R;
                const int bin = Lt.a_index ^ parity;
                const bool xhalo = tx < N;
                const uint32_t psi_bytes = (uint32_t)((TY + 2 * R) * tx * K::CS + (xhalo ? 2 * TY * K::RP * K::CS : 0));
                const uint32_t pih_bytes = (uint32_t)(TY * tx * K::CS);
                const int ym = y0 >= R ? y0 - R : y0 - R + N;
                const int yp = (y0 + TY == N) ? 0 : y0 + TY;
                const int xl = x0 >= K::RP ? x0 - K::RP : x0 - K::RP + N;
                const int xr = (x0 + tx == N) ? 0 : x0 + tx;
                for (int i = 0; i < nload; ++i, ++q) {
                    const int s = (int)(q % S);
                    if (q >= S) {
                        ok = mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)(((q / S) - 1) & 1));
                        if (!ok || *abort_flag) break;
                    }
                    int z = za - R + i;
                    z = z < 0 ? z + N : (z >= N ? z - N : z);
                    unsigned char *slot = smem + s * K::SLOT;
                    const uint32_t bar = smem_u32(&full[s]);
                    const bool with_pih = i >= R && i < nload - R;
                    mbar_expect_tx(bar, psi_bytes + (with_pih ? pih_bytes : 0u) +
                                            (i == 0 ? (uint32_t)Lt.debug_tx_excess : 0u));
                    tma_load_3d(smem_u32(slot), &Lt.tm_row[bin], x0 * K::EU, ym, z, bar);
                    tma_load_3d(smem_u32(slot + R * tx * K::CS), &Lt.tm_main[bin], x0 * K::EU, y0, z, bar);
                    tma_load_3d(smem_u32(slot + (TY + R) * tx * K::CS), &Lt.tm_row[bin], x0 * K::EU, yp, z, bar);
                    if (xhalo) {
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
        const int cid = tid;
        const int setting = R - 1;
        T coef[R + 1];
#pragma unroll
        for (int l = 0; l <= R; ++l) coef[l] = (T)stencil_coef(setting, 3, l);
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
            // ZREG: psi of this thread's vector at planes z-R .. z+R (zr[R] the
            // centre; ZHALF: z-R .. z-1 only); toff is the vector's site offset
            // in a band
            V zr[K::ZREG ? (K::ZHALF ? R : 2 * R + 1) : 1];
            int toff = 0;
            if constexpr (K::ZREG) {
                const int yy = cid < nvec ? cid / nvx : 0, xx = cid < nvec ? (cid % nvx) * K::VS : 0;
                toff = (R + yy) * tx + xx;
                // planes za-R .. za+R-1 (loads 0 .. 2R-1); those below the first
                // centre are released once read
#pragma unroll
                for (int d = 0; d < 2 * R; ++d) {
                    if (!ok) continue;
                    const int wd = warp_wait(smem_u32(&full[(q0 + d) % S]), (uint32_t)(((q0 + d) / S) & 1), abort_flag);
                    if (wd) {
                        if (wd == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                        ok = false;
                        continue;
                    }
                    if (d < (K::ZHALF ? R : 2 * R))
                        zr[d] = *reinterpret_cast<const V *>(reinterpret_cast<const C *>(smem + ((q0 + d) % S) * K::SLOT) + toff);
                    if (d < R) {
                        __syncwarp();
                        if (lane == 0) mbar_arrive(smem_u32(&empty[(q0 + d) % S]));
                    }
                }
            }
            // One vector per thread (MAXV == 1): its row, the byte offsets of its
            // x window's vectors from the centre slot (band, strip or periodic
            // band) and its output offset at plane za are fixed for the item,
            // so the plane loop does no division and no branching for them.
            constexpr int NW = (2 * K::RP + K::VS) / K::VS;   // x window [xx-RP, xx+VS+RP) in 16-byte vectors
            constexpr bool HW = K::MAXV == 1;
            int wo[HW ? NW : 1];
            int yy1 = 0, xx1 = 0;
            int64_t off1 = 0;
            const bool act1 = cid < nvec;
            const int64_t NNl = (int64_t)N * N;
            if constexpr (HW) {
                yy1 = act1 ? cid / nvx : 0;
                xx1 = act1 ? (cid % nvx) * K::VS : 0;
                const int rrow = (R + yy1) * tx;
#pragma unroll
                for (int kw = 0; kw < NW; ++kw) {
                    const int pos = xx1 - K::RP + kw * K::VS;
                    int e;   // element offset from the slot's start
                    if (pos >= 0 && pos < tx) e = rrow + pos;
                    else if (xhalo) e = pos < 0 ? K::C_BYTES / K::CS + yy1 * K::RP + pos + K::RP
                                                : (K::C_BYTES + K::H_PAD) / K::CS + yy1 * K::RP + pos - tx;
                    else e = rrow + (pos < 0 ? pos + tx : pos - tx);
                    wo[kw] = e * K::CS;
                }
                off1 = ((int64_t)za * N + (y0 + yy1)) * N + (x0 + xx1);
            }
            // ring position of load q0 + t (plane z - R) modulo 2S, advanced per
            // plane: the slot of load q0 + t + d is its sum with d modulo S and
            // the load's phase whether that sum modulo 2S reaches S (no 64-bit
            // division per plane). Slot sums stay below 3S (S >= R + 2).
            constexpr bool POW2 = (S & (S - 1)) == 0;
            auto wrap = [](int v) { return POW2 ? v & (S - 1) : (v >= 2 * S ? v - 2 * S : (v >= S ? v - S : v)); };
            int rpos = (int)(q0 % (2 * S));
            for (int t = 0; t < T_steps && ok; ++t) {
                const int s_lo = wrap(rpos);
                int hpos = rpos + 2 * R;   // load q0 + t + 2R
                hpos = POW2 ? hpos & (2 * S - 1) : (hpos >= 2 * S ? hpos - 2 * S : hpos);
                const int s_hi = wrap(hpos);
                const uint32_t ph_hi = hpos >= S ? 1u : 0u;
                int w = 0;
                if (t == 0 && !K::ZREG)
                    for (int d = 0; d < 2 * R && !w; ++d)
                        w = warp_wait(smem_u32(&full[(q0 + d) % S]), (uint32_t)(((q0 + d) / S) & 1), abort_flag);
                if (!w) w = warp_wait(smem_u32(&full[s_hi]), ph_hi, abort_flag);
                if (w) {
                    if (w == 1 && lane == 0) { atomicOr(derr, DEVERR_TIMEOUT); *abort_flag = 1; }
                    ok = false;
                    break;
                }
                const int z = za + t;
                const C *Zp[2 * R + 1];   // planes z-R .. z+R (ZREG: only z and z+R are in the ring)
#pragma unroll
                for (int d = 0; d <= 2 * R; ++d) Zp[d] = reinterpret_cast<const C *>(smem + wrap(s_lo + d) * K::SLOT);
                const C *Cz = Zp[R];
                if constexpr (K::ZREG && !K::ZHALF) zr[2 * R] = *reinterpret_cast<const V *>(Zp[2 * R] + toff);
                const C *Lh = reinterpret_cast<const C *>(reinterpret_cast<const unsigned char *>(Cz) + K::C_BYTES);
                const C *Rh = reinterpret_cast<const C *>(reinterpret_cast<const unsigned char *>(Cz) + K::C_BYTES + K::H_PAD);
                const C *Ph = reinterpret_cast<const C *>(reinterpret_cast<const unsigned char *>(Cz) + K::P_OFF);
#pragma unroll
                for (int jv = 0; jv < K::MAXV; ++jv) {
                    const int v = cid + jv * K::NC;
                    int yy, xx;
                    if constexpr (HW) {
                        if (!act1) continue;
                        yy = yy1;
                        xx = xx1;
                    } else {
                        if (v >= nvec) continue;
                        yy = v / nvx;
                        xx = (v % nvx) * K::VS;
                    }
                    const int rrow = (R + yy) * tx;   // the site's row in the band
                    // The x window [xx-RP, xx+VS+RP) of the site's row as 16-byte
                    // vectors: RP is a multiple of VS, so each vector comes whole
                    // from the band, a strip, or (one x tile) the periodic band.
                    C win[NW * K::VS];
#pragma unroll
                    for (int kw = 0; kw < NW; ++kw) {
                        const C *src;
                        if constexpr (HW) {
                            src = reinterpret_cast<const C *>(reinterpret_cast<const unsigned char *>(Cz) + wo[kw]);
                        } else {
                            const int pos = xx - K::RP + kw * K::VS;
                            if (pos >= 0 && pos < tx) src = &Cz[rrow + pos];
                            else if (xhalo) src = pos < 0 ? &Lh[yy * K::RP + pos + K::RP] : &Rh[yy * K::RP + pos - tx];
                            else src = &Cz[rrow + (pos < 0 ? pos + tx : pos - tx)];
                        }
                        *reinterpret_cast<V *>(&win[kw * K::VS]) = *reinterpret_cast<const V *>(src);
                    }
                    C ctr[K::VS];
#pragma unroll
                    for (int j = 0; j < K::VS; ++j) ctr[j] = win[K::RP + j];
                    T a1[K::VS], a2[K::VS];
#pragma unroll
                    for (int j = 0; j < K::VS; ++j) {
                        a1[j] = coef[0] * ctr[j].x;
                        a2[j] = coef[0] * ctr[j].y;
                    }
#pragma unroll
                    for (int l = 1; l <= R; ++l) {
                        C ym[K::VS], yp[K::VS], zm[K::VS], zp[K::VS];
                        *reinterpret_cast<V *>(ym) = *reinterpret_cast<const V *>(&Cz[rrow - l * tx + xx]);
                        *reinterpret_cast<V *>(yp) = *reinterpret_cast<const V *>(&Cz[rrow + l * tx + xx]);
                        if constexpr (K::ZREG) {
                            *reinterpret_cast<V *>(zm) = zr[R - l];
                            if constexpr (K::ZHALF) *reinterpret_cast<V *>(zp) = *reinterpret_cast<const V *>(&Zp[R + l][rrow + xx]);
                            else *reinterpret_cast<V *>(zp) = zr[R + l];
                        } else {
                            *reinterpret_cast<V *>(zm) = *reinterpret_cast<const V *>(&Zp[R - l][rrow + xx]);
                            *reinterpret_cast<V *>(zp) = *reinterpret_cast<const V *>(&Zp[R + l][rrow + xx]);
                        }
#pragma unroll
                        for (int j = 0; j < K::VS; ++j) {
                            const C xm = win[K::RP + j - l], xp = win[K::RP + j + l];
                            T s1 = (xm.x + xp.x) + (ym[j].x + yp[j].x);
                            T s2 = (xm.y + xp.y) + (ym[j].y + yp[j].y);
                            s1 = s1 + (zm[j].x + zp[j].x);
                            s2 = s2 + (zm[j].y + zp[j].y);
                            a1[j] = fma(coef[l], s1, a1[j]);
                            a2[j] = fma(coef[l], s2, a2[j]);
                        }
                    }
                    T pv[2 * K::VS];
                    *reinterpret_cast<V *>(pv) = *reinterpret_cast<const V *>(&Ph[yy * tx + xx]);
                    C outv[K::VS];
#pragma unroll
                    for (int j = 0; j < K::VS; ++j)
                        site_update<T>(ctr[j].x, ctr[j].y, a1[j], a2[j], pv[2 * j], pv[2 * j + 1], outv[j].x, outv[j].y, cf);
                    const int64_t off = HW ? off1 + (int64_t)t * NNl : ((int64_t)z * N + (y0 + yy)) * N + (x0 + xx);
                    *reinterpret_cast<V *>(&pih[off]) = *reinterpret_cast<V *>(pv);
                    *reinterpret_cast<V *>(&psi_out[off]) = *reinterpret_cast<V *>(outv);
                }
                // this warp is done with plane z-R (load q0+t; ZREG: with the
                // centre z, load q0+t+R); at the last plane also with the
                // item's remaining loads
                V cnew{};   // ZHALF: the centre, next plane's z-1
                if constexpr (K::ZHALF) cnew = *reinterpret_cast<const V *>(Cz + toff);
                __syncwarp();
                const int s_c = wrap(s_lo + R);   // load q0 + t + R (the centre)
                if constexpr (K::ZREG) {
                    if (lane == 0) {
                        mbar_arrive(smem_u32(&empty[s_c]));
                        if (t == T_steps - 1)
                            for (int d = 1; d <= R; ++d) mbar_arrive(smem_u32(&empty[wrap(s_c + d)]));
                    }
                    if constexpr (K::ZHALF) {
#pragma unroll
                        for (int d = 0; d + 1 < R; ++d) zr[d] = zr[d + 1];
                        zr[R - 1] = cnew;
                    } else {
#pragma unroll
                        for (int d = 0; d < 2 * R; ++d) zr[d] = zr[d + 1];
                    }
                } else if (lane == 0) {
                    mbar_arrive(smem_u32(&empty[s_lo]));
                    if (t == T_steps - 1)
                        for (int d = 1; d <= 2 * R; ++d) mbar_arrive(smem_u32(&empty[wrap(s_lo + d)]));
                }
                rpos = rpos + 1 == 2 * S ? 0 : rpos + 1;
            }
            if (!ok) break;
            q0 += T_steps + 2 * R;
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

template <typename T, int TY, int TXMAX, int S, int R, int ZR>
__global__ void __launch_bounds__(ZRCfg<T, TY, TXMAX, S, R, ZR>::NT)
    k_zmarch2r(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity, int *derr) {
    zmarch2r_body<T, TY, TXMAX, S, R, ZR>(lats, nlat, total_items, counters, parity, derr);
}
// Register z-ring: 96 registers, so that two CTAs of nine warps fit the 16K
// registers of each SM sub-partition (at most five warps each).
template <typename T, int TY, int TXMAX, int S, int R, int ZR>
__global__ void __maxnreg__(96)
    k_zmarch2r_zreg(const ZLat *__restrict__ lats, int nlat, int64_t total_items, int *counters, int parity,
                    int *derr) {
    zmarch2r_body<T, TY, TXMAX, S, R, ZR>(lats, nlat, total_items, counters, parity, derr);
}
template <typename T, int TY, int TXMAX, int S, int R, int ZR>
static void (*zr_kernel())(const ZLat *, int, int64_t, int *, int, int *) {
    if constexpr (ZRCfg<T, TY, TXMAX, S, R, ZR>::ZREG) return k_zmarch2r_zreg<T, TY, TXMAX, S, R, ZR>;
    else return k_zmarch2r<T, TY, TXMAX, S, R, ZR>;
}

// ---------------------------------------------------------------- host side

template <typename T, int TY, int TXMAX, int S, int R, int ZR>
static int prepare_r_t() {
    typedef ZRCfg<T, TY, TXMAX, S, R, ZR> K;
    static PerDevice occ;   // the attribute and occupancy belong to the device
    return occ.get([] {
        const auto kern = zr_kernel<T, TY, TXMAX, S, R, ZR>();
        AXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM));
        int o = 0;
        AXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, K::NT, K::SMEM));
        if (o < 1) fail(AXS_ERR_CUDA, "radius-%d z-march kernel does not fit on an SM", R);
        return o;
    });
}

template <typename T, int TY, int TXMAX, int S, int R, int ZR>
static void launch_r_t(const ZLat *d, int nlat, int64_t items, int *counters, int parity, int *derr, cudaStream_t st,
                       int ctas_per_sm) {
    typedef ZRCfg<T, TY, TXMAX, S, R, ZR> K;
    const int occ = prepare_r_t<T, TY, TXMAX, S, R, ZR>();
    const int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    const int64_t grid = std::min<int64_t>((int64_t)per * num_sms(), items);
    zr_kernel<T, TY, TXMAX, S, R, ZR>()<<<(int)grid, K::NT, K::SMEM, st>>>(d, nlat, items, counters, parity, derr);
    AXS_CUDA(cudaGetLastError());
    count_launches(1);
}

// The instantiated shapes (ty, txmax, slots, radius); mirrored by the
// radius-R entries of the variant table in axs_step.cu.
#define AXS_ZR_SHAPES(X) \
    X(8, 128, 6, 2)      \
    X(4, 128, 6, 2)      \
    X(16, 64, 6, 2)      \
    X(8, 64, 8, 3)       \
    X(4, 128, 8, 3)      \
    X(4, 128, 10, 4)     \
    X(8, 64, 10, 4)      \
    X(4, 64, 10, 4)
// register z-ring shapes (S < 2R + 2, or zr = 1 for a deeper ring): float
// fields only; (ty, txmax, slots, radius, zr)
#define AXS_ZR_SHAPES_F(X) \
    X(4, 128, 4, 2, 0)     \
    X(8, 64, 4, 2, 0)      \
    X(4, 128, 5, 3, 0)     \
    X(8, 64, 5, 3, 0)      \
    X(4, 128, 6, 4, 0)     \
    X(8, 64, 6, 4, 0)      \
    X(4, 128, 7, 3, 0)     \
    X(8, 64, 7, 3, 0)      \
    X(8, 64, 8, 4, 0)      \
    X(4, 128, 5, 2, 0)     \
    X(4, 128, 6, 2, 1)     \
    X(4, 128, 7, 2, 1)     \
    X(4, 128, 8, 2, 1)     \
    X(8, 64, 8, 3, 1)      \
    X(8, 64, 9, 3, 1)      \
    X(16, 32, 10, 3, 1)    \
    X(16, 32, 9, 4, 0)     \
    X(16, 32, 10, 4, 1)    \
    X(8, 64, 9, 4, 0)      \
    X(4, 128, 9, 2, 1)

void launch_zmarch_r(int esz, int ty, int txmax, int slots, int r, int zr, const ZLat *d, int nlat, int64_t items,
                     int *counters, int parity, int *derr, cudaStream_t st, int ctas_per_sm) {
#define AXS_ZR_LAUNCH(TY, TX, S, R)                                                                                 \
    if (ty == TY && txmax == TX && slots == S && r == R && !zr) {                                                   \
        if (esz == 4) launch_r_t<float, TY, TX, S, R, 0>(d, nlat, items, counters, parity, derr, st, ctas_per_sm); \
        else launch_r_t<double, TY, TX, S, R, 0>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);         \
        return;                                                                                                     \
    }
    AXS_ZR_SHAPES(AXS_ZR_LAUNCH)
#undef AXS_ZR_LAUNCH
#define AXS_ZR_LAUNCH_F(TY, TX, S, R, ZR)                                                                  \
    if (ty == TY && txmax == TX && slots == S && r == R && zr == ZR) {                                     \
        if (esz != 4) fail(AXS_ERR_ARG, "the register z-ring radius-%d kernel needs float fields", r);       \
        launch_r_t<float, TY, TX, S, R, ZR>(d, nlat, items, counters, parity, derr, st, ctas_per_sm);      \
        return;                                                                                            \
    }
    AXS_ZR_SHAPES_F(AXS_ZR_LAUNCH_F)
#undef AXS_ZR_LAUNCH_F
    fail(AXS_ERR_ARG, "no radius-%d z-march kernel for tile %dx%d, %d slots", r, txmax, ty, slots);
}

void prepare_zmarch_r(int esz, int ty, int txmax, int slots, int r, int zr) {
#define AXS_ZR_PREP(TY, TX, S, R)                                       \
    if (ty == TY && txmax == TX && slots == S && r == R && !zr) {       \
        if (esz == 4) prepare_r_t<float, TY, TX, S, R, 0>();            \
        else prepare_r_t<double, TY, TX, S, R, 0>();                    \
        return;                                                         \
    }
    AXS_ZR_SHAPES(AXS_ZR_PREP)
#undef AXS_ZR_PREP
#define AXS_ZR_PREP_F(TY, TX, S, R, ZR)                                 \
    if (ty == TY && txmax == TX && slots == S && r == R && zr == ZR) {  \
        if (esz == 4) prepare_r_t<float, TY, TX, S, R, ZR>();           \
        return;                                                         \
    }
    AXS_ZR_SHAPES_F(AXS_ZR_PREP_F)
#undef AXS_ZR_PREP_F
    fail(AXS_ERR_ARG, "no radius-%d z-march kernel for tile %dx%d, %d slots", r, txmax, ty, slots);
}

}  // namespace axs
