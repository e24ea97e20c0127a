// Internal declarations shared by the CUDA translation units of libaxs.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <atomic>
#include <map>
#include <string>
#include <vector>

#include "../../include/axs.h"

namespace axs {

// ---------------------------------------------------------------- errors
struct Error {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const char *fmt, ...);
void set_last_error(int code, const std::string &msg);
void clear_last_error();

#define AXS_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) ::axs::fail(AXS_ERR_CUDA, "%s failed: %s (%s:%d)", #call,       \
                                           cudaGetErrorString(e_), __FILE__, __LINE__);         \
    } while (0)
#define AXS_CUFFT(call)                                                                         \
    do {                                                                                        \
        cufftResult r_ = (call);                                                                \
        if (r_ != CUFFT_SUCCESS) ::axs::fail(AXS_ERR_CUDA, "%s failed: cufft status %d", #call, \
                                             (int)r_);                                          \
    } while (0)

// Count of kernels launched by the library (host-side claim for benches).
void count_launches(int64_t n);

// Device error-flag bits (Lattice::derr).
enum : int { DEVERR_TIMEOUT = 1 };

// ---------------------------------------------------------------- lattice
struct StepConfig {
    int kind = 0;        // 0 = generic per-site kernel, 1 = TMA z-march kernel
    int variant = 0;     // z-march template variant index
    int zchunk = 64;     // planes per work item
    int tx = 0;          // x tile (sites)
    int ctas_per_sm = 0; // persistent grid occupancy
    std::string describe() const;
};

struct Lattice;

// One lattice's slot in a z-march launch (device-resident table entry).
struct ZLat {
    CUtensorMap tm_row[2];   // box {tx, 1, 1} over psi[b]
    CUtensorMap tm_main[2];  // box {tx, TY, 1}
    CUtensorMap tm_xh[2];    // box {16-byte halo, TY, 1}
    CUtensorMap tm_pih[2];   // box {tx, TY, 1} over pih[b]
    // two-step (halo depth 2) kernel only
    CUtensorMap t2_row2[2];  // box {tx, 2, 1} over psi[b]
    CUtensorMap t2_str2[2];  // box {16-byte halo, 2, 1} over psi[b]
    CUtensorMap t2_prow[2];  // box {tx, 1, 1} over pih[b]
    CUtensorMap t2_pstr[2];  // box {16-byte halo, TY, 1} over pih[b]
    // three-step (halo depth 3) kernel only
    CUtensorMap t3_row3[2];  // box {tx, 3, 1} over psi[b]
    CUtensorMap t3_strm[2];  // box {4 sites, TY, 1} over psi[b]
    CUtensorMap t3_str2[2];  // box {4 sites, 2, 1} over psi[b]
    CUtensorMap t3_prow2[2]; // box {tx, 2, 1} over pih[b]
    CUtensorMap t3_pst1[2];  // box {16-byte halo, 1, 1} over pih[b]
    void *psi[2];
    // pih[b]: the half-step momentum that goes with psi[b] as current field.
    // A launch reads pih[bin] and writes pih[bin ^ 1]; both are the same
    // buffer when the momentum is updated in place.
    void *pih[2];
    double *clock;           // [2] tau at the parity of psi
    int N, tx, ntx, nty, nzc;
    int a_index;             // which of psi[0]/psi[1] is "current" at launch parity 0
    int64_t item_base;
    double dt, inv_dx2, lambda, T0sq3;
    int prs, form;
    int debug_tx_excess;     // test-only: bytes the first load of each item expects but never gets
};

// The table entry that owns work item `item`: the last entry whose item_base
// is <= item (item bases ascend from 0). Binary search: an ensemble table has
// up to hundreds of entries, ~1 KB apart (tensor maps), read per item.
__device__ __forceinline__ int find_lat(const ZLat *__restrict__ lats, int nlat, int64_t item) {
    int lo = 0, hi = nlat - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (lats[mid].item_base <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// A captured interval is keyed by its length and the state it starts from
// (current psi buffer, and where the momentum lives); it ends in a fixed state.
struct GraphKey {
    int nsteps, parity;
    uint64_t state;   // hash of the members' (cur, pih) pairs
    bool operator<(const GraphKey &o) const {
        if (nsteps != o.nsteps) return nsteps < o.nsteps;
        if (parity != o.parity) return parity < o.parity;
        return state < o.state;
    }
};
struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;             // kernels in the graph
    std::vector<int> cur_after;       // per member
    std::vector<uint8_t> swapped;     // per member: pih and scratch exchanged an odd number of times
};

struct Lattice {
    axs_params p{};
    int64_t length = 0;   // N^NDIMS
    int esz = 8;          // bytes per real component (4 or 8)
    void *psi[2] = {nullptr, nullptr};
    void *pih = nullptr;  // half-step momentum (or pi_0 when fresh)
    // complex, length sites: synchronised pi for the analysis, and the
    // destination of the momentum in two-step mode (the two pointers are then
    // exchanged after every launch; the contents of scratch never outlive a call)
    void *scratch = nullptr;
    double *dclock = nullptr; // [2]
    int *derr = nullptr;      // device error flags
    int *dcounter = nullptr;  // [2] work counters of the persistent step kernel
    int cur = 0;              // psi[cur] holds the current field; dclock[cur] its tau
    int fresh = 1;            // next step is the pure drift of a freshly set state (2: an upload
                              // formed it already into psi[cur ^ 1] and the next clock)
    double tau = 1.0;
    int64_t steps = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    bool in_ensemble = false;
    StepConfig cfg;
    bool tuned = false;
    // z-march launch table for this lattice alone
    ZLat *dzlat = nullptr;
    int zlat_variant = -1, zlat_tx = -1, zlat_zchunk = -1;
    void *zlat_pih[2] = {nullptr, nullptr};   // host copy of the table's pih[]
    int debug_tx_excess = 0;  // set by axs_inject_wait_timeout for one step
    int64_t zitems = 0;
    // analysis buffers (lazily allocated)
    uint8_t *dmask = nullptr;
    int64_t *dcount = nullptr;       // [4] scratch counters
    int32_t *dlist = nullptr;        // ascending flagged offsets (compacted)
    int64_t list_cap = 0;
    int64_t last_nplaq = -1;
    bool list_valid = false;
    double *dtheta = nullptr;        // caller theta upload
    void *fft_in = nullptr;          // real, length
    void *fft_out = nullptr;         // complex, R2C half spectrum
    cufftHandle plan_r2c = 0;
    bool have_plan = false;
    double *dpartials = nullptr;     // reduction partials
    size_t partials_cap = 0;
    void *dstage = nullptr;          // transfer staging (length reals)
    // small per-call work buffers of the analysis, kept between calls (grow only):
    // 0 = string-finder chunk counts, 1 = spectrum block partials, 2 = bin thresholds
    void *tmp[3] = {nullptr, nullptr, nullptr};
    size_t tmp_cap[3] = {0, 0, 0};
    // per-bin |n| sums and mode counts of the spectrum binnings used so far:
    // they depend on N and the bin edges alone, so later spectra with the same
    // edges bin the power only (kind 0 = linear bins of output_powerspec,
    // 1 = log bins of the axion spectrum; edges identify the binning)
    struct BinGeom {
        int kind;
        std::vector<int> edges;
        std::vector<double> nsum;
        std::vector<unsigned long long> cnt;
    };
    std::vector<BinGeom> bin_geom;
    // spectral Laplacian (axs_params.laplacian = 1): complex transform plan and
    // the per-axis k^2 table (N doubles, then N floats)
    cufftHandle plan_c2c = 0;
    bool have_c2c = false;
    void *dksq = nullptr;
    std::map<GraphKey, GraphEntry> graphs;
};

struct Ensemble {
    std::vector<Lattice *> members;
    cudaStream_t stream = nullptr;
    StepConfig cfg;
    bool tuned = false;
    ZLat *dzlat = nullptr;
    int64_t zitems = 0;
    int *dcounter = nullptr;
    int *derr = nullptr;
    // per member (in members order): its cur when the table was built, and the
    // table's pih[] for it
    std::vector<int> tab_cur;
    std::vector<void *> tab_pih;   // 2 per member
    std::map<GraphKey, GraphEntry> graphs;
    // page-locked host buffer of the batched analysis calls (grow only): the
    // members' results land here asynchronously, one synchronisation per call
    void *hpin = nullptr;
    size_t hpin_cap = 0;
    // streams of the batched analysis: members' kernels run concurrently
    // (small members fill few SMs each), joined back by events
    std::vector<cudaStream_t> pool;
    std::vector<cudaEvent_t> pool_ev;
    cudaEvent_t ev_fork = nullptr;
};

// ---- step module (axs_step.cu)
void step_setup(Lattice *L);
void step_release(Lattice *L);
bool zmarch_supported(const axs_params &p);
int lattice_advance(Lattice *L, int max_steps);       // one launch (eager or inside capture); steps taken
void clear_graphs(std::map<GraphKey, GraphEntry> &g);
void lattice_evolve(Lattice *L, int nsteps);          // graph-cached
void lattice_autotune(Lattice *L);
void ensemble_setup(Ensemble *E);
void ensemble_evolve(Ensemble *E, int nsteps);
void ensemble_autotune(Ensemble *E);
// radius-R z-march kernels (axs_step_r.cu), by tile shape; zr = 1 keeps the
// z-neighbours in registers with a ring of 2R + 2 or more slots
void launch_zmarch_r(int esz, int ty, int txmax, int slots, int r, int zr, const ZLat *d, int nlat, int64_t items,
                     int *counters, int parity, int *derr, cudaStream_t st, int ctas_per_sm);
void prepare_zmarch_r(int esz, int ty, int txmax, int slots, int r, int zr);
std::string ensemble_describe(const Ensemble *E);
// ---- batched analysis over the members (axs_analysis.cu)
void ensemble_find_strings(Ensemble *E, int64_t *nplaq, int64_t *ncores);
void ensemble_axion_spectrum(Ensemble *E, int nbins, double *kmean, double *pk, int64_t *count);
void ensemble_release_pool(Ensemble *E);
void launch_sync_pi(Lattice *L);                      // scratch <- pi_n
void launch_laplacian(Lattice *L, int comp, double *dout);
void launch_unpack(Lattice *L, const void *src, int which, int comp, void *dst_real, int dst_is_double);
void launch_pack(Lattice *L, const void *src_real, int src_is_double, int which, int comp);
void launch_pack2(Lattice *L, const void *a, const void *b, int src_is_double, void *dst_cplx, int64_t n,
                  cudaStream_t st);
// the momentum pair into pih[off, off + n) with the first (pure drift) step of
// a fresh state into psi[cur ^ 1] and the next clock
void launch_pack2_drift(Lattice *L, const void *a, const void *b, int src_is_double, int64_t off, int64_t n,
                        cudaStream_t st);
void launch_unpack2(Lattice *L, const void *src_cplx, void *a, void *b, int dst_is_double, int64_t n, cudaStream_t st);
void check_device_errors(Lattice *L);
void check_device_error_flag(int *derr, cudaStream_t s);

// ---- init module (axs_init.cu)
void init_gaussian(Lattice *L, uint64_t seed, int thermal, double kcut);

// ---- analysis module (axs_analysis.cu)
void find_strings(Lattice *L, const double *theta_host, uint8_t *mask_host, int64_t *nplaq, int64_t *ncores);
void string_positions(Lattice *L, int32_t *pos, int64_t cap, int64_t *n);
void powerspec(Lattice *L, int field, double *pk, double *ks, int *count);
void axion_spectrum(Lattice *L, int nbins, double *kmean, double *pk, int64_t *count);
void background(Lattice *L, double out[6]);
void energies(Lattice *L, double out[3]);
int check_finite(Lattice *L);
void field_distance(Lattice *A, Lattice *B, double out[8]);
void analysis_release(Lattice *L);

// helpers
inline int64_t lattice_length(const axs_params &p) {
    int64_t N = p.N;
    return p.NDIMS == 3 ? N * N * N : N * N;
}
int num_sms();                  // of the current device
int current_device();
// A value set up once per device (its SM count or shared-memory limit, a
// kernel's attribute and occupancy there): one process may drive several
// GPUs (axs_set_device), and their values may differ. make() runs with the
// device current; concurrent first calls may both run it (same result).
constexpr int kMaxDevices = 128;
struct PerDevice {
    std::atomic<int> v[kMaxDevices];
    PerDevice() {
        for (auto &x : v) x = -1;
    }
    template <class F>
    int get(F make) {
        const int d = current_device();
        if (d < 0 || d >= kMaxDevices) return make();
        int r = v[d].load();
        if (r < 0) {
            r = make();
            v[d] = r;
        }
        return r;
    }
};
int reduce_grid(int64_t len);   // fixed grid size of the deterministic reductions
// Sum per-block partials (nblocks x K, device) in block order on the host.
void sum_partials(const double *dpart, int nblocks, int K, double *out, cudaStream_t s);
void *dalloc(size_t bytes);
void dfree(void *p);

}  // namespace axs

// ------------------------------------------------------------------ device side
#ifdef __CUDACC__
namespace axs {

// Stencil coefficients of build_coefficient_matrix (src/standard/s_integrate.cpp:9-14):
// float expressions, as the reference stores them.
__host__ __device__ inline float stencil_coef(int setting, int ndims, int l) {
    switch (setting) {
    case 0: { const float c[2] = {-2.0f * ndims, 1.0f}; return c[l]; }
    case 1: { const float c[3] = {-5.0f / 2.0f * ndims, 4.0f / 3.0f, -1.0f / 12.0f}; return c[l]; }
    case 2: { const float c[4] = {-49.0f / 18.0f * ndims, 3.0f / 2.0f, -3.0f / 20.0f, 1.0f / 90.0f}; return c[l]; }
    default: { const float c[5] = {-205.0f / 72.0f * ndims, 8.0f / 5.0f, -1.0f / 5.0f, 8.0f / 315.0f, -1.0f / 560.0f}; return c[l]; }
    }
}

template <typename T> struct Cplx;
template <> struct Cplx<float> { typedef float2 type; };
template <> struct Cplx<double> { typedef double2 type; };

// Per-step scalars, derived from tau (double) once per CTA.
template <typename T> struct StepCoefs {
    T dt;        // drift
    T kdt_idx2;  // kick * 1/dx^2
    T kdt_coef;  // kick * (-lambda / tau^(2 prs))
    T c0;        // T0^2/3 - tau^2
};

// form 0, field-rescaled (s_integrate.cpp:305-348): K = L/dx^2 - lambda/tau^(2 prs)
//   psi (|psi|^2 - tau^2 + T0^2/3), drift dt.
// form 1, Hamiltonian-like (s_integrate.cpp:358-395): K = tau^2 L/dx^2 - lambda tau^2
//   phi (|phi|^2 - 1 + T0^2/(3 tau^2)), drift dt / tau_{n+1}^2 (tau is advanced
//   before the drift there).
template <typename T>
__device__ __forceinline__ StepCoefs<T> make_coefs(double tau, double dt, double kick, double inv_dx2,
                                                    double lambda, double T0sq3, int prs, int form) {
    StepCoefs<T> c;
    if (form == 1) {
        const double t1 = tau + dt, tsq = tau * tau;
        c.dt = (T)(dt / (t1 * t1));
        c.kdt_idx2 = (T)(kick * tsq * inv_dx2);
        c.kdt_coef = (T)(kick * (-lambda * tsq));
        c.c0 = (T)(T0sq3 / tsq - 1.0);
        return c;
    }
    double coef = prs ? -lambda / (tau * tau) : -lambda;
    c.dt = (T)dt;
    c.kdt_idx2 = (T)(kick * inv_dx2);
    c.kdt_coef = (T)(kick * coef);
    c.c0 = (T)(T0sq3 - tau * tau);
    return c;
}

// Radius-1 stencil sum, fixed association order shared by every kernel:
// ((x- + x+) + (y- + y+)) + (z- + z+), then centre * (-2 d) fused.
template <typename T>
__device__ __forceinline__ T lap7(T c, T xm, T xp, T ym, T yp, T zm, T zp) {
    T s = ((xm + xp) + (ym + yp)) + (zm + zp);
    return fma((T)-6, c, s);
}
template <typename T>
__device__ __forceinline__ T lap5(T c, T xm, T xp, T ym, T yp) {
    T s = (xm + xp) + (ym + yp);
    return fma((T)-4, c, s);
}

// The fused kick + drift of one site. (a, b) = psi, L = stencil sums (not
// divided by dx^2), (p1, p2) = half-step momentum in/out, (an, bn) = new psi.
template <typename T>
__device__ __forceinline__ void site_update(T a, T b, T L1, T L2, T &p1, T &p2, T &an, T &bn,
                                            const StepCoefs<T> &c) {
    T r = fma(a, a, fma(b, b, c.c0));
    T g = c.kdt_coef * r;
    p1 = fma(c.kdt_idx2, L1, fma(g, a, p1));
    p2 = fma(c.kdt_idx2, L2, fma(g, b, p2));
    an = fma(c.dt, p1, a);
    bn = fma(c.dt, p2, b);
}

// Plain FP64 steps of radius 1 fold the stencil's centre weight w0 = -2 NDIMS
// into the local coefficient: the kick is kdt_idx2 S + (kdt_coef r +
// kdt_idx2 w0) psi with S the neighbour sum, two FP64 operations per site
// fewer than forming the Laplacian first (GB300's FP64 pipe bounds the plain
// FP64 step); kctr = kdt_idx2 w0. Float steps keep the Laplacian form.
template <typename T>
__device__ __forceinline__ void site_update_fold(T a, T b, T S1, T S2, T &p1, T &p2, T &an, T &bn,
                                                 const StepCoefs<T> &c, T kctr) {
    T r = fma(a, a, fma(b, b, c.c0));
    T g = fma(c.kdt_coef, r, kctr);
    p1 = fma(c.kdt_idx2, S1, fma(g, a, p1));
    p2 = fma(c.kdt_idx2, S2, fma(g, b, p2));
    an = fma(c.dt, p1, a);
    bn = fma(c.dt, p2, b);
}
template <typename T>
__device__ __forceinline__ T nsum7(T xm, T xp, T ym, T yp, T zm, T zp) { return ((xm + xp) + (ym + yp)) + (zm + zp); }
template <typename T>
__device__ __forceinline__ T nsum5(T xm, T xp, T ym, T yp) { return (xm + xp) + (ym + yp); }

// Synchronised momentum of one site: pi_n = pih_{n-1} + dt/2 K(psi_n) with
// c = make_coefs(tau_n, dt, dt/2, ...); (L1, L2) the stencil sums.
template <typename T>
__device__ __forceinline__ void sync_pi_site(T a, T b, T L1, T L2, T &p1, T &p2, const StepCoefs<T> &c) {
    T r = fma(a, a, fma(b, b, c.c0));
    T g = c.kdt_coef * r;
    p1 = fma(c.kdt_idx2, L1, fma(g, a, p1));
    p2 = fma(c.kdt_idx2, L2, fma(g, b, p2));
}

// The axion field of the kinetic spectrum, f = |phi| dtheta/dtau =
// (psi2 pi1 - psi1 pi2) / (tau |psi|), with itau = 1/tau.
template <typename T>
__device__ __forceinline__ T axion_f(T a, T b, T p1, T p2, T itau) {
    T r = sqrt(a * a + b * b);
    return r > (T)0 ? (b * p1 - a * p2) * itau / r : (T)0;
}
// Float fields: one rsqrtf (2 ulp) in place of a correctly rounded square
// root and division; float spectra are compared to the double ones within
// 1e-4, far above this.
template <>
__device__ __forceinline__ float axion_f<float>(float a, float b, float p1, float p2, float itau) {
    const float r2 = a * a + b * b;
    return r2 > 0.f ? (b * p1 - a * p2) * itau * rsqrtf(r2) : 0.f;
}
// FP64 fields: 1/|psi| by two Newton-Raphson steps for the reciprocal square
// root, y <- y (3/2 - s y^2 / 2), from the float rsqrtf (within 1-2 ulp of the
// correctly rounded square root and division, at a third of their cost on
// GB300's FP64 pipe); |psi|^2 outside float range takes those.
template <>
__device__ __forceinline__ double axion_f<double>(double a, double b, double p1, double p2, double itau) {
    const double s = a * a + b * b;
    if (s > 1e-36 && s < 1e36) {
        const double hs = 0.5 * s;
        double y = (double)rsqrtf((float)s);
        y = y * fma(-hs * y, y, 1.5);
        y = y * fma(-hs * y, y, 1.5);
        return (b * p1 - a * p2) * itau * y;
    }
    const double r = sqrt(s);
    return r > 0.0 ? (b * p1 - a * p2) * itau / r : 0.0;
}

// Philox-4x32-10 (Salmon et al., SC'11) and Box-Muller; the deviate for
// array a at offset m. Must agree with the oracle's definition.
// Both deviates of arrays 2*pair and 2*pair+1 at offset m from one Philox block
// and one logarithm (the same values as two normal_draw calls).
__device__ __forceinline__ void normal_pair(uint64_t seed, int pair, int64_t m, double &g0, double &g1) {
    uint32_t c0 = (uint32_t)((uint64_t)m & 0xffffffffu), c1 = (uint32_t)((uint64_t)m >> 32);
    uint32_t c2 = (uint32_t)pair, c3 = 0x41585331u;
    uint32_t k0 = (uint32_t)(seed & 0xffffffffu), k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    uint64_t b1 = (((uint64_t)c0 << 21) ^ (uint64_t)(c1 >> 11)) & ((1ull << 53) - 1);
    uint64_t b2 = (((uint64_t)c2 << 21) ^ (uint64_t)(c3 >> 11)) & ((1ull << 53) - 1);
    const double two_m53 = 1.1102230246251565404e-16;
    double u1 = (double)(b1 + 1) * two_m53;
    double u2 = (double)b2 * two_m53;
    double rr = sqrt(-2.0 * log(u1));
    double ang = 6.283185307179586232 * u2;
    g0 = rr * cos(ang);
    g1 = rr * sin(ang);
}

__device__ __forceinline__ double normal_draw(uint64_t seed, int a, int64_t m) {
    uint32_t c0 = (uint32_t)((uint64_t)m & 0xffffffffu), c1 = (uint32_t)((uint64_t)m >> 32);
    uint32_t c2 = (uint32_t)(a >> 1), c3 = 0x41585331u;
    uint32_t k0 = (uint32_t)(seed & 0xffffffffu), k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    uint64_t b1 = (((uint64_t)c0 << 21) ^ (uint64_t)(c1 >> 11)) & ((1ull << 53) - 1);
    uint64_t b2 = (((uint64_t)c2 << 21) ^ (uint64_t)(c3 >> 11)) & ((1ull << 53) - 1);
    const double two_m53 = 1.1102230246251565404e-16;
    double u1 = (double)(b1 + 1) * two_m53;
    double u2 = (double)b2 * two_m53;
    double rr = sqrt(-2.0 * log(u1));
    double ang = 6.283185307179586232 * u2;
    return (a & 1) ? rr * sin(ang) : rr * cos(ang);
}

__device__ __forceinline__ int64_t wrapi(int64_t i, int64_t N) { return i < 0 ? i + N : (i >= N ? i - N : i); }

// Deterministic block reduction of K doubles (fixed shuffle tree, warps summed
// in order); thread 0 writes the block's K partial sums to out[blockIdx.x*K+k].
// blockDim.x must be 256.
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&v)[K], double *out) {
    __shared__ double red[8][K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        v[k] = x;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[w][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0.0;
            for (int i = 0; i < 8; ++i) s += red[i][k];
            out[(int64_t)blockIdx.x * K + k] = s;
        }
    }
    __syncthreads();
}

}  // namespace axs
#endif
