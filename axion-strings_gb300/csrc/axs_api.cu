// C ABI of libaxs (declared in include/axs.h). Every entry point catches the
// library's internal errors and returns a status code; the message is kept
// per thread for axs_last_error().
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <map>
#include <new>
#include <vector>
#include <algorithm>

#include <mutex>

#include "axs_internal.h"

struct axs_lattice {
    axs::Lattice L;
};
struct axs_ensemble {
    axs::Ensemble E;
    std::vector<axs_lattice *> members;
};

namespace axs {

static thread_local int t_err_code = AXS_OK;
static thread_local std::string t_err_msg;

void fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error{code, buf};
}
void set_last_error(int code, const std::string &msg) {
    t_err_code = code;
    t_err_msg = msg;
}
void clear_last_error() {
    t_err_code = AXS_OK;
    t_err_msg.clear();
}

void *dalloc(size_t bytes) {
    void *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        fail(AXS_ERR_NOMEM, "cudaMalloc of %zu bytes failed: out of device memory", bytes);
    }
    if (e != cudaSuccess) fail(AXS_ERR_CUDA, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return p;
}
void dfree(void *p) {
    if (p) cudaFree(p);
}

int reduce_grid(int64_t len) {
    int64_t want = (len + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)num_sms() * 8));
}

void sum_partials(const double *dpart, int nblocks, int K, double *out, cudaStream_t s) {
    std::vector<double> h((size_t)nblocks * K);
    AXS_CUDA(cudaMemcpyAsync(h.data(), dpart, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    AXS_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < K; ++k) {
        double acc = 0.0;
        for (int b = 0; b < nblocks; ++b) acc += h[(size_t)b * K + k];
        out[k] = acc;
    }
}

int64_t total_launches();

static void validate(const axs_params &p) {
    if (p.NDIMS != 2 && p.NDIMS != 3) fail(AXS_ERR_ARG, "NDIMS must be 2 or 3 (got %d)", p.NDIMS);
    if (p.N < 4 || (p.N % 2) != 0) fail(AXS_ERR_ARG, "N must be even and >= 4 (got %d)", p.N);   // s_run.cpp:32
    if (p.stencil_setting < 0 || p.stencil_setting > 3) fail(AXS_ERR_ARG, "stencil_setting must be 0..3");
    if (p.N <= 2 * (p.stencil_setting + 1)) fail(AXS_ERR_ARG, "N too small for the stencil radius");
    if (p.precision != AXS_F32 && p.precision != AXS_F64) fail(AXS_ERR_ARG, "precision must be 32 or 64");
    if (!(p.space_step > 0.0f)) fail(AXS_ERR_ARG, "space_step must be positive");
    if (!std::isfinite(p.time_step)) fail(AXS_ERR_ARG, "time_step must be finite");
    // 3D: |n|^2 of the spectrum binner stays below 2^24 (4096^3 would not fit
    // the device anyway); 2D: in-plane offsets and |n|^2 stay below 2^31
    const int nmax = p.NDIMS == 2 ? 32768 : 4096;
    if (p.N > nmax) fail(AXS_ERR_ARG, "N=%d exceeds the supported maximum %d for %dD", p.N, nmax, p.NDIMS);
    if (p.form != 0 && p.form != 1) fail(AXS_ERR_ARG, "form must be 0 (field-rescaled) or 1 (Hamiltonian)");
    if (p.laplacian != 0 && p.laplacian != 1) fail(AXS_ERR_ARG, "laplacian must be 0 (stencil) or 1 (spectral)");
}

static void set_device_clock(Lattice *L) {
    AXS_CUDA(cudaMemcpyAsync(L->dclock + L->cur, &L->tau, sizeof(double), cudaMemcpyHostToDevice, L->stream));
}

static void lattice_init(Lattice *L, const axs_params &p, cudaStream_t shared) {
    validate(p);
    L->p = p;
    L->length = lattice_length(p);
    L->esz = p.precision == AXS_F32 ? 4 : 8;
    if (shared) {
        L->stream = shared;
        L->own_stream = false;
    } else {
        AXS_CUDA(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
        L->own_stream = true;
    }
    size_t cbytes = (size_t)L->length * 2 * L->esz;
    L->psi[0] = dalloc(cbytes);
    L->psi[1] = dalloc(cbytes);
    L->pih = dalloc(cbytes);
    L->scratch = dalloc(cbytes);
    L->dclock = (double *)dalloc(2 * sizeof(double));
    L->derr = (int *)dalloc(sizeof(int));
    AXS_CUDA(cudaMemsetAsync(L->psi[0], 0, cbytes, L->stream));
    AXS_CUDA(cudaMemsetAsync(L->psi[1], 0, cbytes, L->stream));
    AXS_CUDA(cudaMemsetAsync(L->pih, 0, cbytes, L->stream));
    AXS_CUDA(cudaMemsetAsync(L->derr, 0, sizeof(int), L->stream));
    L->cur = 0;
    L->fresh = 1;
    L->tau = p.tau_initial;
    L->steps = 0;
    set_device_clock(L);
    step_setup(L);
    AXS_CUDA(cudaStreamSynchronize(L->stream));
}

static void xfer_release(Lattice *L);

static void lattice_free(Lattice *L) {
    if (L->stream) cudaStreamSynchronize(L->stream);
    xfer_release(L);
    step_release(L);
    analysis_release(L);
    dfree(L->psi[0]);
    dfree(L->psi[1]);
    dfree(L->pih);
    dfree(L->scratch);
    dfree(L->dclock);
    dfree(L->derr);
    dfree(L->dstage);
    if (L->own_stream && L->stream) cudaStreamDestroy(L->stream);
    L->stream = nullptr;
}

static void *stage(Lattice *L) {
    if (!L->dstage) L->dstage = dalloc((size_t)L->length * sizeof(double));
    return L->dstage;
}

// Device-addressable alias of a caller buffer (device or managed memory, or
// page-locked host memory, which the GPU reads and writes over NVLink-C2C /
// PCIe), or nullptr for pageable host memory.
static void *device_alias(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void *>(p);
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    return nullptr;
}

// Chunked, double-buffered staging of pageable host arrays: copies run on a
// second stream and overlap the (un)packing kernels on the lattice stream.
static const int64_t kXferChunk = (int64_t)1 << 25;   // elements per chunk

struct Xfer {
    cudaStream_t copy = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, done[2] = {nullptr, nullptr}, entry = nullptr;
    char *buf = nullptr;   // [2 slots][2 arrays][chunk] of 8-byte elements
    int64_t chunk = 0;     // elements per chunk (<= kXferChunk, <= the lattice length)
};
static std::map<Lattice *, Xfer> g_xfer;
static std::mutex g_xfer_mu;   // handles may be driven from different threads

static Xfer &xfer(Lattice *L) {
    std::lock_guard<std::mutex> lk(g_xfer_mu);
    Xfer &x = g_xfer[L];   // map nodes stay put: the reference outlives the lock
    if (!x.buf) {
        AXS_CUDA(cudaStreamCreateWithFlags(&x.copy, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            AXS_CUDA(cudaEventCreateWithFlags(&x.copied[i], cudaEventDisableTiming));
            AXS_CUDA(cudaEventCreateWithFlags(&x.done[i], cudaEventDisableTiming));
        }
        AXS_CUDA(cudaEventCreateWithFlags(&x.entry, cudaEventDisableTiming));
        x.chunk = std::min(kXferChunk, L->length);
        x.buf = (char *)dalloc((size_t)4 * x.chunk * sizeof(double));
    }
    return x;
}
static void xfer_release(Lattice *L) {
    std::lock_guard<std::mutex> lk(g_xfer_mu);
    auto it = g_xfer.find(L);
    if (it == g_xfer.end()) return;
    Xfer &x = it->second;
    if (x.copy) { cudaStreamSynchronize(x.copy); cudaStreamDestroy(x.copy); }
    for (int i = 0; i < 2; ++i) {
        if (x.copied[i]) cudaEventDestroy(x.copied[i]);
        if (x.done[i]) cudaEventDestroy(x.done[i]);
    }
    if (x.entry) cudaEventDestroy(x.entry);
    dfree(x.buf);
    g_xfer.erase(it);
}

// drift: dst is pih and psi[cur] holds the new psi; the first (pure drift)
// step of the fresh state goes along with the packing (launch_pack2_drift)
template <typename S>
static void upload_pair(Lattice *L, const S *a, const S *b, void *dst, bool drift = false) {
    const int is_d = sizeof(S) == 8;
    void *da = device_alias(a), *db = device_alias(b);
    if (da && db) {
        if (drift) launch_pack2_drift(L, da, db, is_d, 0, L->length, L->stream);
        else launch_pack2(L, da, db, is_d, dst, L->length, L->stream);
        return;
    }
    Xfer &x = xfer(L);
    // the staging slots may still be read by packing kernels of an earlier
    // transfer on the lattice stream: copies start after them
    AXS_CUDA(cudaEventRecord(x.entry, L->stream));
    AXS_CUDA(cudaStreamWaitEvent(x.copy, x.entry, 0));
    const size_t cs = (size_t)2 * L->esz;
    int64_t nch = (L->length + x.chunk - 1) / x.chunk;
    for (int64_t c = 0; c < nch; ++c) {
        int s = (int)(c & 1);
        int64_t off = c * x.chunk, n = std::min(x.chunk, L->length - off);
        char *sa = x.buf + (size_t)(2 * s) * x.chunk * sizeof(double);
        char *sb = sa + (size_t)x.chunk * sizeof(double);
        if (c >= 2) AXS_CUDA(cudaStreamWaitEvent(x.copy, x.done[s], 0));
        AXS_CUDA(cudaMemcpyAsync(sa, a + off, (size_t)n * sizeof(S), cudaMemcpyHostToDevice, x.copy));
        AXS_CUDA(cudaMemcpyAsync(sb, b + off, (size_t)n * sizeof(S), cudaMemcpyHostToDevice, x.copy));
        AXS_CUDA(cudaEventRecord(x.copied[s], x.copy));
        AXS_CUDA(cudaStreamWaitEvent(L->stream, x.copied[s], 0));
        if (drift) launch_pack2_drift(L, sa, sb, is_d, off, n, L->stream);
        else launch_pack2(L, sa, sb, is_d, (char *)dst + (size_t)off * cs, n, L->stream);
        AXS_CUDA(cudaEventRecord(x.done[s], L->stream));
    }
}

template <typename S>
static void download_pair(Lattice *L, const void *src, S *a, S *b) {
    const int is_d = sizeof(S) == 8;
    void *da = device_alias(a), *db = device_alias(b);
    if (da && db) {
        launch_unpack2(L, src, da, db, is_d, L->length, L->stream);
        return;
    }
    Xfer &x = xfer(L);
    // unpacking into the staging slots starts after earlier copies out of them
    AXS_CUDA(cudaEventRecord(x.entry, x.copy));
    AXS_CUDA(cudaStreamWaitEvent(L->stream, x.entry, 0));
    const size_t cs = (size_t)2 * L->esz;
    int64_t nch = (L->length + x.chunk - 1) / x.chunk;
    for (int64_t c = 0; c < nch; ++c) {
        int s = (int)(c & 1);
        int64_t off = c * x.chunk, n = std::min(x.chunk, L->length - off);
        char *sa = x.buf + (size_t)(2 * s) * x.chunk * sizeof(double);
        char *sb = sa + (size_t)x.chunk * sizeof(double);
        if (c >= 2) AXS_CUDA(cudaStreamWaitEvent(L->stream, x.done[s], 0));
        launch_unpack2(L, (const char *)src + (size_t)off * cs, sa, sb, is_d, n, L->stream);
        AXS_CUDA(cudaEventRecord(x.copied[s], L->stream));
        AXS_CUDA(cudaStreamWaitEvent(x.copy, x.copied[s], 0));
        AXS_CUDA(cudaMemcpyAsync(a + off, sa, (size_t)n * sizeof(S), cudaMemcpyDeviceToHost, x.copy));
        AXS_CUDA(cudaMemcpyAsync(b + off, sb, (size_t)n * sizeof(S), cudaMemcpyDeviceToHost, x.copy));
        AXS_CUDA(cudaEventRecord(x.done[s], x.copy));
    }
    AXS_CUDA(cudaStreamSynchronize(x.copy));
}

template <typename S>
static void upload_fields(Lattice *L, const S *f0, const S *f1, const S *f2, const S *f3) {
    const S *src[4] = {f0, f1, f2, f3};
    const int is_d = sizeof(S) == 8;
    set_device_clock(L);   // before the drift that reads it
    // a full state (psi and pi): the first step, a pure drift, is formed while
    // the momentum uploads (the link bounds the upload)
    const bool drift = f0 && f1 && f2 && f3;
    for (int pr = 0; pr < 2; ++pr) {
        void *dst = pr == 0 ? L->psi[L->cur] : L->pih;
        if (src[2 * pr] && src[2 * pr + 1]) {
            upload_pair<S>(L, src[2 * pr], src[2 * pr + 1], dst, drift && pr == 1);
            continue;
        }
        for (int f = 2 * pr; f < 2 * pr + 2; ++f) {   // one component of the pair
            if (!src[f]) continue;
            void *st = stage(L);
            AXS_CUDA(cudaMemcpyAsync(st, src[f], (size_t)L->length * sizeof(S), cudaMemcpyHostToDevice, L->stream));
            launch_pack(L, st, is_d, pr, f & 1);
        }
    }
    L->fresh = drift ? 2 : 1;
    L->last_nplaq = -1;
    L->list_valid = false;
    AXS_CUDA(cudaStreamSynchronize(L->stream));
}

template <typename S>
static void download_fields(Lattice *L, S *f0, S *f1, S *f2, S *f3) {
    S *dst[4] = {f0, f1, f2, f3};
    const int is_d = sizeof(S) == 8;
    if (f2 || f3) launch_sync_pi(L);
    for (int pr = 0; pr < 2; ++pr) {
        const void *src = pr == 1 ? L->scratch : L->psi[L->cur];
        if (dst[2 * pr] && dst[2 * pr + 1]) {
            download_pair<S>(L, src, dst[2 * pr], dst[2 * pr + 1]);
            continue;
        }
        for (int f = 2 * pr; f < 2 * pr + 2; ++f) {
            if (!dst[f]) continue;
            void *st = stage(L);
            launch_unpack(L, src, 0, f & 1, st, is_d);
            AXS_CUDA(cudaMemcpyAsync(dst[f], st, (size_t)L->length * sizeof(S), cudaMemcpyDeviceToHost, L->stream));
            AXS_CUDA(cudaStreamSynchronize(L->stream));
        }
    }
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    check_device_errors(L);
}

struct CkptHeader {
    char magic[8];
    int32_t version, NDIMS, N, esz;
    int32_t fresh, pad;
    double tau;
    int64_t steps;
};

}  // namespace axs

using namespace axs;

#define API_BEGIN try {
#define API_END                                                   \
    }                                                             \
    catch (const axs::Error &e) {                                 \
        set_last_error(e.code, e.msg);                            \
        return e.code;                                            \
    }                                                             \
    catch (const std::bad_alloc &) {                              \
        set_last_error(AXS_ERR_NOMEM, "host allocation failed");  \
        return AXS_ERR_NOMEM;                                     \
    }                                                             \
    catch (...) {                                                 \
        set_last_error(AXS_ERR_CUDA, "unexpected internal error");\
        return AXS_ERR_CUDA;                                      \
    }                                                             \
    return AXS_OK;

#define CHECK_HANDLE(h) \
    if (!(h)) fail(AXS_ERR_ARG, "null handle");

extern "C" {

void axs_default_params(axs_params *p) {
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->lambda = 1.0f;          // default.param:5
    p->enable_PRS = 1;         // :6
    p->T_initial = 4.0f;       // :7
    p->NDIMS = 2;              // :9
    p->N = 128;                // :10
    p->space_step = 1.0f;      // :11
    p->time_step = 0.3f;       // :12
    p->stencil_setting = 0;    // :13
    p->seed = 1998;            // :14
    p->thr = 1;                // :42
    p->precision = AXS_F64;
    p->prs = 1;
    p->tau_initial = 1.0;      // physics.cpp:50
    p->form = 0;               // vvsl_field_rescaled, the integrator s_run.cpp calls
    p->laplacian = 0;          // the sparse-matrix stencil branch, s_integrate.cpp:321-325
}

int axs_last_error(char *buf, size_t len) {
    if (buf && len) {
        snprintf(buf, len, "%s", t_err_msg.c_str());
    }
    return t_err_code;
}

int axs_create(const axs_params *p, axs_lattice **out) {
    API_BEGIN
    if (!p || !out) fail(AXS_ERR_ARG, "null argument");
    *out = nullptr;
    axs_lattice *h = new axs_lattice();
    try {
        lattice_init(&h->L, *p, nullptr);
    } catch (...) {
        lattice_free(&h->L);
        delete h;
        throw;
    }
    *out = h;
    API_END
}

int axs_destroy(axs_lattice *h) {
    API_BEGIN
    if (!h) return AXS_OK;
    if (h->L.in_ensemble) fail(AXS_ERR_STATE, "ensemble members are destroyed with their ensemble");
    lattice_free(&h->L);
    delete h;
    API_END
}

int axs_upload(axs_lattice *h, const double *a, const double *b, const double *c, const double *d) {
    API_BEGIN
    CHECK_HANDLE(h);
    upload_fields<double>(&h->L, a, b, c, d);
    API_END
}
int axs_upload_f32(axs_lattice *h, const float *a, const float *b, const float *c, const float *d) {
    API_BEGIN
    CHECK_HANDLE(h);
    upload_fields<float>(&h->L, a, b, c, d);
    API_END
}
int axs_download(axs_lattice *h, double *a, double *b, double *c, double *d) {
    API_BEGIN
    CHECK_HANDLE(h);
    download_fields<double>(&h->L, a, b, c, d);
    API_END
}
int axs_download_f32(axs_lattice *h, float *a, float *b, float *c, float *d) {
    API_BEGIN
    CHECK_HANDLE(h);
    download_fields<float>(&h->L, a, b, c, d);
    API_END
}

int axs_get_time(axs_lattice *h, double *tau, int64_t *steps) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (tau) *tau = h->L.tau;
    if (steps) *steps = h->L.steps;
    API_END
}
int axs_set_time(axs_lattice *h, double tau, int64_t steps) {
    API_BEGIN
    CHECK_HANDLE(h);
    h->L.tau = tau;
    h->L.steps = steps;
    if (h->L.fresh == 2) h->L.fresh = 1;   // the drift formed at upload used the old time
    set_device_clock(&h->L);
    AXS_CUDA(cudaStreamSynchronize(h->L.stream));
    API_END
}

int axs_init_gaussian_thermal(axs_lattice *h, uint64_t seed) {
    API_BEGIN
    CHECK_HANDLE(h);
    Lattice *L = &h->L;
    L->tau = L->p.tau_initial;
    L->steps = 0;
    init_gaussian(L, seed, 1, 0.0);
    L->fresh = 1;
    L->last_nplaq = -1;
    set_device_clock(L);
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    API_END
}
int axs_init_flat(axs_lattice *h, uint64_t seed, double kcut) {
    API_BEGIN
    CHECK_HANDLE(h);
    Lattice *L = &h->L;
    L->tau = L->p.tau_initial;
    L->steps = 0;
    init_gaussian(L, seed, 0, kcut);
    L->fresh = 1;
    L->last_nplaq = -1;
    set_device_clock(L);
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    API_END
}

int axs_evolve(axs_lattice *h, int nsteps) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (nsteps < 0) fail(AXS_ERR_ARG, "nsteps < 0");
    if (h->L.in_ensemble) fail(AXS_ERR_STATE, "evolve ensemble members with axs_ensemble_evolve");
    h->L.last_nplaq = -1;
    lattice_evolve(&h->L, nsteps);
    API_END
}

int axs_evolve_timed(axs_lattice *h, int nsteps, double *ms) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (nsteps < 0) fail(AXS_ERR_ARG, "nsteps < 0");
    if (h->L.in_ensemble) fail(AXS_ERR_STATE, "evolve ensemble members with axs_ensemble_evolve");
    Lattice *L = &h->L;
    if (!L->tuned) lattice_evolve(L, 0);
    cudaEvent_t a, b;
    AXS_CUDA(cudaEventCreate(&a));
    AXS_CUDA(cudaEventCreate(&b));
    AXS_CUDA(cudaEventRecord(a, L->stream));
    lattice_evolve(L, nsteps);
    AXS_CUDA(cudaEventRecord(b, L->stream));
    AXS_CUDA(cudaEventSynchronize(b));
    float t = 0;
    AXS_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    check_device_errors(L);
    L->last_nplaq = -1;
    API_END
}

int axs_laplacian(axs_lattice *h, int field, double *out) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (field != AXS_PHI1 && field != AXS_PHI2) fail(AXS_ERR_ARG, "field must be AXS_PHI1 or AXS_PHI2");
    if (!out) fail(AXS_ERR_ARG, "null output");
    Lattice *L = &h->L;
    double *d = (double *)stage(L);
    launch_laplacian(L, field, d);
    AXS_CUDA(cudaMemcpyAsync(out, d, (size_t)L->length * sizeof(double), cudaMemcpyDeviceToHost, L->stream));
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    API_END
}

int axs_find_strings(axs_lattice *h, const double *theta, uint8_t *mask, int64_t *n_plaquettes, int64_t *num_cores) {
    API_BEGIN
    CHECK_HANDLE(h);
    find_strings(&h->L, theta, mask, n_plaquettes, num_cores);
    API_END
}

int axs_string_positions(axs_lattice *h, int32_t *pos, int64_t cap, int64_t *n) {
    API_BEGIN
    CHECK_HANDLE(h);
    string_positions(&h->L, pos, cap, n);
    API_END
}

int axs_xi(const axs_params *p, int64_t n_plaquettes, int64_t num_cores, double tau, float *xi) {
    API_BEGIN
    if (!p || !xi) fail(AXS_ERR_ARG, "null argument");
    // physical_time() and scale_factor() return float (physics.cpp:43-50)
    float t_phys = (float)(0.5f * (tau * tau));
    float a = (float)tau;
    float side = p->N * p->space_step * a;
    if (p->NDIMS == 2) {                                   // s_run.cpp:111-114
        float area = (float)((double)side * (double)side);
        *xi = (float)((int)num_cores * ((double)t_phys * (double)t_phys) / area);
    } else {                                               // s_run.cpp:123-129
        float total_length = (int)n_plaquettes * 2.0f / 3.0f;
        float physical_length = total_length * a;
        float volume = (float)((double)side * (double)side * (double)side);
        *xi = (float)(physical_length * ((double)t_phys * (double)t_phys) / volume);
    }
    API_END
}

int axs_powerspec(axs_lattice *h, int field, double *pk, double *ks, int *count) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (field < AXS_PHI1 || field > AXS_PHIDOT2) fail(AXS_ERR_ARG, "bad field id %d", field);
    if (!pk || !ks || !count) fail(AXS_ERR_ARG, "null output");
    powerspec(&h->L, field, pk, ks, count);
    API_END
}

int axs_axion_spectrum(axs_lattice *h, int nbins, double *kmean, double *pk, int64_t *count) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (!kmean || !pk || !count) fail(AXS_ERR_ARG, "null output");
    axion_spectrum(&h->L, nbins, kmean, pk, count);
    API_END
}

int axs_background(axs_lattice *h, double out[6]) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (!out) fail(AXS_ERR_ARG, "null output");
    background(&h->L, out);
    API_END
}

int axs_energies(axs_lattice *h, double out[3]) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (!out) fail(AXS_ERR_ARG, "null output");
    energies(&h->L, out);
    API_END
}

int axs_check_finite(axs_lattice *h, int *finite) {
    API_BEGIN
    CHECK_HANDLE(h);
    int ok = check_finite(&h->L);
    if (finite) *finite = ok;
    if (!ok) {
        set_last_error(AXS_ERR_NONFINITE, "NaN or Inf in the fields");
        return AXS_ERR_NONFINITE;
    }
    API_END
}

int axs_field_distance(axs_lattice *a, axs_lattice *b, double out[8]) {
    API_BEGIN
    if (!a || !b || !out) fail(AXS_ERR_ARG, "null argument");
    field_distance(&a->L, &b->L, out);
    API_END
}

int axs_checkpoint_size(axs_lattice *h, size_t *bytes) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (!bytes) fail(AXS_ERR_ARG, "null output");
    *bytes = sizeof(CkptHeader) + (size_t)h->L.length * 2 * h->L.esz * 2;
    API_END
}

int axs_checkpoint(axs_lattice *h, void *buf, size_t bytes) {
    API_BEGIN
    CHECK_HANDLE(h);
    Lattice *L = &h->L;
    size_t cb = (size_t)L->length * 2 * L->esz;
    if (!buf || bytes < sizeof(CkptHeader) + 2 * cb) fail(AXS_ERR_ARG, "checkpoint buffer too small");
    CkptHeader hd;
    memset(&hd, 0, sizeof hd);
    memcpy(hd.magic, "AXSCKPT1", 8);
    hd.version = 1;
    hd.NDIMS = L->p.NDIMS;
    hd.N = L->p.N;
    hd.esz = L->esz;
    hd.fresh = L->fresh ? 1 : 0;   // psi[cur ^ 1] is not saved
    hd.tau = L->tau;
    hd.steps = L->steps;
    memcpy(buf, &hd, sizeof hd);
    char *b = (char *)buf + sizeof hd;
    AXS_CUDA(cudaMemcpyAsync(b, L->psi[L->cur], cb, cudaMemcpyDeviceToHost, L->stream));
    AXS_CUDA(cudaMemcpyAsync(b + cb, L->pih, cb, cudaMemcpyDeviceToHost, L->stream));
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    API_END
}

int axs_restore(axs_lattice *h, const void *buf, size_t bytes) {
    API_BEGIN
    CHECK_HANDLE(h);
    Lattice *L = &h->L;
    size_t cb = (size_t)L->length * 2 * L->esz;
    if (!buf || bytes < sizeof(CkptHeader) + 2 * cb) fail(AXS_ERR_ARG, "checkpoint buffer too small");
    CkptHeader hd;
    memcpy(&hd, buf, sizeof hd);
    if (memcmp(hd.magic, "AXSCKPT1", 8) != 0 || hd.version != 1) fail(AXS_ERR_ARG, "not a checkpoint");
    if (hd.NDIMS != L->p.NDIMS || hd.N != L->p.N || hd.esz != L->esz)
        fail(AXS_ERR_ARG, "checkpoint shape/precision does not match the lattice");
    const char *b = (const char *)buf + sizeof hd;
    AXS_CUDA(cudaMemcpyAsync(L->psi[L->cur], b, cb, cudaMemcpyHostToDevice, L->stream));
    AXS_CUDA(cudaMemcpyAsync(L->pih, b + cb, cb, cudaMemcpyHostToDevice, L->stream));
    L->fresh = hd.fresh;
    L->tau = hd.tau;
    L->steps = hd.steps;
    L->last_nplaq = -1;
    set_device_clock(L);
    AXS_CUDA(cudaStreamSynchronize(L->stream));
    API_END
}

int axs_ensemble_create(const axs_params *members, int n, axs_ensemble **out) {
    API_BEGIN
    if (!members || n < 1 || !out) fail(AXS_ERR_ARG, "bad ensemble arguments");
    *out = nullptr;
    for (int i = 1; i < n; ++i) {
        const axs_params &a = members[0], &b = members[i];
        if (a.NDIMS != b.NDIMS || a.precision != b.precision || a.time_step != b.time_step ||
            a.space_step != b.space_step || a.stencil_setting != b.stencil_setting || a.form != b.form ||
            a.laplacian != b.laplacian)
            fail(AXS_ERR_ARG, "ensemble members must share NDIMS, precision, dt, dx, stencil, form and Laplacian");
    }
    axs_ensemble *e = new axs_ensemble();
    try {
        AXS_CUDA(cudaStreamCreateWithFlags(&e->E.stream, cudaStreamNonBlocking));
        for (int i = 0; i < n; ++i) {
            axs_lattice *m = new axs_lattice();
            e->members.push_back(m);
            lattice_init(&m->L, members[i], e->E.stream);
            m->L.in_ensemble = true;
            e->E.members.push_back(&m->L);
        }
        ensemble_setup(&e->E);
    } catch (...) {
        for (axs_lattice *m : e->members) { lattice_free(&m->L); delete m; }
        if (e->E.stream) cudaStreamDestroy(e->E.stream);
        delete e;
        throw;
    }
    *out = e;
    API_END
}

int axs_ensemble_destroy(axs_ensemble *e) {
    API_BEGIN
    if (!e) return AXS_OK;
    cudaStreamSynchronize(e->E.stream);
    if (e->E.hpin) cudaFreeHost(e->E.hpin);
    ensemble_release_pool(&e->E);
    clear_graphs(e->E.graphs);
    dfree(e->E.dzlat);
    dfree(e->E.dcounter);
    dfree(e->E.derr);
    for (axs_lattice *m : e->members) { lattice_free(&m->L); delete m; }
    cudaStreamDestroy(e->E.stream);
    delete e;
    API_END
}

int axs_ensemble_member(axs_ensemble *e, int i, axs_lattice **out) {
    API_BEGIN
    if (!e || !out || i < 0 || i >= (int)e->members.size()) fail(AXS_ERR_ARG, "bad member index");
    *out = e->members[i];
    API_END
}

int axs_ensemble_evolve(axs_ensemble *e, int nsteps) {
    API_BEGIN
    if (!e) fail(AXS_ERR_ARG, "null ensemble");
    if (nsteps < 0) fail(AXS_ERR_ARG, "nsteps < 0");
    for (Lattice *m : e->E.members) m->last_nplaq = -1;
    ensemble_evolve(&e->E, nsteps);
    API_END
}

int axs_ensemble_evolve_timed(axs_ensemble *e, int nsteps, double *ms) {
    API_BEGIN
    if (!e) fail(AXS_ERR_ARG, "null ensemble");
    if (nsteps < 0) fail(AXS_ERR_ARG, "nsteps < 0");
    if (!e->E.tuned) ensemble_evolve(&e->E, 0);
    cudaEvent_t a, b;
    AXS_CUDA(cudaEventCreate(&a));
    AXS_CUDA(cudaEventCreate(&b));
    AXS_CUDA(cudaEventRecord(a, e->E.stream));
    ensemble_evolve(&e->E, nsteps);
    AXS_CUDA(cudaEventRecord(b, e->E.stream));
    AXS_CUDA(cudaEventSynchronize(b));
    float t = 0;
    AXS_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    check_device_error_flag(e->E.derr, e->E.stream);
    for (Lattice *m : e->E.members) m->last_nplaq = -1;
    API_END
}

int axs_ensemble_find_strings(axs_ensemble *e, int64_t *n_plaquettes, int64_t *num_cores) {
    API_BEGIN
    if (!e || !n_plaquettes || !num_cores) fail(AXS_ERR_ARG, "null argument");
    ensemble_find_strings(&e->E, n_plaquettes, num_cores);
    API_END
}

int axs_ensemble_axion_spectrum(axs_ensemble *e, int nbins, double *kmean, double *pk, int64_t *count) {
    API_BEGIN
    if (!e || !kmean || !pk || !count) fail(AXS_ERR_ARG, "null argument");
    ensemble_axion_spectrum(&e->E, nbins, kmean, pk, count);
    API_END
}

int axs_inject_wait_timeout(axs_lattice *h) {
    API_BEGIN
    CHECK_HANDLE(h);
    Lattice *L = &h->L;
    if (L->in_ensemble)
        fail(AXS_ERR_STATE, "timeout injection on an ensemble member is not supported; use a standalone lattice");
    if (!L->tuned) lattice_evolve(L, 0);   // the configuration the next step will use (tuned unless AXS_AUTOTUNE=0)
    if (L->cfg.kind != 1 || L->p.laplacian != 0)
        fail(AXS_ERR_STATE, "the step kernel in use (%s) has no device-side waits",
             L->p.laplacian != 0 ? "spectral Laplacian step" : L->cfg.describe().c_str());
    L->debug_tx_excess = 16;
    L->zlat_variant = -1;
    clear_graphs(L->graphs);
    API_END
}

int axs_autotune(axs_lattice *h) {
    API_BEGIN
    CHECK_HANDLE(h);
    lattice_autotune(&h->L);
    API_END
}

int axs_ensemble_describe(axs_ensemble *e, char *buf, size_t len) {
    API_BEGIN
    if (!e) fail(AXS_ERR_ARG, "null ensemble");
    if (buf && len) snprintf(buf, len, "%s", ensemble_describe(&e->E).c_str());
    API_END
}

int axs_describe(axs_lattice *h, char *buf, size_t len) {
    API_BEGIN
    CHECK_HANDLE(h);
    if (buf && len) {
        if (h->L.p.laplacian == 1)
            snprintf(buf, len, "spectral Laplacian step (cuFFT transform pair of the complex field per step)");
        else snprintf(buf, len, "%s", h->L.cfg.describe().c_str());
    }
    API_END
}

int64_t axs_kernel_launches(void) { return total_launches(); }

int axs_set_device(int device) {
    API_BEGIN
    AXS_CUDA(cudaSetDevice(device));
    API_END
}

int axs_host_alloc(size_t bytes, void **out) {
    API_BEGIN
    if (!out) fail(AXS_ERR_ARG, "null output");
    AXS_CUDA(cudaMallocHost(out, bytes));
    API_END
}
int axs_host_free(void *p) {
    API_BEGIN
    if (p) AXS_CUDA(cudaFreeHost(p));
    API_END
}

}  // extern "C"
