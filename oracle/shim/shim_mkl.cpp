/* Project-written implementations behind oracle/shim/mkl*.h (test
 * infrastructure only). Only what the reference calls is implemented. */
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "mkl.h"
#include "mkl_vsl.h"
#include "mkl_spblas.h"
#include "../orc_philox.h"

struct sparse_matrix {
    MKL_INT rows, cols;
    std::vector<MKL_INT> r, c;          /* COO as handed over */
    std::vector<double> v;
    /* symmetric/upper expansion, built on first use, as CSR */
    bool sym_built = false;
    std::vector<long> sym_ptr;
    std::vector<MKL_INT> sym_col;
    std::vector<double> sym_val;
    /* CSR export buffers */
    std::vector<MKL_INT> csr_start, csr_end, csr_col;
    std::vector<double> csr_val;
    std::vector<float> csr_valf;
};

template <typename T>
static sparse_status_t create_coo(sparse_matrix_t *A, sparse_index_base_t base, MKL_INT rows, MKL_INT cols, MKL_INT nnz,
                                  MKL_INT *ri, MKL_INT *ci, T *val) {
    if (!A || rows < 0 || cols < 0 || nnz < 0) return SPARSE_STATUS_INVALID_VALUE;
    sparse_matrix *m = new sparse_matrix();
    m->rows = rows; m->cols = cols;
    int off = (base == SPARSE_INDEX_BASE_ONE) ? 1 : 0;
    m->r.resize(nnz); m->c.resize(nnz); m->v.resize(nnz);
    for (MKL_INT q = 0; q < nnz; ++q) { m->r[q] = ri[q] - off; m->c[q] = ci[q] - off; m->v[q] = (double)val[q]; }
    /* MKL would keep pointing at the caller's arrays and never free them; the
     * reference never touches them after creating the handle
     * (s_integrate.cpp:147-148), so the shim keeps a copy and releases them. */
    free(ri); free(ci); free(val);
    *A = m;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_create_coo(sparse_matrix_t *A, const sparse_index_base_t b, const MKL_INT rows,
        const MKL_INT cols, const MKL_INT nnz, MKL_INT *ri, MKL_INT *ci, double *v) { return create_coo(A, b, rows, cols, nnz, ri, ci, v); }
extern "C" sparse_status_t mkl_sparse_s_create_coo(sparse_matrix_t *A, const sparse_index_base_t b, const MKL_INT rows,
        const MKL_INT cols, const MKL_INT nnz, MKL_INT *ri, MKL_INT *ci, float *v) { return create_coo(A, b, rows, cols, nnz, ri, ci, v); }

static void build_sym(sparse_matrix *m) {
    if (m->sym_built) return;
    long n = m->rows;
    std::vector<long> cnt(n + 1, 0);
    for (size_t q = 0; q < m->r.size(); ++q) {
        if (m->c[q] < m->r[q]) continue;
        cnt[m->r[q] + 1]++;
        if (m->c[q] != m->r[q]) cnt[m->c[q] + 1]++;
    }
    for (long i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    m->sym_ptr = cnt;
    m->sym_col.resize(cnt[n]); m->sym_val.resize(cnt[n]);
    std::vector<long> pos(cnt.begin(), cnt.end() - 1);
    for (size_t q = 0; q < m->r.size(); ++q) {
        MKL_INT r = m->r[q], c = m->c[q];
        if (c < r) continue;
        m->sym_col[pos[r]] = c; m->sym_val[pos[r]++] = m->v[q];
        if (c != r) { m->sym_col[pos[c]] = r; m->sym_val[pos[c]++] = m->v[q]; }
    }
    m->sym_built = true;
}

template <typename T>
static sparse_status_t mv(sparse_operation_t op, T alpha, sparse_matrix_t A, matrix_descr d, const T *x, T beta, T *y) {
    if (!A) return SPARSE_STATUS_NOT_INITIALIZED;
    if (op != SPARSE_OPERATION_NON_TRANSPOSE) return SPARSE_STATUS_NOT_SUPPORTED;
    long n = A->rows;
    if (d.type == SPARSE_MATRIX_TYPE_SYMMETRIC) {
        if (d.mode != SPARSE_FILL_MODE_UPPER) return SPARSE_STATUS_NOT_SUPPORTED;
        build_sym(A);
        const long *ptr = A->sym_ptr.data();
        const MKL_INT *col = A->sym_col.data();
        const double *val = A->sym_val.data();
        #pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            T acc = 0;
            for (long q = ptr[i]; q < ptr[i + 1]; ++q) acc += (T)val[q] * x[col[q]];
            y[i] = (beta == (T)0) ? alpha * acc : alpha * acc + beta * y[i];
        }
        return SPARSE_STATUS_SUCCESS;
    }
    std::vector<T> acc(n, (T)0);
    for (size_t q = 0; q < A->r.size(); ++q) acc[A->r[q]] += (T)A->v[q] * x[A->c[q]];
    for (long i = 0; i < n; ++i) y[i] = (beta == (T)0) ? alpha * acc[i] : alpha * acc[i] + beta * y[i];
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_mv(const sparse_operation_t op, const double alpha, const sparse_matrix_t A,
        const struct matrix_descr d, const double *x, const double beta, double *y) { return mv(op, alpha, A, d, x, beta, y); }
extern "C" sparse_status_t mkl_sparse_s_mv(const sparse_operation_t op, const float alpha, const sparse_matrix_t A,
        const struct matrix_descr d, const float *x, const float beta, float *y) { return mv(op, alpha, A, d, x, beta, y); }

extern "C" sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) { delete A; return SPARSE_STATUS_SUCCESS; }

/* General (as stored) COO -> CSR with duplicates summed and columns sorted. */
extern "C" sparse_status_t mkl_sparse_convert_csr(const sparse_matrix_t s, const sparse_operation_t op, sparse_matrix_t *dest) {
    if (!s || !dest) return SPARSE_STATUS_NOT_INITIALIZED;
    if (op != SPARSE_OPERATION_NON_TRANSPOSE) return SPARSE_STATUS_NOT_SUPPORTED;
    sparse_matrix *m = new sparse_matrix();
    m->rows = s->rows; m->cols = s->cols;
    std::vector<std::vector<std::pair<MKL_INT, double>>> rowsv(s->rows);
    for (size_t q = 0; q < s->r.size(); ++q) {
        auto &rv = rowsv[s->r[q]];
        bool merged = false;
        for (auto &e : rv) if (e.first == s->c[q]) { e.second += s->v[q]; merged = true; break; }
        if (!merged) rv.push_back(std::make_pair(s->c[q], s->v[q]));
    }
    for (long i = 0; i < s->rows; ++i) {
        auto &rv = rowsv[i];
        for (size_t a = 1; a < rv.size(); ++a)
            for (size_t b = a; b > 0 && rv[b - 1].first > rv[b].first; --b) std::swap(rv[b - 1], rv[b]);
        m->csr_start.push_back((MKL_INT)m->csr_col.size());
        for (auto &e : rv) { m->csr_col.push_back(e.first); m->csr_val.push_back(e.second); m->csr_valf.push_back((float)e.second);
                             m->r.push_back((MKL_INT)i); m->c.push_back(e.first); m->v.push_back(e.second); }
        m->csr_end.push_back((MKL_INT)m->csr_col.size());
    }
    *dest = m;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t s, sparse_index_base_t *ix, MKL_INT *rows, MKL_INT *cols,
        MKL_INT **rs, MKL_INT **re, MKL_INT **ci, double **v) {
    if (!s || s->csr_start.empty()) return SPARSE_STATUS_NOT_INITIALIZED;
    *ix = SPARSE_INDEX_BASE_ZERO; *rows = s->rows; *cols = s->cols;
    *rs = s->csr_start.data(); *re = s->csr_end.data(); *ci = s->csr_col.data(); *v = s->csr_val.data();
    return SPARSE_STATUS_SUCCESS;
}
extern "C" sparse_status_t mkl_sparse_s_export_csr(const sparse_matrix_t s, sparse_index_base_t *ix, MKL_INT *rows, MKL_INT *cols,
        MKL_INT **rs, MKL_INT **re, MKL_INT **ci, float **v) {
    if (!s || s->csr_start.empty()) return SPARSE_STATUS_NOT_INITIALIZED;
    *ix = SPARSE_INDEX_BASE_ZERO; *rows = s->rows; *cols = s->cols;
    *rs = s->csr_start.data(); *re = s->csr_end.data(); *ci = s->csr_col.data(); *v = s->csr_valf.data();
    return SPARSE_STATUS_SUCCESS;
}

extern "C" void cblas_daxpy(const MKL_INT n, const double a, const double *x, const MKL_INT incx, double *y, const MKL_INT incy) {
    for (MKL_INT i = 0; i < n; ++i) y[(long)i * incy] += a * x[(long)i * incx];
}
extern "C" void cblas_saxpy(const MKL_INT n, const float a, const float *x, const MKL_INT incx, float *y, const MKL_INT incy) {
    for (MKL_INT i = 0; i < n; ++i) y[(long)i * incy] += a * x[(long)i * incx];
}
extern "C" void cblas_dcopy(const MKL_INT n, const double *x, const MKL_INT incx, double *y, const MKL_INT incy) {
    for (MKL_INT i = 0; i < n; ++i) y[(long)i * incy] = x[(long)i * incx];
}
extern "C" void cblas_scopy(const MKL_INT n, const float *x, const MKL_INT incx, float *y, const MKL_INT incy) {
    for (MKL_INT i = 0; i < n; ++i) y[(long)i * incy] = x[(long)i * incx];
}

/* A stream draws array after array: call c of vdRngGaussian fills deviate m of
 * "array" c with orc_normal(seed, c, m). init.cpp:49-52 makes exactly four
 * calls of `length` deviates, so array c = 0..3 matches the GPU initialiser. */
struct vsl_stream { uint64_t seed; int calls; };

extern "C" int vslNewStream(VSLStreamStatePtr *stream, const MKL_INT brng, const MKL_UINT seed) {
    (void)brng;
    vsl_stream *s = new vsl_stream();
    s->seed = seed; s->calls = 0;
    *stream = s;
    return 0;
}
extern "C" int vslDeleteStream(VSLStreamStatePtr *stream) { delete (vsl_stream *)*stream; *stream = 0; return 0; }

extern "C" int vdRngGaussian(const MKL_INT method, VSLStreamStatePtr stream, const MKL_INT n, double r[], const double a, const double sigma) {
    (void)method;
    vsl_stream *s = (vsl_stream *)stream;
    int c = s->calls++;
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < n; ++m) r[m] = a + sigma * orc_normal(s->seed, c, m);
    return 0;
}
extern "C" int vsRngGaussian(const MKL_INT method, VSLStreamStatePtr stream, const MKL_INT n, float r[], const float a, const float sigma) {
    (void)method;
    vsl_stream *s = (vsl_stream *)stream;
    int c = s->calls++;
    #pragma omp parallel for schedule(static)
    for (long m = 0; m < n; ++m) r[m] = (float)(a + sigma * orc_normal(s->seed, c, m));
    return 0;
}
