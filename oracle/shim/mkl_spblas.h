/* Project-written stand-in for the MKL sparse BLAS (inspector-executor) subset
 * the reference calls (src/common/mkl_wrapper.cpp:3-17, src/standard/
 * s_integrate.cpp:147,322,324, src/tests/fdm_matrix.cpp:56-90). Semantics
 * follow MKL's documentation: a COO handle; mv computes
 * y = alpha*op(A)*x + beta*y, where a SYMMETRIC descriptor with fill mode UPPER
 * reads only stored entries with col >= row and mirrors the strict upper part. */
#ifndef AXS_SHIM_MKL_SPBLAS_H
#define AXS_SHIM_MKL_SPBLAS_H
#include "mkl.h"
typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_INITIALIZED = 1, SPARSE_STATUS_ALLOC_FAILED = 2,
               SPARSE_STATUS_INVALID_VALUE = 3, SPARSE_STATUS_EXECUTION_FAILED = 4,
               SPARSE_STATUS_INTERNAL_ERROR = 5, SPARSE_STATUS_NOT_SUPPORTED = 6 } sparse_status_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11,
               SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_SYMMETRIC = 21 } sparse_matrix_type_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41, SPARSE_FILL_MODE_FULL = 42 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
struct matrix_descr { sparse_matrix_type_t type; sparse_fill_mode_t mode; sparse_diag_type_t diag; };
struct sparse_matrix;
typedef struct sparse_matrix *sparse_matrix_t;
#ifdef __cplusplus
extern "C" {
#endif
sparse_status_t mkl_sparse_d_create_coo(sparse_matrix_t *A, const sparse_index_base_t indexing, const MKL_INT rows,
                                        const MKL_INT cols, const MKL_INT nnz, MKL_INT *row_indx, MKL_INT *col_indx, double *values);
sparse_status_t mkl_sparse_s_create_coo(sparse_matrix_t *A, const sparse_index_base_t indexing, const MKL_INT rows,
                                        const MKL_INT cols, const MKL_INT nnz, MKL_INT *row_indx, MKL_INT *col_indx, float *values);
sparse_status_t mkl_sparse_d_mv(const sparse_operation_t operation, const double alpha, const sparse_matrix_t A,
                                const struct matrix_descr descr, const double *x, const double beta, double *y);
sparse_status_t mkl_sparse_s_mv(const sparse_operation_t operation, const float alpha, const sparse_matrix_t A,
                                const struct matrix_descr descr, const float *x, const float beta, float *y);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t A);
sparse_status_t mkl_sparse_convert_csr(const sparse_matrix_t source, const sparse_operation_t operation, sparse_matrix_t *dest);
sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t source, sparse_index_base_t *indexing, MKL_INT *rows, MKL_INT *cols,
                                        MKL_INT **rows_start, MKL_INT **rows_end, MKL_INT **col_indx, double **values);
sparse_status_t mkl_sparse_s_export_csr(const sparse_matrix_t source, sparse_index_base_t *indexing, MKL_INT *rows, MKL_INT *cols,
                                        MKL_INT **rows_start, MKL_INT **rows_end, MKL_INT **col_indx, float **values);
#ifdef __cplusplus
}
#endif
#endif
