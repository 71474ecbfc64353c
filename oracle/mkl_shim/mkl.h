/* MKL-API shim: the subset of Intel MKL's C interface that the reference's CPU minimizer
 * (src/cpp/cpp_mkl_minimizer.cpp of MaMMoS-project/mumag_matrixfree2) calls.
 *
 * TEST INFRASTRUCTURE ONLY (oracle).  Intel MKL is not installed on either machine of this
 * project, so the reference's translation unit is compiled unchanged against this header and
 * mkl_shim.cpp.  Declared here, written from MKL's public documentation:
 *
 *   inspector-executor sparse BLAS   mkl_sparse_d_create_csr, mkl_sparse_optimize,
 *                                    mkl_sparse_d_mv, mkl_sparse_destroy
 *                                    (cpp_mkl_minimizer.cpp:185-186,214,282,558-562,758-760)
 *   CBLAS level 1                    cblas_ddot, cblas_daxpy, cblas_daxpby, cblas_dscal,
 *                                    cblas_dnrm2, cblas_idamax  (:205,271,298,311-345,604,691)
 *   PARDISO                          pardiso  (:52,78,103)
 *
 * Deviation: PARDISO is a sparse direct solver.  The shim's pardiso() solves the symmetric
 * positive definite system by conjugate gradients preconditioned with a smoothed-aggregation
 * V-cycle to a relative residual of 1e-12 (settable with mkl_shim_set_pardiso_tol), which is
 * far below every tolerance the reference's results are compared at.
 */
#ifndef MUMAG_ORACLE_MKL_SHIM_H
#define MUMAG_ORACLE_MKL_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MKL_INT;
typedef size_t CBLAS_INDEX;

typedef enum {
    SPARSE_STATUS_SUCCESS = 0,
    SPARSE_STATUS_NOT_INITIALIZED = 1,
    SPARSE_STATUS_ALLOC_FAILED = 2,
    SPARSE_STATUS_INVALID_VALUE = 3,
    SPARSE_STATUS_EXECUTION_FAILED = 4,
    SPARSE_STATUS_INTERNAL_ERROR = 5,
    SPARSE_STATUS_NOT_SUPPORTED = 6
} sparse_status_t;

typedef enum {
    SPARSE_OPERATION_NON_TRANSPOSE = 10,
    SPARSE_OPERATION_TRANSPOSE = 11,
    SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12
} sparse_operation_t;

typedef enum {
    SPARSE_MATRIX_TYPE_GENERAL = 20,
    SPARSE_MATRIX_TYPE_SYMMETRIC = 21,
    SPARSE_MATRIX_TYPE_HERMITIAN = 22,
    SPARSE_MATRIX_TYPE_TRIANGULAR = 23,
    SPARSE_MATRIX_TYPE_DIAGONAL = 24,
    SPARSE_MATRIX_TYPE_BLOCK_TRIANGULAR = 25,
    SPARSE_MATRIX_TYPE_BLOCK_DIAGONAL = 26
} sparse_matrix_type_t;

typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;

typedef enum {
    SPARSE_FILL_MODE_LOWER = 40,
    SPARSE_FILL_MODE_UPPER = 41,
    SPARSE_FILL_MODE_FULL = 42
} sparse_fill_mode_t;

typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;

struct matrix_descr {
    sparse_matrix_type_t type;
    sparse_fill_mode_t mode;
    sparse_diag_type_t diag;
};

struct mkl_shim_csr;
typedef struct mkl_shim_csr* sparse_matrix_t;

/* Sparse BLAS: a handle records the caller's CSR arrays (it does not copy them). */
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t* A, sparse_index_base_t indexing, MKL_INT rows,
                                        MKL_INT cols, MKL_INT* rows_start, MKL_INT* rows_end,
                                        MKL_INT* col_indx, double* values);
sparse_status_t mkl_sparse_optimize(sparse_matrix_t A);
/* y = alpha * op(A) x + beta * y (y is not read when beta == 0); general matrices only */
sparse_status_t mkl_sparse_d_mv(sparse_operation_t operation, double alpha, sparse_matrix_t A,
                                struct matrix_descr descr, const double* x, double beta, double* y);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t A);

/* CBLAS level 1 */
double cblas_ddot(MKL_INT n, const double* x, MKL_INT incx, const double* y, MKL_INT incy);
void cblas_daxpy(MKL_INT n, double a, const double* x, MKL_INT incx, double* y, MKL_INT incy);
void cblas_daxpby(MKL_INT n, double a, const double* x, MKL_INT incx, double b, double* y, MKL_INT incy);
void cblas_dscal(MKL_INT n, double a, double* x, MKL_INT incx);
double cblas_dnrm2(MKL_INT n, const double* x, MKL_INT incx);
CBLAS_INDEX cblas_idamax(MKL_INT n, const double* x, MKL_INT incx);

/* PARDISO (real matrices; phases 11, 12, 13, 22, 23, 33, 0 and -1; nrhs = 1).  For mtype 2 / -2 the
 * upper triangle of the CSR arrays is read, as PARDISO requires; iparm[34] != 0 selects zero-based
 * indices.  error: 0 success, -1 bad input, -2 out of memory, -4 the iteration did not converge. */
void pardiso(void** pt, const MKL_INT* maxfct, const MKL_INT* mnum, const MKL_INT* mtype, const MKL_INT* phase,
             const MKL_INT* n, const void* a, const MKL_INT* ia, const MKL_INT* ja, MKL_INT* perm,
             const MKL_INT* nrhs, MKL_INT* iparm, const MKL_INT* msglvl, void* b, void* x, MKL_INT* error);

/* Shim-only controls and statistics (not part of MKL). */
void mkl_shim_set_pardiso_tol(double tol);
double mkl_shim_get_pardiso_tol(void);
/* iterations and true relative residual of the last pardiso() solve phase on this thread */
int mkl_shim_last_iterations(void);
double mkl_shim_last_relres(void);
/* levels and rows per level of the hierarchy held by a pardiso handle (pt): returns the level count */
int mkl_shim_hierarchy(void** pt, int* rows_out, int max_levels);
/* OpenMP threads a parallel region of the shim uses (1 without OpenMP) */
int mkl_shim_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
