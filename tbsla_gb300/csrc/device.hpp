// Interface between the C ABI (capi.cpp, host compiler) and the CUDA side
// (device.cu).  Plain pointers only.
#pragma once

#include <cstddef>

#include "host/matrix.hpp"

struct tbsla_mpnn;

namespace tbsla_impl {

int dev_select(int device);
// Device of the compute calls, after checking that it is usable.
int dev_ready(int* device);
int dev_host_alloc(void** p, size_t bytes);
int dev_host_free(void* p);

int dev_upload(const tbsla_matrix* m);
int dev_bytes(const tbsla_matrix* m, size_t* bytes);
int dev_launches(const tbsla_matrix* m, int* launches);

// Ax / spmv.  host = true: r and v are host pointers, copied in and out.
int dev_ax(const tbsla_matrix* m, double* r, const double* v, int vect_incr, bool zero_first,
           bool host, void* stream);
int dev_a_axpx(const tbsla_matrix* m, double* r, const double* v, int vect_incr);
int dev_aaxpax(const tbsla_matrix* m, double* r, const double* v, double* buffer, int vect_incr,
               bool plus_x);

int dev_col_sums(tbsla_matrix* m, double* s, bool zero_first);
int dev_normalize_cols(tbsla_matrix* m, const double* s);
int dev_make_stochastic(tbsla_matrix* m, double* s);

// MatrixCSR::dense_multiply, get_row_max_abs, apply_exponential (host buffers).
int dev_dense_multiply(const tbsla_matrix* m, const double* B, double* C, int cols);
int dev_row_max_abs(const tbsla_matrix* m, double* max_abs);
// MatrixCSR::get_row_sums / normalize_rows (host buffers).
int dev_row_sums(const tbsla_matrix* m, double* s);
int dev_normalize_rows(tbsla_matrix* m, const double* s);
int dev_apply_exponential(tbsla_matrix* m, const double* max_abs, int base);

int dev_page_rank(tbsla_matrix* m, double beta, double eps, int max_it, double* result,
                  int* iterations, double* error);
int dev_page_rank_batched(tbsla_matrix* m, int nvec, const double* tele, double beta, double eps,
                          int max_it, double* result, int* iterations);

int dev_cg(tbsla_matrix* m, const double* b, double* x, int max_it, double rel_tol, int precond,
           int refresh, int* iterations, double* rel_residual);

// COO -> CSR ordering on the GPU: start[n_row + 1] row starts and perm[n]
// the storage indices in (row, col) order, ties in storage order.
int dev_coo_order(const int* row, const int* col, long n, int n_row, int n_col, long* start, long* perm);
// COO -> DENSE on the GPU (MatrixDENSE.cpp:15-37): entries ordered by the
// radix sort, duplicates summed in storage order from 0, the ln_row x
// ln_col row-major result copied to dense_host.
int dev_coo_to_dense(const int* row, const int* col, const double* val, long n, int ln_row, int ln_col,
                     double* dense_host);

// Autotuner: times the CSR kernel configurations, keeps the fastest.
int dev_autotune(tbsla_matrix* m, int reps, tbsla_tuning* best, tbsla_tuning* trials, int max_trials,
                 int* ntrials);

// Merge-path CSR SpMV on caller-owned device arrays with file-scope scratch
// (allocates nothing); n_row + nnz at most dev_noalloc_max_items().
long dev_noalloc_max_items();
int dev_csr_ax_noalloc(int n_row, long nnz, int f_col, const int* rowptr, const int* colidx,
                       const double* values, const double* v, double* r, void* stream);

// The learned factor of every system of a batch, computed on the device from
// the batch's diagonal-slot copy of A (FP64 values a64[k * n + i], slot deltas
// adelta[sys * 8 + k], row_sys[i] the system of row i) and written straight
// into the batch's diagonal-slot factor lvals[q * n + i] in lprec (F32 /
// BF16; slot deltas ldelta: slot 0 the diagonal, then A's negative deltas).
// TBSLA_ERR_BAD_MATRIX when a diagonal entry of A is <= 0.
int mpnn_factor_dia(tbsla_mpnn* net, long n, int K, const double* a64, const int* adelta, const int* row_sys,
                    int KL, const int* ldelta, void* lvals, int lprec, void* stream);

}  // namespace tbsla_impl
