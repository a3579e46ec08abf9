/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the reference TBSLA CPU algorithms on the SpMV /
 * PageRank / CG path.  Only the test suite, the smoke check and the CPU
 * baseline leg of bench.py load it, and only as the checker: the product
 * library never links, calls or falls back to anything in this directory.
 *
 * Every function cites the reference file:line it restates (paths are
 * relative to the TBSLA source tree).
 */
#ifndef TBSLA_ORACLE_H
#define TBSLA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- SpMV restatements (Ax semantics of each format) ------------------- */
void orc_csr_ax(int ln_row, int f_col, long nnz, const double* values,
                const int* rowptr, const int* colidx, const double* v, double* r);
void orc_csr_ax_omp(int ln_row, int f_col, long nnz, const double* values,
                    const int* rowptr, const int* colidx, const double* v, double* r);
void orc_csr_ax_f32_omp(int ln_row, int f_col, long nnz, const float* values,
                        const int* rowptr, const int* colidx, const double* v, double* r);
void orc_csr_absrow(int ln_row, int f_col, const double* values, const int* rowptr,
                    const int* colidx, const double* v, double* out);
void orc_ell_ax(int ln_row, int max_col, int f_col, long nnz, const double* values,
                const int* columns, const double* v, double* r);
void orc_coo_ax(int n_row, long nnz, const double* values, const int* row,
                const int* col, const double* v, double* r, int vect_incr);
void orc_scoo_ax(int ln_row, int f_row, int f_col, long nnz, const double* values,
                 const int* row, const int* col, const double* v, double* r, int vect_incr);
void orc_dense_ax(int ln_row, int ln_col, long nnz, const double* values,
                  const double* v, double* r);
void orc_dense_ax_omp(int ln_row, int ln_col, long nnz, const double* values,
                      const double* v, double* r);

/* ---- format conversions --------------------------------------------- */
int orc_coo_to_csr(int n_row, long nnz, const int* row, const int* col, const double* val,
                   int* rowptr, int* colidx, double* values);
int orc_ell_max_col(int n_row, long nnz, const int* row);
int orc_coo_to_ell(int n_row, long nnz, const int* row, const int* col, const double* val,
                   int max_col, int* columns, double* values);
void orc_coo_to_dense(int ln_row, int ln_col, long nnz, const int* row, const int* col,
                      const double* val, double* dense);

/* ---- composite ops --------------------------------------------------- */
void orc_csr_col_sums(int ln_row, int f_col, long nnz, const double* values,
                      const int* rowptr, const int* colidx, double* s);
void orc_csr_normalize_cols(int ln_row, int f_col, long nnz, double* values,
                            const int* rowptr, const int* colidx, const double* s);

/* ---- SpMM and sparse-softmax helpers (CSR) */
void orc_csr_dense_multiply(int n_row, const double* values, const int* rowptr, const int* colidx,
                            const double* B, double* Cm, int cols_B);
void orc_csr_row_max_abs(int ln_row, const double* values, const int* rowptr, double* max_abs);
void orc_csr_row_sums(int ln_row, const double* values, const int* rowptr, double* s);
void orc_csr_normalize_rows(int ln_row, double* values, const int* rowptr, const double* s);
void orc_csr_apply_exponential(int ln_row, double* values, const int* rowptr, const double* max_abs,
                               int base);

/* ---- PageRank / CG restatements (reference bugs fixed, see tbsla_oracle.c) */
int orc_pagerank(int n, const int* rowptr, const int* colidx, const double* values,
                 const double* teleport, double beta, double epsilon, int max_iterations,
                 int stop_early, double* x, double* last_error);
int orc_cg(int n, const int* rowptr, const int* colidx, const double* values,
           const double* diag_inv, const double* b, double* x, int max_iterations,
           double rel_tol, double* rel_residual);

/* ---- the power-law workload matrix (this library's generator, restated) */
long orc_gen_powerlaw_rows(int n, double mean_len, double zipf_s, int max_len, double local_frac, int band,
                           unsigned long long seed, int* rowptr);
void orc_gen_powerlaw_entries(int n, double local_frac, int band, unsigned long long seed,
                              const int* rowptr, int* colidx, double* values);
void orc_gen_uniform(double* out, long n, double lo, double hi, unsigned long long seed);

#ifdef __cplusplus
}
#endif

#endif
