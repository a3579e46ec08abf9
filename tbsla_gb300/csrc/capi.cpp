// extern "C" entry points of include/tbsla_gb300.h.
#include <cstring>
#include <memory>
#include <new>

#include "api_guard.hpp"
#include "device.hpp"
#include "host/matrix.hpp"
#include "tbsla_gb300.h"

using namespace tbsla_impl;

namespace {

bool valid_format(int f) { return f >= TBSLA_COO && f <= TBSLA_DENSE; }

bool sane_info(const tbsla_info* I) {
  return I && I->n_row >= 0 && I->n_col >= 0 && I->ln_row >= 0 && I->ln_col >= 0 &&
         I->f_row >= 0 && I->f_col >= 0 && I->nnz >= 0 && I->NR >= 1 && I->NC >= 1 &&
         I->max_col >= 0;
}

}  // namespace

extern "C" {

const char* tbsla_status_string(int status) {
  switch (status) {
    case TBSLA_OK: return "ok";
    case TBSLA_ERR_INVALID_ARG: return "invalid argument";
    case TBSLA_ERR_BAD_MATRIX: return "matrix arrays fail validation";
    case TBSLA_ERR_ALLOC: return "allocation failed";
    case TBSLA_ERR_CUDA: return "CUDA error";
    case TBSLA_ERR_IO: return "file missing, short or malformed";
    case TBSLA_ERR_NOT_CONVERGED: return "iteration limit reached before convergence";
    case TBSLA_ERR_TIMEOUT: return "bounded device wait timed out";
    case TBSLA_ERR_UNSUPPORTED: return "operation not supported for this format";
    case TBSLA_ERR_NO_DEVICE: return "no usable CUDA device";
  }
  return "unknown status";
}

const char* tbsla_version(void) { return "tbsla_gb300 0.1 (sm_103a)"; }

int tbsla_device_init(int device) { return dev_select(device); }

int tbsla_host_alloc(void** ptr, size_t bytes) try {
  if (!ptr) return TBSLA_ERR_INVALID_ARG;
  return dev_host_alloc(ptr, bytes);
} TBSLA_API_CATCH

int tbsla_host_free(void* ptr) { return ptr ? dev_host_free(ptr) : TBSLA_OK; }

int tbsla_matrix_create(tbsla_matrix** m, int format) try {
  if (!m || !valid_format(format)) return TBSLA_ERR_INVALID_ARG;
  *m = new (std::nothrow) tbsla_matrix();
  if (!*m) return TBSLA_ERR_ALLOC;
  (*m)->format = format;
  (*m)->info.NR = (*m)->info.NC = 1;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_destroy(tbsla_matrix* m) try {
  delete m;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_format(const tbsla_matrix* m, int* format) try {
  if (!m || !format) return TBSLA_ERR_INVALID_ARG;
  *format = m->format;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_info(const tbsla_matrix* m, tbsla_info* info) try {
  if (!m || !info) return TBSLA_ERR_INVALID_ARG;
  *info = m->info;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_set_coo(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* row, const int* col) try {
  if (!m || (m->format != TBSLA_COO && m->format != TBSLA_SCOO) || !sane_info(info))
    return TBSLA_ERR_INVALID_ARG;
  if (info->nnz > 0 && (!values || !row || !col)) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  m->info = *info;
  m->values.assign(values, info->nnz);
  m->idx0.assign(row, info->nnz);
  m->idx1.assign(col, info->nnz);
  return TBSLA_OK;
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_push_back(tbsla_matrix* m, int row, int col, double value) try {
  if (!m || (m->format != TBSLA_COO && m->format != TBSLA_SCOO)) return TBSLA_ERR_INVALID_ARG;
  if ((size_t)m->info.nnz != m->values.size()) return TBSLA_ERR_BAD_MATRIX;
  m->invalidate();
  m->values.push(value);
  m->idx0.push(row);
  m->idx1.push(col);
  m->info.nnz += 1;
  return TBSLA_OK;
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_set_csr(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* rowptr, const int* colidx) try {
  if (!m || m->format != TBSLA_CSR || !sane_info(info)) return TBSLA_ERR_INVALID_ARG;
  if (info->nnz > 0 && (!values || !rowptr || !colidx)) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  m->info = *info;
  m->values.assign(values, info->nnz);
  m->idx1.assign(colidx, info->nnz);
  if (rowptr) m->idx0.assign(rowptr, (size_t)info->ln_row + 1);
  else m->idx0.zeros((size_t)info->ln_row + 1);
  return TBSLA_OK;
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_set_ell(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* columns) try {
  if (!m || m->format != TBSLA_ELL || !sane_info(info)) return TBSLA_ERR_INVALID_ARG;
  size_t n = (size_t)info->ln_row * info->max_col;
  if (n > 0 && (!values || !columns)) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  m->info = *info;
  m->values.assign(values, n);
  m->idx0.assign(columns, n);
  m->idx1.clear();
  return TBSLA_OK;
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_set_dense(tbsla_matrix* m, const tbsla_info* info, const double* values) try {
  if (!m || m->format != TBSLA_DENSE || !sane_info(info)) return TBSLA_ERR_INVALID_ARG;
  size_t n = (size_t)info->ln_row * info->ln_col;
  if (n > 0 && !values) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  m->info = *info;
  m->values.assign(values, n);
  m->idx0.clear();
  m->idx1.clear();
  return TBSLA_OK;
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_arrays(const tbsla_matrix* m, const double** values, const int** idx0,
                        const int** idx1) try {
  if (!m) return TBSLA_ERR_INVALID_ARG;
  if (values) *values = m->values.data();
  if (idx0) *idx0 = m->idx0.data();
  if (idx1) *idx1 = m->idx1.data();
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_fill_cdiag(tbsla_matrix* m, int n_row, int n_col, int cdiag, int pr, int pc,
                            int NR, int NC) try {
  if (!m || n_row < 0 || n_col < 0 || cdiag < 0 || NR < 1 || NC < 1 || pr < 0 || pc < 0 ||
      pr >= NR || pc >= NC)
    return TBSLA_ERR_INVALID_ARG;
  return fill_cdiag(m, n_row, n_col, cdiag, pr, pc, NR, NC);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_cqmat(tbsla_matrix* m, int n_row, int n_col, int c, double q,
                            unsigned int seed_mult, int pr, int pc, int NR, int NC) try {
  if (!m || n_row < 0 || n_col <= 0 || c <= 0 || NR < 1 || NC < 1 || pr < 0 || pc < 0 ||
      pr >= NR || pc >= NC)
    return TBSLA_ERR_INVALID_ARG;
  return fill_cqmat(m, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_random(tbsla_matrix* m, int n_row, int n_col, double nnz_ratio,
                             unsigned int seed_mult, int pr, int pc, int NR, int NC) try {
  if (!m || n_row < 0 || n_col <= 0 || nnz_ratio <= 0 || NR < 1 || NC < 1 || pr < 0 || pc < 0 ||
      pr >= NR || pc >= NC)
    return TBSLA_ERR_INVALID_ARG;
  return fill_random(m, n_row, n_col, nnz_ratio, seed_mult, pr, pc, NR, NC);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_uniform_rows(tbsla_matrix* m, int n, int k, unsigned long long seed) try {
  if (!m) return TBSLA_ERR_INVALID_ARG;
  return fill_uniform_rows(m, n, k, seed);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_powerlaw(tbsla_matrix* m, int n, double mean_len, double zipf_s,
                               int max_len, double local_frac, int band,
                               unsigned long long seed) try {
  if (!m || mean_len <= 0 || zipf_s <= 0 || local_frac < 0 || local_frac > 1)
    return TBSLA_ERR_INVALID_ARG;
  return fill_powerlaw(m, n, mean_len, zipf_s, max_len, local_frac, band, seed);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_dense_uniform(tbsla_matrix* m, int n_row, int n_col,
                                    unsigned long long seed) try {
  if (!m) return TBSLA_ERR_INVALID_ARG;
  return fill_dense_uniform(m, n_row, n_col, seed);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_pa_graph(tbsla_matrix* m, int n, double mean_deg, double zipf_s,
                               int max_deg, double dangling_frac, unsigned long long seed) try {
  if (!m || mean_deg <= 0 || zipf_s <= 0 || dangling_frac < 0 || dangling_frac >= 1)
    return TBSLA_ERR_INVALID_ARG;
  return fill_pa_graph(m, n, mean_deg, zipf_s, max_deg, dangling_frac, seed);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_fill_diffusion7(tbsla_matrix* m, int n, double sigma, double corr_len,
                                 unsigned long long seed) try {
  if (!m || sigma < 0) return TBSLA_ERR_INVALID_ARG;
  return fill_diffusion7(m, n, sigma, corr_len, seed);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_fill_uniform(double* out, long n, double lo, double hi, unsigned long long seed) try {
  if ((!out && n > 0) || n < 0) return TBSLA_ERR_INVALID_ARG;
  fill_uniform(out, n, lo, hi, seed);
  return TBSLA_OK;
} TBSLA_API_CATCH

static int convert(tbsla_matrix** out, const tbsla_matrix* coo, int format, bool device) {
  if (!out || !coo || coo->format != TBSLA_COO || !valid_format(format) || format == TBSLA_COO)
    return TBSLA_ERR_INVALID_ARG;
  std::unique_ptr<tbsla_matrix> m(new (std::nothrow) tbsla_matrix());  // freed if the conversion throws
  if (!m) return TBSLA_ERR_ALLOC;
  m->format = format;
  int st = convert_from_coo(m.get(), coo, format, device);
  if (st) return st;
  *out = m.release();
  return TBSLA_OK;
}

int tbsla_matrix_convert(tbsla_matrix** out, const tbsla_matrix* coo, int format) try {
  return convert(out, coo, format, false);
} TBSLA_API_CATCH

int tbsla_matrix_convert_device(tbsla_matrix** out, const tbsla_matrix* coo, int format) try {
  return convert(out, coo, format, true);
} TBSLA_API_CATCH

int tbsla_matrix_write(const tbsla_matrix* m, const char* path, int append) try {
  if (!m || !path) return TBSLA_ERR_INVALID_ARG;
  return write_file(m, path, append != 0);
} TBSLA_API_CATCH

int tbsla_matrix_read(tbsla_matrix* m, const char* path, long offset) try {
  if (!m || !path || offset < 0) return TBSLA_ERR_INVALID_ARG;
  return read_file(m, path, offset);
} TBSLA_API_CATCH_EMPTY(m)

int tbsla_matrix_set_precision(tbsla_matrix* m, int precision) try {
  if (!m || precision < TBSLA_F64 || precision > TBSLA_BF16) return TBSLA_ERR_INVALID_ARG;
  if (m->precision != precision) {
    m->invalidate();
    m->precision = precision;
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_upload(tbsla_matrix* m) try {
  if (!m) return TBSLA_ERR_INVALID_ARG;
  return dev_upload(m);
} TBSLA_API_CATCH

int tbsla_matrix_device_bytes(const tbsla_matrix* m, size_t* bytes) try {
  if (!m || !bytes) return TBSLA_ERR_INVALID_ARG;
  return dev_bytes(m, bytes);
} TBSLA_API_CATCH

int tbsla_matrix_kernel_launches(const tbsla_matrix* m, int* launches) try {
  if (!m || !launches) return TBSLA_ERR_INVALID_ARG;
  return dev_launches(m, launches);
} TBSLA_API_CATCH

int tbsla_matrix_set_csr_tile(tbsla_matrix* m, int nnz_per_block) try {
  if (!m || nnz_per_block < 256 || nnz_per_block > 4096 || nnz_per_block % 256 != 0)
    return TBSLA_ERR_INVALID_ARG;
  int items = nnz_per_block <= 1024 ? 4 : nnz_per_block <= 2048 ? 8 : 16;
  if (m->csr_tile != 256 * items) {
    m->invalidate();
    m->csr_tile = 256 * items;
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_set_pagerank_gather(tbsla_matrix* m, int gather) try {
  if (!m || (gather != 8 && gather != 16)) return TBSLA_ERR_INVALID_ARG;
  m->pr_gather = gather;  // a launch parameter: the device copy stays
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_set_pagerank_stream(tbsla_matrix* m, int stream) try {
  if (!m || (stream != 0 && stream != 1)) return TBSLA_ERR_INVALID_ARG;
  m->pr_stream = stream;  // a launch choice: the device copy stays
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_set_pagerank_fused(tbsla_matrix* m, int fused) try {
  if (!m || (fused != 0 && fused != 1)) return TBSLA_ERR_INVALID_ARG;
  m->pr_fused = fused;  // a launch choice: the device copy stays
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_matrix_set_sell_params(tbsla_matrix* m, int short_thr, int long_thr, int sigma, int col_block) try {
  if (!m || short_thr < 0 || short_thr > 255 || long_thr < 0 || sigma < 32 || sigma > (1 << 23) ||
      col_block < 0)
    return TBSLA_ERR_INVALID_ARG;
  if (m->sell_short != short_thr || m->sell_long != long_thr || m->sell_sigma != sigma ||
      m->sell_colblock != col_block) {
    m->invalidate();
    m->sell_short = short_thr;
    m->sell_long = long_thr;
    m->sell_sigma = sigma;
    m->sell_colblock = col_block;
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_dense_multiply(const tbsla_matrix* m, const double* B, double* C, int cols_B) try {
  if (!m || cols_B < 0 || (cols_B > 0 && (!B || !C))) return TBSLA_ERR_INVALID_ARG;
  if (cols_B == 0) return TBSLA_OK;
  return dev_dense_multiply(m, B, C, cols_B);
} TBSLA_API_CATCH

int tbsla_get_row_max_abs(const tbsla_matrix* m, double* max_abs) try {
  if (!m || !max_abs) return TBSLA_ERR_INVALID_ARG;
  return dev_row_max_abs(m, max_abs);
} TBSLA_API_CATCH

int tbsla_get_row_sums(const tbsla_matrix* m, double* s) try {
  if (!m || !s) return TBSLA_ERR_INVALID_ARG;
  return dev_row_sums(m, s);
} TBSLA_API_CATCH

int tbsla_normalize_rows(tbsla_matrix* m, const double* s) try {
  if (!m || !s) return TBSLA_ERR_INVALID_ARG;
  return dev_normalize_rows(m, s);
} TBSLA_API_CATCH

int tbsla_apply_exponential(tbsla_matrix* m, const double* max_abs, int base) try {
  if (!m) return TBSLA_ERR_INVALID_ARG;
  return dev_apply_exponential(m, max_abs, base);
} TBSLA_API_CATCH

int tbsla_matrix_autotune(tbsla_matrix* m, int reps, tbsla_tuning* best, tbsla_tuning* trials, int max_trials,
                          int* ntrials) try {
  if (!m || max_trials < 0 || (max_trials > 0 && !trials)) return TBSLA_ERR_INVALID_ARG;
  return dev_autotune(m, reps, best, trials, max_trials, ntrials);
} TBSLA_API_CATCH

int tbsla_matrix_set_csr_algorithm(tbsla_matrix* m, int algorithm, int items) try {
  if (!m || algorithm < TBSLA_CSR_AUTO || algorithm > TBSLA_CSR_SELL ||
      (algorithm != TBSLA_CSR_ROWBLOCK && items != 0 && items != 4 && items != 8 && items != 16))
    return TBSLA_ERR_INVALID_ARG;
  if (algorithm == TBSLA_CSR_MERGE && items == 0) items = 8;
  if (algorithm == TBSLA_CSR_SELL) m->sell_unroll = items;  // a launch parameter only; 0 = automatic
  if (m->csr_algo != algorithm || (algorithm == TBSLA_CSR_MERGE && m->merge_items != items)) {
    m->invalidate();
    m->csr_algo = algorithm;
    if (algorithm == TBSLA_CSR_MERGE) m->merge_items = items;
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_Ax(const tbsla_matrix* m, double* r, const double* v, int vect_incr) try {
  if (!m || !r || !v) return TBSLA_ERR_INVALID_ARG;
  return dev_ax(m, r, v, vect_incr, false, true, nullptr);
} TBSLA_API_CATCH

int tbsla_spmv(const tbsla_matrix* m, double* r, const double* v, int vect_incr) try {
  if (!m || !r || !v) return TBSLA_ERR_INVALID_ARG;
  return dev_ax(m, r, v, vect_incr, true, true, nullptr);
} TBSLA_API_CATCH

int tbsla_Ax_device(const tbsla_matrix* m, double* r, const double* v, int vect_incr,
                    void* stream) try {
  if (!m || !r || !v) return TBSLA_ERR_INVALID_ARG;
  return dev_ax(m, r, v, vect_incr, false, false, stream);
} TBSLA_API_CATCH

int tbsla_spmv_device(const tbsla_matrix* m, double* r, const double* v, int vect_incr,
                      void* stream) try {
  if (!m || !r || !v) return TBSLA_ERR_INVALID_ARG;
  return dev_ax(m, r, v, vect_incr, true, false, stream);
} TBSLA_API_CATCH

int tbsla_csr_Ax_device_noalloc(int n_row, long nnz, int f_col, const int* rowptr, const int* colidx,
                                const double* values, const double* v, double* r, void* stream) try {
  if (n_row < 0 || nnz < 0 || f_col < 0 ||
      (nnz > 0 && (!rowptr || !colidx || !values || !v || !r)))
    return TBSLA_ERR_INVALID_ARG;
  if ((long)n_row + nnz > dev_noalloc_max_items()) return TBSLA_ERR_INVALID_ARG;
  if (nnz == 0) return TBSLA_OK;  // MatrixCSR::Ax leaves r untouched
  return dev_csr_ax_noalloc(n_row, nnz, f_col, rowptr, colidx, values, v, r, stream);
} TBSLA_API_CATCH

int tbsla_a_axpx_(const tbsla_matrix* m, double* r, const double* v, int vect_incr) try {
  if (!m || !r || !v) return TBSLA_ERR_INVALID_ARG;
  return dev_a_axpx(m, r, v, vect_incr);
} TBSLA_API_CATCH

int tbsla_AAxpAx(const tbsla_matrix* m, double* r, const double* v, double* buffer,
                 int vect_incr) try {
  if (!m || !r || !v || !buffer) return TBSLA_ERR_INVALID_ARG;
  return dev_aaxpax(m, r, v, buffer, vect_incr, false);
} TBSLA_API_CATCH

int tbsla_AAxpAxpx(const tbsla_matrix* m, double* r, const double* v, double* buffer,
                   int vect_incr) try {
  if (!m || !r || !v || !buffer) return TBSLA_ERR_INVALID_ARG;
  return dev_aaxpax(m, r, v, buffer, vect_incr, true);
} TBSLA_API_CATCH

int tbsla_get_col_sums(tbsla_matrix* m, double* s) try {
  if (!m || !s) return TBSLA_ERR_INVALID_ARG;
  return dev_col_sums(m, s, false);
} TBSLA_API_CATCH

int tbsla_normalize_cols(tbsla_matrix* m, const double* s) try {
  if (!m || !s) return TBSLA_ERR_INVALID_ARG;
  return dev_normalize_cols(m, s);
} TBSLA_API_CATCH

int tbsla_make_stochastic(tbsla_matrix* m, double* s) try {
  if (!m || !s) return TBSLA_ERR_INVALID_ARG;
  return dev_make_stochastic(m, s);
} TBSLA_API_CATCH

int tbsla_page_rank(tbsla_matrix* m, double beta, double epsilon, int max_iterations,
                    double* result, int* iterations, double* error) try {
  if (!m || !result || beta < 0 || beta > 1) return TBSLA_ERR_INVALID_ARG;
  return dev_page_rank(m, beta, epsilon, max_iterations, result, iterations, error);
} TBSLA_API_CATCH

int tbsla_page_rank_batched(tbsla_matrix* m, int nvec, const double* teleport, double beta,
                            double epsilon, int max_iterations, double* result,
                            int* iterations) try {
  if (!m || !teleport || !result || beta < 0 || beta > 1) return TBSLA_ERR_INVALID_ARG;
  return dev_page_rank_batched(m, nvec, teleport, beta, epsilon, max_iterations, result,
                               iterations);
} TBSLA_API_CATCH

int tbsla_cg(tbsla_matrix* m, const double* b, double* x, int max_iterations, double rel_tol,
             int precond, int refresh, int* iterations, double* rel_residual) try {
  if (!m || !b || !x || rel_tol < 0 || precond < 0 || precond > 1 || refresh < 0)
    return TBSLA_ERR_INVALID_ARG;
  return dev_cg(m, b, x, max_iterations, rel_tol, precond, refresh, iterations, rel_residual);
} TBSLA_API_CATCH

}  // extern "C"
