/*
 * ORACLE — test infrastructure only.
 *
 * Plain-C restatement of the reference TBSLA CPU algorithms on the SpMV /
 * PageRank / CG path, used by the tests, the smoke check and the CPU
 * baseline leg of bench.py as the checker.  Nothing in the product library
 * links or calls this file.
 *
 * Floating-point contract: the file is compiled with -ffp-contract=off, so
 * every product is rounded before it is added, exactly as the reference's
 * loops are evaluated by g++ -O3 on x86-64 (no FMA contraction there).  The
 * sequential summation order of each restated loop is the reference's order.
 *
 * Reference paths below are relative to the TBSLA source tree.
 */
#include "tbsla_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* MatrixCSR::Ax, src/cpp/matrix/MatrixCSR.cpp:209-233 (scalar build).
 * Overwrites r[0..ln_row); returns without touching r when nnz == 0.      */
void orc_csr_ax(int ln_row, int f_col, long nnz, const double* values,
                const int* rowptr, const int* colidx, const double* v, double* r) {
  if (nnz == 0) return;
  for (int i = 0; i < ln_row; i++) {
    double acc = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) acc += values[j] * v[colidx[j] - f_col];
    r[i] = acc;
  }
}

/* Same loop with the reference's `omp parallel for schedule(static)` row
 * split (MatrixCSR.cpp:212-213); used as the timed CPU baseline.          */
void orc_csr_ax_omp(int ln_row, int f_col, long nnz, const double* values,
                    const int* rowptr, const int* colidx, const double* v, double* r) {
  if (nnz == 0) return;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ln_row; i++) {
    double acc = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) acc += values[j] * v[colidx[j] - f_col];
    r[i] = acc;
  }
}

/* The FP32-valued storage form of the same loop: values widened to FP64. */
void orc_csr_ax_f32_omp(int ln_row, int f_col, long nnz, const float* values,
                        const int* rowptr, const int* colidx, const double* v, double* r) {
  if (nnz == 0) return;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ln_row; i++) {
    double acc = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
      acc += (double)values[j] * v[colidx[j] - f_col];
    r[i] = acc;
  }
}

/* sum_j |a_ij * v_j| per row: the scale the SpMV parity tolerance is relative to. */
void orc_csr_absrow(int ln_row, int f_col, const double* values, const int* rowptr,
                    const int* colidx, const double* v, double* out) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ln_row; i++) {
    double acc = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) acc += fabs(values[j] * v[colidx[j] - f_col]);
    out[i] = acc;
  }
}

/* MatrixELL::Ax, src/cpp/matrix/MatrixELL.cpp:181-205.  Row-major padded
 * storage values[i*max_col + j]; every slot (pads included) is multiplied
 * and added; with f_col != 0 a negative shifted index is clamped to 0.    */
void orc_ell_ax(int ln_row, int max_col, int f_col, long nnz, const double* values,
                const int* columns, const double* v, double* r) {
  if (nnz == 0 || max_col == 0 || values == NULL || columns == NULL) return;
  for (int i = 0; i < ln_row; i++) {
    double acc = 0;
    for (int j = 0; j < max_col; j++) {
      long k = (long)i * max_col + j;
      int idx = columns[k] - f_col;
      if (f_col != 0 && idx < 0) idx = 0;
      acc += values[k] * v[idx];
    }
    r[i] = acc;
  }
}

/* MatrixCOO::Ax, src/cpp/matrix/MatrixCOO.cpp:135-142 with the OpenMP array
 * reduction of src/cpp/include/tbsla/cpp/reduction.hpp:6-34, evaluated with
 * one thread: a zeroed private array accumulates the triplets in storage
 * order, then is added into r.  Accumulates into r.                        */
void orc_coo_ax(int n_row, long nnz, const double* values, const int* row,
                const int* col, const double* v, double* r, int vect_incr) {
  double* priv = (double*)calloc((size_t)(n_row > 0 ? n_row : 1), sizeof(double));
  for (long k = 0; k < nnz; k++) priv[row[k] + vect_incr] += values[k] * v[col[k]];
  for (int i = 0; i < n_row; i++) r[i] += priv[i];
  free(priv);
}

/* MatrixSCOO::Ax, src/cpp/matrix/MatrixSCOO.cpp:154-164: global indices
 * shifted by the block origin (f_row, f_col); same one-thread reduction.  */
void orc_scoo_ax(int ln_row, int f_row, int f_col, long nnz, const double* values,
                 const int* row, const int* col, const double* v, double* r, int vect_incr) {
  if (nnz == 0) return;
  double* priv = (double*)calloc((size_t)(ln_row > 0 ? ln_row : 1), sizeof(double));
  for (long k = 0; k < nnz; k++)
    priv[row[k] + vect_incr - f_row] += values[k] * v[col[k] - f_col];
  for (int i = 0; i < ln_row; i++) r[i] += priv[i];
  free(priv);
}

/* MatrixDENSE::Ax, src/cpp/matrix/MatrixDENSE.cpp:77-86: r_i accumulates
 * each product directly, starting from the caller's r_i.                  */
void orc_dense_ax(int ln_row, int ln_col, long nnz, const double* values,
                  const double* v, double* r) {
  if (nnz == 0 || values == NULL) return;
  for (int i = 0; i < ln_row; i++)
    for (int j = 0; j < ln_col; j++) r[i] += values[(long)i * ln_col + j] * v[j];
}

void orc_dense_ax_omp(int ln_row, int ln_col, long nnz, const double* values,
                      const double* v, double* r) {
  if (nnz == 0 || values == NULL) return;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ln_row; i++)
    for (int j = 0; j < ln_col; j++) r[i] += values[(long)i * ln_col + j] * v[j];
}

/* ---- conversions ------------------------------------------------------ */

typedef struct {
  const int* row;
  const int* col;
} key_ctx;
static key_ctx g_ctx; /* qsort has no user pointer in C99; tests are single-threaded */

static int cmp_row_col_idx(const void* a, const void* b) {
  long i = *(const long*)a, j = *(const long*)b;
  if (g_ctx.row[i] != g_ctx.row[j]) return g_ctx.row[i] < g_ctx.row[j] ? -1 : 1;
  if (g_ctx.col[i] != g_ctx.col[j]) return g_ctx.col[i] < g_ctx.col[j] ? -1 : 1;
  return i < j ? -1 : (i > j);
}

static long* sorted_order(long nnz, const int* row, const int* col) {
  long* p = (long*)malloc(sizeof(long) * (size_t)(nnz > 0 ? nnz : 1));
  for (long k = 0; k < nnz; k++) p[k] = k;
  g_ctx.row = row;
  g_ctx.col = col;
  qsort(p, (size_t)nnz, sizeof(long), cmp_row_col_idx);
  return p;
}

/* MatrixCSR(const MatrixCOO&), src/cpp/matrix/MatrixCSR.cpp:49-96 with
 * compare_row, src/cpp/utils/csr.cpp:3-8: entries ordered by (row, col)
 * (ties keep storage order), rowptr[r+1] = #entries with row <= r.        */
int orc_coo_to_csr(int n_row, long nnz, const int* row, const int* col, const double* val,
                   int* rowptr, int* colidx, double* values) {
  long* p = sorted_order(nnz, row, col);
  for (int i = 0; i <= n_row; i++) rowptr[i] = 0;
  for (long k = 0; k < nnz; k++) {
    colidx[k] = col[p[k]];
    values[k] = val[p[k]];
    rowptr[row[p[k]] + 1]++;
  }
  for (int i = 0; i < n_row; i++) rowptr[i + 1] += rowptr[i];
  free(p);
  return 0;
}

/* max entries per row: MatrixELL.cpp:53-59 */
int orc_ell_max_col(int n_row, long nnz, const int* row) {
  if (nnz == 0) return 0;
  int* cnt = (int*)calloc((size_t)n_row, sizeof(int));
  int m = 0;
  for (long k = 0; k < nnz; k++) cnt[row[k]]++;
  for (int i = 0; i < n_row; i++) m = cnt[i] > m ? cnt[i] : m;
  free(cnt);
  return m;
}

/* MatrixELL(const MatrixCOO&), src/cpp/matrix/MatrixELL.cpp:25-79: sorted
 * entries packed left in each row of a row-major n_row x max_col array,
 * pads are column 0 / value 0.                                            */
int orc_coo_to_ell(int n_row, long nnz, const int* row, const int* col, const double* val,
                   int max_col, int* columns, double* values) {
  long total = (long)n_row * max_col;
  for (long k = 0; k < total; k++) {
    columns[k] = 0;
    values[k] = 0;
  }
  if (nnz == 0) return 0;
  long* p = sorted_order(nnz, row, col);
  int* fill = (int*)calloc((size_t)n_row, sizeof(int));
  for (long k = 0; k < nnz; k++) {
    int r = row[p[k]];
    long slot = (long)r * max_col + fill[r]++;
    columns[slot] = col[p[k]];
    values[slot] = val[p[k]];
  }
  free(fill);
  free(p);
  return 0;
}

/* MatrixDENSE(const MatrixCOO&), src/cpp/matrix/MatrixDENSE.cpp:15-37:
 * duplicates are summed in storage order.                                 */
void orc_coo_to_dense(int ln_row, int ln_col, long nnz, const int* row, const int* col,
                      const double* val, double* dense) {
  memset(dense, 0, sizeof(double) * (size_t)ln_row * (size_t)ln_col);
  for (long k = 0; k < nnz; k++) dense[(long)row[k] * ln_col + col[k]] += val[k];
}

/* ---- column-stochastic preparation ------------------------------------ */

/* MatrixCSR::get_col_sums, src/cpp/matrix/MatrixCSR.cpp:1192-1213, in its
 * intended sequential form (the reference's OpenMP loop races on s[]).
 * Accumulates into the caller-zeroed s.                                   */
void orc_csr_col_sums(int ln_row, int f_col, long nnz, const double* values,
                      const int* rowptr, const int* colidx, double* s) {
  if (nnz == 0) return;
  for (int i = 0; i < ln_row; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) s[colidx[j] - f_col] += values[j];
}

/* MatrixCSR::normalize_cols, src/cpp/matrix/MatrixCSR.cpp:1215-1232:
 * a_ij /= s_j where s_j > 0 (zero columns, the dangling nodes, stay 0).  */
void orc_csr_normalize_cols(int ln_row, int f_col, long nnz, double* values,
                            const int* rowptr, const int* colidx, const double* s) {
  if (nnz == 0) return;
  for (int i = 0; i < ln_row; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
      double sv = s[colidx[j] - f_col];
      if (sv > 0) values[j] /= sv;
    }
}

/* ---- SpMM and the sparse-softmax helpers (CSR) ---------------------------- */

/* C = A B, MatrixCSR::dense_multiply (src/cpp/matrix/MatrixCSR.cpp:1269-1281):
 * C zero-filled over n_row x cols_B, then C[i][k] += a_ij * B[colidx_j][k]
 * in entry order (the column index is used as stored, without f_col). */
void orc_csr_dense_multiply(int n_row, const double* values, const int* rowptr, const int* colidx,
                            const double* B, double* Cm, int cols_B) {
  for (long t = 0; t < (long)n_row * cols_B; t++) Cm[t] = 0.0;
  for (int i = 0; i < n_row; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
      const int col = colidx[j];
      const double v = values[j];
      for (int k = 0; k < cols_B; k++) Cm[(long)i * cols_B + k] += v * B[(long)col * cols_B + k];
    }
}

/* max_abs[i] = max over the row's nonzero values of |a_ij| (0 for an empty
 * row), MatrixCSR::get_row_max_abs (MatrixCSR.cpp:1283-1312). */
void orc_csr_row_max_abs(int ln_row, const double* values, const int* rowptr, double* max_abs) {
  for (int i = 0; i < ln_row; i++) {
    double m = 0.0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
      const double z = values[j];
      if (z != 0 && fabs(z) > m) m = fabs(z);
    }
    max_abs[i] = m;
  }
}

/* s[i] = sum of row i's values in entry order, MatrixCSR::get_row_sums
 * (MatrixCSR.cpp:1147-1164). */
void orc_csr_row_sums(int ln_row, const double* values, const int* rowptr, double* s) {
  for (int i = 0; i < ln_row; i++) {
    double sum = 0.0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) sum += values[j];
    s[i] = sum;
  }
}

/* a_ij /= s[i], or 0 where s[i] == 0, MatrixCSR::normalize_rows
 * (MatrixCSR.cpp:1177-1190). */
void orc_csr_normalize_rows(int ln_row, double* values, const int* rowptr, const double* s) {
  for (int i = 0; i < ln_row; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) values[j] = s[i] != 0 ? values[j] / s[i] : 0.0;
}

/* MatrixCSR::apply_exponential (MatrixCSR.cpp:1315-1334): every nonzero
 * a_ij becomes exp(a_ij - max_abs[i]) (base <= 0) or base^(a_ij - max_abs[i]),
 * without the shift when max_abs is NULL; zeros stay. */
void orc_csr_apply_exponential(int ln_row, double* values, const int* rowptr, const double* max_abs,
                               int base) {
  for (int i = 0; i < ln_row; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
      const double z = values[j];
      if (z == 0) continue;
      const double a = max_abs ? z - max_abs[i] : z;
      values[j] = base <= 0 ? exp(a) : pow((double)base, a);
    }
}

/* ---- PageRank --------------------------------------------------------- */

/* Power iteration following src/mpi/matrix/Matrix.cpp:540-602 (loop),
 * :106-146 (teleport + L1 error) and :149-171 (final normalisation), with
 * the start vector 1/n of page_rank_opticom (Matrix.cpp:713).  Fixed
 * relative to the reference:
 *   - damping is applied to the vector that is iterated (Matrix.cpp:745-754
 *     applies it to a buffer that is then discarded);
 *   - the mass of dangling nodes is redistributed along the teleport vector
 *     instead of being lost and renormalised away;
 * and each iterate is normalised by its sum before it is used, as
 * pagerank_normalization does (Matrix.cpp:106-146).  With w_j the sum of
 * column j of the values given (1 for a node with out-links when A is
 * column-stochastic, 0 for a dangling node), S = sum(x_k),
 * M = sum_j w_j x_k[j] and s = 1/S:
 *   x_{k+1}[i] = (beta*(A x_k)[i])*s + (1 - (beta*M)*s) * t_i
 * with t_i = 1/n (uniform) or teleport[i] (personalised, summing to 1).
 * For exactly column-stochastic A, 1 - beta*M*s = (1 - beta) + beta*D*s
 * (D = mass on dangling nodes): the usual dangling-node redistribution.
 * For values rounded in storage (FP32, BF16) it also hands back the mass
 * the rounding loses, so every iterate sums to 1 and the L1 change below
 * goes to zero.  The error is sum_i |x_{k+1}[i] - x_k[i]*s|; the loop stops
 * when it drops below epsilon (if stop_early) or after max_iterations.  The
 * result is divided by its sum at the end.  Returns the iterations done.  */
int orc_pagerank(int n, const int* rowptr, const int* colidx, const double* values,
                 const double* teleport, double beta, double epsilon, int max_iterations,
                 int stop_early, double* x, double* last_error) {
  double* y = (double*)calloc((size_t)n, sizeof(double));
  double* cur = (double*)malloc(sizeof(double) * (size_t)n);
  double* w = (double*)calloc((size_t)n, sizeof(double));
  long nnz = rowptr[n];
  for (int i = 0; i < n; i++)
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) w[colidx[j]] += values[j];
  for (int i = 0; i < n; i++) cur[i] = 1.0 / n;
  int it = 0;
  double err = 0;
  while (it < max_iterations) {
    double S = 0, M = 0;
    for (int i = 0; i < n; i++) {
      S += cur[i];
      M += w[i] * cur[i];
    }
    for (int i = 0; i < n; i++) y[i] = 0;
    orc_csr_ax(n, 0, nnz, values, rowptr, colidx, cur, y);
    double s = 1.0 / S;
    double t = 1.0 - beta * M * s;
    double c = t / n;
    err = 0;
    for (int i = 0; i < n; i++) {
      double xn = beta * y[i] * s + (teleport ? t * teleport[i] : c);
      err += fabs(xn - cur[i] * s);
      y[i] = xn;
    }
    double* tmp = cur;
    cur = y;
    y = tmp;
    it++;
    if (stop_early && err < epsilon) break;
  }
  double s = 0;
  for (int i = 0; i < n; i++) s += cur[i];
  for (int i = 0; i < n; i++) x[i] = cur[i] / s;
  if (last_error) *last_error = err;
  free(w);
  free(y);
  free(cur);
  return it;
}

/* ---- CG ----------------------------------------------------------------- */

static double dot(const double* a, const double* b, int n) {
  double s = 0;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Conjugate gradients following src/mpi/matrix/CG.cpp:32-73 and its vector
 * helpers :7-30, restated:
 *   - the SpMV is Ax(r = AP, v = P) (CG.cpp:61 passes the arguments in the
 *     opposite order, so the reference never advances);
 *   - the stop test is relative, ||r|| <= rel_tol * ||b|| (the reference
 *     uses ||r|| < 1e-10 absolute);
 *   - the reference floors p.Ap and r_old.r_old at 1e-10 (CG.cpp:63,69),
 *     which stalls the last digits of a relative 1e-8 solve; here only a
 *     zero denominator is guarded;
 *   - optional Jacobi preconditioning z = diag_inv .* r (the reference has
 *     no preconditioner).
 * x holds the start vector on entry.  Returns the number of SpMVs with P;
 * rel_residual receives ||b - A x|| / ||b|| recomputed from scratch.     */
int orc_cg(int n, const int* rowptr, const int* colidx, const double* values,
           const double* diag_inv, const double* b, double* x, int max_iterations,
           double rel_tol, double* rel_residual) {
  long nnz = rowptr[n];
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* ap = (double*)calloc((size_t)n, sizeof(double));
  orc_csr_ax(n, 0, nnz, values, rowptr, colidx, x, ap);
  for (int i = 0; i < n; i++) r[i] = b[i] - ap[i];
  for (int i = 0; i < n; i++) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
  memcpy(p, z, sizeof(double) * (size_t)n);
  double rz = dot(r, z, n);
  double bnorm = sqrt(dot(b, b, n));
  int it = 0;
  if (sqrt(dot(r, r, n)) > rel_tol * bnorm) {
    while (it < max_iterations) {
      orc_csr_ax(n, 0, nnz, values, rowptr, colidx, p, ap);
      double pap = dot(p, ap, n);
      double alpha = pap != 0 ? rz / pap : 0;
      for (int i = 0; i < n; i++) x[i] += alpha * p[i];
      for (int i = 0; i < n; i++) r[i] -= alpha * ap[i];
      it++;
      if (sqrt(dot(r, r, n)) <= rel_tol * bnorm) break;
      for (int i = 0; i < n; i++) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
      double rz_new = dot(r, z, n);
      double beta = rz != 0 ? rz_new / rz : 0;
      for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
      rz = rz_new;
    }
  }
  orc_csr_ax(n, 0, nnz, values, rowptr, colidx, x, ap);
  double rr = 0;
  for (int i = 0; i < n; i++) {
    double d = b[i] - ap[i];
    rr += d * d;
  }
  if (rel_residual) *rel_residual = bnorm > 0 ? sqrt(rr) / bnorm : sqrt(rr);
  free(r);
  free(z);
  free(p);
  free(ap);
  return it;
}

/* ---- workload generator: the power-law SpMV matrix ----------------------
 * Not a reference function: a restatement of this library's own generator
 * (fill_powerlaw / fill_uniform of its host code), so that the CPU baseline
 * can build the large-SpMV matrix without loading the library it is timed
 * against.  Rows draw their length from a truncated Zipf law rescaled to the
 * requested mean (stochastic rounding), their columns (a share `local_frac`
 * within +-band of the diagonal, the rest uniform) from a counter-based
 * SplitMix64 hash of (seed, row, draw), so every row depends only on its
 * index.  Compiled with -ffp-contract=off, as the library's host code is, the
 * arrays are identical to the library's on every host. */
#include <stdint.h>

static uint64_t gen_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t gen_hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return gen_mix64(gen_mix64(seed ^ gen_mix64(a + 0x632BE59BD9B4E019ull)) + b);
}
static double gen_u01(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }
static double gen_um11(uint64_t h) { return 2.0 * gen_u01(h) - 1.0; }

typedef struct {
  double* cdf;
  int kmax;
  double mean;
} gen_zipf;

static void zipf_init(gen_zipf* z, double s, int kmax) {
  z->cdf = (double*)malloc(sizeof(double) * (size_t)kmax);
  z->kmax = kmax;
  double tot = 0, m = 0;
  for (int k = 1; k <= kmax; k++) {
    double p = pow((double)k, -s);
    tot += p;
    m += k * p;
    z->cdf[k - 1] = tot;
  }
  for (int k = 0; k < kmax; k++) z->cdf[k] /= tot;
  z->mean = m / tot;
}

/* first index whose cdf exceeds u, plus one */
static int zipf_draw(const gen_zipf* z, double u) {
  int lo = 0, hi = z->kmax;
  while (lo < hi) {
    int mid = lo + (hi - lo) / 2;
    if (z->cdf[mid] > u) hi = mid;
    else lo = mid + 1;
  }
  return lo + 1;
}

static long zipf_rescale(int k, double scale, double u, long lo, long kmax) {
  double y = k * scale;
  long r = (long)floor(y);
  if (u < y - (double)r) r++;
  if (r < lo) r = lo;
  if (r > kmax) r = kmax;
  return r;
}

static double zipf_mean_at(const gen_zipf* z, double sc, long lo, long kmax) {
  double m = 0, prev = 0;
  for (int k = 1; k <= z->kmax; k++) {
    double v = (double)k * sc;
    if (v < (double)lo) v = (double)lo;
    if (v > (double)kmax) v = (double)kmax;
    m += (z->cdf[k - 1] - prev) * v;
    prev = z->cdf[k - 1];
  }
  return m;
}

static double zipf_scale_for(const gen_zipf* z, double target, long lo, long kmax) {
  double a = 0, b = 2.0 * target / z->mean + 1.0;
  while (zipf_mean_at(z, b, lo, kmax) < target && b < 1e9) b *= 2;
  for (int it = 0; it < 200; it++) {
    double c = 0.5 * (a + b);
    if (zipf_mean_at(z, c, lo, kmax) < target) a = c;
    else b = c;
  }
  return b;
}

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

long orc_gen_powerlaw_rows(int n, double mean_len, double zipf_s, int max_len, double local_frac, int band,
                           unsigned long long seed, int* rowptr) {
  if (n <= 0 || max_len <= 0 || max_len > n) return -1;
  gen_zipf z;
  zipf_init(&z, zipf_s, max_len);
  const double scale = zipf_scale_for(&z, mean_len, 1, max_len);
  rowptr[0] = 0;
  long acc = 0;
  for (long i = 0; i < n; i++) {
    int k = zipf_draw(&z, gen_u01(gen_hash3(seed, 1, (uint64_t)i)));
    long len = zipf_rescale(k, scale, gen_u01(gen_hash3(seed, 12, (uint64_t)i)), 1, max_len);
    if (local_frac >= 1.0) { /* all columns near the diagonal: at most the band's columns */
      long lo = i - band < 0 ? 0 : i - band, hi = i + band > (long)n - 1 ? (long)n - 1 : i + band;
      if (len > hi - lo + 1) len = hi - lo + 1;
    }
    acc += len;
    if (acc > 0x7fffffffL) {
      free(z.cdf);
      return -1;
    }
    rowptr[i + 1] = (int)acc;
  }
  free(z.cdf);
  return acc;
}

void orc_gen_powerlaw_entries(int n, double local_frac, int band, unsigned long long seed,
                              const int* rowptr, int* colidx, double* values) {
#pragma omp parallel
  {
    int cap = 16;
    int* cols = (int*)malloc(sizeof(int) * (size_t)cap);
#pragma omp for schedule(dynamic, 4096)
    for (long i = 0; i < n; i++) {
      int L = rowptr[i + 1] - rowptr[i];
      long lo = i - band < 0 ? 0 : i - band;
      long hi = i + band > (long)n - 1 ? (long)n - 1 : i + band;
      int want = L < n ? L : n;
      if (want > cap) {
        cap = want;
        cols = (int*)realloc(cols, sizeof(int) * (size_t)cap);
      }
      int size = 0;
      uint64_t t = 0;
      while (size < want) {
        int need = want - size;
        for (int d = 0; d < need; d++) {
          uint64_t h = gen_hash3(seed, 2 + (uint64_t)i * 2, t++);
          int local = gen_u01(h) < local_frac;
          uint64_t h2 = gen_hash3(seed, 3 + (uint64_t)i * 2, t);
          long c = local ? lo + (long)(h2 % (uint64_t)(hi - lo + 1)) : (long)(h2 % (uint64_t)n);
          cols[size++] = (int)c;
        }
        qsort(cols, (size_t)size, sizeof(int), cmp_int);
        int u = 0;
        for (int q = 0; q < size; q++)
          if (q == 0 || cols[q] != cols[u - 1]) cols[u++] = cols[q];
        size = u;
      }
      long p0 = rowptr[i];
      for (int j = 0; j < want; j++) {
        colidx[p0 + j] = cols[j];
        values[p0 + j] = gen_um11(gen_hash3(seed ^ 0xC3C3C3C3ull, 4, (uint64_t)(p0 + j)));
      }
    }
    free(cols);
  }
}

void orc_gen_uniform(double* out, long n, double lo, double hi, unsigned long long seed) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) out[i] = lo + (hi - lo) * gen_u01(gen_hash3(seed, 0x5eed, (uint64_t)i));
}
