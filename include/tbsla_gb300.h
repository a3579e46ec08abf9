/*
 * tbsla_gb300 — C ABI of the GB300-native TBSLA SpMV / PageRank / CG path.
 *
 * This is the drop-in boundary.  It replaces the reference's per-format C
 * interface C_CPP_Matrix<FMT>_* (src/cpp/interface/c/include/tbsla/cpp/
 * MatrixCSR.h:13-21, which no longer compiles against the reference's own
 * headers) with one working interface over an opaque matrix handle, and it
 * is what the C++ classes tbsla::cpp::Matrix* of this library are built on.
 *
 * Conventions
 *  - Every entry point returns an int status: TBSLA_OK (0) or a negative
 *    TBSLA_ERR_* code; tbsla_status_string() names it.  Nothing throws across
 *    the ABI: a host allocation that fails returns TBSLA_ERR_ALLOC, and a
 *    matrix whose arrays were being replaced (setters, push_back,
 *    generators, read) is then left empty, as after tbsla_matrix_create.
 *    Bad input (out-of-range index, non-monotone row pointer, truncated
 *    file, size mismatch) is rejected on the host before any kernel runs.
 *  - A handle keeps the reference's host layout (the arrays a reference
 *    Matrix object owns) plus a device copy built on first use (or by
 *    tbsla_matrix_upload); any host-side mutation drops the device copy.
 *  - Entry points with host pointers (tbsla_Ax, tbsla_spmv, ...) copy the
 *    input vector to the GPU, run the kernels and copy the result back
 *    before returning.  *_device entry points take device pointers and a
 *    cudaStream_t (passed as void*, NULL = the handle's own stream) and do
 *    not synchronise.
 *  - Handles are not thread-safe; one stream per handle, as the reference's
 *    objects are used from one thread.
 *  - No CPU fallback: with no usable GPU every compute entry point returns
 *    TBSLA_ERR_NO_DEVICE.
 */
#ifndef TBSLA_GB300_H
#define TBSLA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define TBSLA_OK 0
#define TBSLA_ERR_INVALID_ARG (-1)   /* bad argument (null handle, wrong format, size) */
#define TBSLA_ERR_BAD_MATRIX (-2)    /* matrix arrays fail validation */
#define TBSLA_ERR_ALLOC (-3)         /* host or device allocation failed */
#define TBSLA_ERR_CUDA (-4)          /* a CUDA call failed */
#define TBSLA_ERR_IO (-5)            /* file missing, short or malformed */
#define TBSLA_ERR_NOT_CONVERGED (-6) /* iteration limit reached (results still written) */
#define TBSLA_ERR_TIMEOUT (-7)       /* a bounded device wait gave up */
#define TBSLA_ERR_UNSUPPORTED (-8)   /* operation not defined for this format */
#define TBSLA_ERR_NO_DEVICE (-9)     /* no CUDA device usable */

/* ---- formats and value precisions ----------------------------------------- */
#define TBSLA_COO 0
#define TBSLA_SCOO 1
#define TBSLA_CSR 2
#define TBSLA_ELL 3
#define TBSLA_DENSE 4

#define TBSLA_F64 0  /* values stored as double on the device (default) */
#define TBSLA_F32 1  /* values stored as float, products and sums in double (DENSE Ax and
                        batched PageRank: double-float, about 2^-48 relative) */
#define TBSLA_BF16 2 /* values stored as bfloat16, products and sums as for TBSLA_F32 */

typedef struct tbsla_matrix tbsla_matrix;

/* Distribution metadata of a block, as in tbsla::cpp::Matrix
 * (src/cpp/include/tbsla/cpp/Matrix.hpp:54-55), plus ELL's max_col
 * (MatrixELL.hpp:43). */
typedef struct tbsla_info {
  int n_row, n_col, ln_row, ln_col, f_row, f_col;
  long nnz;
  int pr, pc, NR, NC;
  int max_col;
} tbsla_info;

const char* tbsla_status_string(int status);
/* Library version string. */
const char* tbsla_version(void);
/* Selects the CUDA device used by handles created afterwards (default 0). */
int tbsla_device_init(int device);
/* Pinned host buffers, for callers that want full-speed host<->device copies. */
int tbsla_host_alloc(void** ptr, size_t bytes);
int tbsla_host_free(void* ptr);

/* ---- handle lifecycle: C_CPP_Matrix<FMT>_create/_destroy
 *      (interface/c/include/tbsla/cpp/MatrixCSR.h:13-14) ------------------- */
int tbsla_matrix_create(tbsla_matrix** m, int format);
int tbsla_matrix_destroy(tbsla_matrix* m);
int tbsla_matrix_format(const tbsla_matrix* m, int* format);
int tbsla_matrix_info(const tbsla_matrix* m, tbsla_info* info);

/* Copies caller arrays into the handle (the caller keeps ownership).  Array
 * lengths follow the reference layouts: COO/SCOO values/row/col[nnz]; CSR
 * values[nnz], rowptr[ln_row+1], colidx[nnz]; ELL values/columns
 * [ln_row*max_col] row-major; DENSE values[ln_row*ln_col] row-major. */
int tbsla_matrix_set_coo(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* row, const int* col);
int tbsla_matrix_set_csr(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* rowptr, const int* colidx);
/* Appends one entry (row, col, value) to a COO / SCOO handle (nnz grows by
 * one; indices as stored, i.e. global for SCOO blocks); replaces
 * MatrixSCOO::push_back (src/cpp/include/tbsla/cpp/MatrixSCOO.hpp:25), which
 * the reference declares but never defines. */
int tbsla_matrix_push_back(tbsla_matrix* m, int row, int col, double value);
int tbsla_matrix_set_ell(tbsla_matrix* m, const tbsla_info* info, const double* values,
                         const int* columns);
int tbsla_matrix_set_dense(tbsla_matrix* m, const tbsla_info* info, const double* values);
/* Borrowed pointers to the handle's host arrays (valid until the next
 * mutation).  idx0/idx1: COO/SCOO row/col, CSR rowptr/colidx, ELL columns/NULL,
 * DENSE NULL/NULL. */
int tbsla_matrix_arrays(const tbsla_matrix* m, const double** values, const int** idx0,
                        const int** idx1);

/* ---- generators: tbsla::cpp::Matrix::fill_* (Matrix.hpp:40-42) -------------- */
int tbsla_matrix_fill_cdiag(tbsla_matrix* m, int n_row, int n_col, int cdiag, int pr, int pc,
                            int NR, int NC);
int tbsla_matrix_fill_cqmat(tbsla_matrix* m, int n_row, int n_col, int c, double q,
                            unsigned int seed_mult, int pr, int pc, int NR, int NC);
int tbsla_matrix_fill_random(tbsla_matrix* m, int n_row, int n_col, double nnz_ratio,
                             unsigned int seed_mult, int pr, int pc, int NR, int NC);

/* Synthetic workload generators (no counterpart in the reference; the
 * reference's generators only emit all-ones values).  All are
 * deterministic functions of their arguments, independent of thread count.
 *  - uniform_rows: square n x n; row i holds column i plus k-1 further
 *    distinct columns uniform in [0,n), sorted; values U[-1,1).
 *  - powerlaw: square n x n; row lengths Zipf(zipf_s) on [1,max_len]
 *    rescaled to mean `mean_len` (rounded stochastically, clipped to
 *    [1,max_len], the scale chosen so that the expected length is exactly
 *    mean_len); each
 *    column is uniform on [0,n) with probability 1-local_frac, else uniform
 *    within +-band of the diagonal; distinct and sorted per row; values
 *    U[-1,1).
 *  - dense_uniform: n_row x n_col DENSE with values U[-1,1).
 *  - pa_graph: PageRank graph, CSR of the transposed adjacency (A[i][j] = 1
 *    for an edge j -> i) of a directed graph on n nodes with out-degrees
 *    Zipf(zipf_s) rescaled to mean `mean_deg`, a fraction `dangling_frac`
 *    of nodes with out-degree 0, targets by preferential attachment
 *    (probability proportional to in-degree + 1).
 *  - diffusion7: SPD 7-point finite-volume diffusion matrix on an n^3 grid
 *    with Dirichlet boundaries and face coefficients exp(g), g a Gaussian
 *    random field with standard deviation sigma and correlation length
 *    corr_len cells. */
int tbsla_matrix_fill_uniform_rows(tbsla_matrix* m, int n, int k, unsigned long long seed);
int tbsla_matrix_fill_powerlaw(tbsla_matrix* m, int n, double mean_len, double zipf_s,
                               int max_len, double local_frac, int band,
                               unsigned long long seed);
int tbsla_matrix_fill_dense_uniform(tbsla_matrix* m, int n_row, int n_col,
                                    unsigned long long seed);
int tbsla_matrix_fill_pa_graph(tbsla_matrix* m, int n, double mean_deg, double zipf_s,
                               int max_deg, double dangling_frac, unsigned long long seed);
int tbsla_matrix_fill_diffusion7(tbsla_matrix* m, int n, double sigma, double corr_len,
                                 unsigned long long seed);
/* Deterministic vector fills: U[lo,hi) per index from (seed, i). */
int tbsla_fill_uniform(double* out, long n, double lo, double hi, unsigned long long seed);

/* ---- conversions: MatrixCSR/ELL/SCOO/DENSE(const MatrixCOO&)
 *      (MatrixCSR.cpp:49-96, MatrixELL.cpp:25-79, MatrixSCOO.cpp:75-101,
 *      MatrixDENSE.cpp:15-37) --------------------------------------------- */
int tbsla_matrix_convert(tbsla_matrix** out, const tbsla_matrix* coo, int format);
/* The same conversion on the GPU: the (row, column) ordering of CSR / ELL by
 * a stable radix sort (MatrixCSR.cpp:49-96 sorts on the host), the DENSE
 * scatter-add (MatrixDENSE.cpp:15-37) by a kernel over that order, which
 * sums duplicate positions in storage order from 0 as the reference does:
 * identical arrays, TBSLA_ERR_NO_DEVICE without a GPU.  SCOO, a plain copy
 * of the arrays (MatrixSCOO.cpp:75-101), stays on the host. */
int tbsla_matrix_convert_device(tbsla_matrix** out, const tbsla_matrix* coo, int format);

/* ---- binary I/O: write/read (e.g. MatrixCSR.cpp:236-295), the reference's
 *      wire format byte for byte --------------------------------------------- */
int tbsla_matrix_write(const tbsla_matrix* m, const char* path, int append);
int tbsla_matrix_read(tbsla_matrix* m, const char* path, long offset);

/* ---- device copy ------------------------------------------------------------- */
/* Value storage precision of the device copy (TBSLA_F64 default).  DENSE
 * with TBSLA_F32 / TBSLA_BF16 values computes Ax in double-float on the FP32
 * pipes when every nonzero |value| is in [2^-40, 2^40] (checked when the
 * device copy is built) and, per call, every nonzero |v| too (otherwise that
 * call computes in FP64); results stay within the FP64 tolerance. */
int tbsla_matrix_set_precision(tbsla_matrix* m, int precision);
/* Builds the device copy now (otherwise built by the first compute call). */
int tbsla_matrix_upload(tbsla_matrix* m);
/* Device bytes held by the handle's matrix copy. */
int tbsla_matrix_device_bytes(const tbsla_matrix* m, size_t* bytes);
/* Kernel launches one Ax / spmv makes on the device copy (builds it if
 * needed): one per sliced-ELL plan (a column block, the last of several
 * split in two by rows), two for the merge path, one otherwise, none for an
 * empty matrix.  No counterpart in the reference (a property of this
 * implementation's kernels). */
int tbsla_matrix_kernel_launches(const tbsla_matrix* m, int* launches);
/* CSR: block budget of the row-block partition (nnz per block, multiple of
 * 256, default 2048); changing it rebuilds the partition. */
int tbsla_matrix_set_csr_tile(tbsla_matrix* m, int nnz_per_block);
/* CSR SpMV kernel: TBSLA_CSR_AUTO (default: row blocks below 2^19 stored
 * entries, where one short launch is latency-bound, else sliced ELL),
 * TBSLA_CSR_SELL (sliced-ELL device layout, slices of 32 lanes over rows of
 * similar length, see tbsla_matrix_set_sell_params; `items` = steps per
 * lane in flight, 4/8/16, 0 = 8), TBSLA_CSR_MERGE (merge-path split,
 * `items` row ends + entries per thread, 4/8/16, 0 = 8) or
 * TBSLA_CSR_ROWBLOCK (row-block adaptive, see
 * tbsla_matrix_set_csr_tile; `items` unused).  Changing the kernel or the
 * merge split rebuilds the device copy. */
#define TBSLA_CSR_AUTO (-1)
#define TBSLA_CSR_MERGE 0
#define TBSLA_CSR_ROWBLOCK 1
#define TBSLA_CSR_SELL 2
int tbsla_matrix_set_csr_algorithm(tbsla_matrix* m, int algorithm, int items);
/* Sliced-ELL layout: the columns are split into blocks of at most
 * col_block columns (0 = 8,388,608, i.e. 64 MiB of FP64 x, about what L2
 * keeps for gathers), processed one launch each (the last of several in two
 * parts by rows), the first writing r and the others adding to it.  Within
 * a block, rows of at most short_thr (0..255) entries take one
 * lane each and are sorted by length within windows of `sigma` (32..2^23)
 * consecutive rows; longer rows take the fewest lanes (a power of two up to
 * 32) that keep their slice at most long_thr steps wide and are sorted by
 * length over the whole block (defaults 0, 0, 16384, 0; a threshold of 0
 * is automatic: 128 for FP64 values with several column blocks, whose
 * per-block row lengths are about halved, else 64).  Changing them rebuilds the
 * device copy. */
int tbsla_matrix_set_sell_params(tbsla_matrix* m, int short_thr, int long_thr, int sigma, int col_block);
/* Batched personalised PageRank with FP32 / BF16 values: gathers of X rows
 * in flight per warp, 8 (default) or 16; a tuning choice, same results. */
int tbsla_matrix_set_pagerank_gather(tbsla_matrix* m, int gather);
/* Batched PageRank with FP32 / BF16 values: 1 (default) a warp takes a
 * whole row block and walks its entries as one stream, `gather` X rows in
 * flight across row boundaries; 0 a warp per row.  The same Y bit for bit
 * (each row sums in entry order either way); the norms' partial sums are
 * added in another order.  The row-block form keeps X row offsets in 32
 * bits, so with n_col * nvec >= 2^31 the warp-per-row form runs whatever
 * this setting.  No reference counterpart. */
int tbsla_matrix_set_pagerank_stream(tbsla_matrix* m, int stream);
/* PageRank with the sliced-ELL kernel and one column block: 1 (default)
 * runs each step's epilogue -- the new iterate and its three FP64 sums --
 * inside the SpMV launch; 0 writes A x and runs the epilogue as a pass of
 * its own (the form used with several column blocks).  Both sum in a fixed
 * order; their vectors agree to rounding.  No reference counterpart. */
int tbsla_matrix_set_pagerank_fused(tbsla_matrix* m, int fused);

/* One CSR kernel configuration and its measured time. */
typedef struct {
  int algorithm;  /* TBSLA_CSR_SELL / _MERGE / _ROWBLOCK */
  int items;      /* set_csr_algorithm's `items` (SELL: steps in flight) */
  int short_thr, long_thr, sigma, col_block; /* SELL layout */
  int tile;       /* ROWBLOCK entries per block */
  double ms;      /* mean device time of one Ax, CUDA events, L2 warm */
} tbsla_tuning;
/* Autotuner (CSR): times every candidate configuration -- the sliced-ELL
 * kernel over its layout thresholds, column blocks and steps in flight, the
 * merge-path kernel and the row-block kernel -- on this matrix (`reps` Ax
 * each after one warm-up, x = 1), leaves the handle set to the fastest and
 * writes it to *best.  trials (optional): the first max_trials timings in
 * candidate order, their count in *ntrials.  The device copy is rebuilt for
 * every layout tried. */
int tbsla_matrix_autotune(tbsla_matrix* m, int reps, tbsla_tuning* best, tbsla_tuning* trials, int max_trials,
                          int* ntrials);

/* ---- SpMV: Matrix::Ax / Matrix::spmv (Matrix.hpp:14-15) ----------------------- */
/* r <- A v (CSR, ELL: overwrite; returns without touching r when nnz == 0)
 * r += A v (COO, SCOO, DENSE: accumulate into the caller's r).
 * vect_incr shifts output rows for COO/SCOO (MatrixCOO.cpp:140,
 * MatrixSCOO.cpp:162); other formats ignore it, as in the reference.
 * Lengths: v has n_col (COO) or ln_col entries; r has n_row (COO) or ln_row. */
int tbsla_Ax(const tbsla_matrix* m, double* r, const double* v, int vect_incr);
/* r <- A v into a zero-filled r (the reference returns a new[] array). */
int tbsla_spmv(const tbsla_matrix* m, double* r, const double* v, int vect_incr);
/* The same on device pointers r and v, enqueued on `stream` (a
 * cudaStream_t; NULL = the handle's own stream) and not waited for.  Work the
 * call forks onto the handle's internal streams (the second row part of a
 * blocked sliced-ELL layout) is joined back into `stream` before it returns,
 * so everything enqueued on `stream` afterwards sees r complete.  One call
 * at a time per handle: the internal streams, events and work counters are
 * the handle's. */
int tbsla_Ax_device(const tbsla_matrix* m, double* r, const double* v, int vect_incr,
                    void* stream);
int tbsla_spmv_device(const tbsla_matrix* m, double* r, const double* v, int vect_incr,
                      void* stream);

/* Allocation-free CSR SpMV: r <- A v for a CSR matrix already in device
 * memory owned by the caller (rowptr: n_row + 1 ints, nnz = rowptr[n_row] -
 * rowptr[0]; colidx, FP64 values: nnz; v indexed by colidx - f_col; r:
 * n_row), on `stream` of the current device.  No reference counterpart: the
 * reference has no device memory.  It is for callers that may not allocate
 * on the call path -- an application whose memory pool owns the device, or
 * a loop that must not call the CUDA allocator -- and that cannot build a
 * handle, which copies the matrix and allocates per-matrix scratch.  The
 * merge-path kernel's scratch (tile starts and carries) lives in a fixed
 * device array inside the library of 1,048,832 bytes (about 1 MiB: 65,536
 * FP64 carries, 65,536 int32 carry rows and 65,537 int32 tile starts),
 * which every device that loads the library holds until exit, so n_row +
 * nnz may not exceed TBSLA_NOALLOC_MAX_ITEMS (TBSLA_ERR_INVALID_ARG
 * otherwise).  Each call looks the array's device address up; the first
 * call on a device loads the library's module there and should come before
 * any stream capture.
 * Calls that overlap in time share the array and race: serialise them.
 * Results equal tbsla_Ax_device on a handle set to TBSLA_CSR_MERGE with 8
 * items. */
#define TBSLA_NOALLOC_MAX_ITEMS 134217728L
int tbsla_csr_Ax_device_noalloc(int n_row, long nnz, int f_col, const int* rowptr, const int* colidx,
                                const double* values, const double* v, double* r, void* stream);

/* ---- composite ops: Matrix.cpp:5-31 ------------------------------------------ */
/* r <- A(Av + v) (a_axpx_, returns a new array in the reference). */
int tbsla_a_axpx_(const tbsla_matrix* m, double* r, const double* v, int vect_incr);
/* buffer <- Av; buffer += v; r <- A buffer (Ax semantics of the format). */
int tbsla_AAxpAx(const tbsla_matrix* m, double* r, const double* v, double* buffer,
                 int vect_incr);
/* AAxpAx, then r += v. */
int tbsla_AAxpAxpx(const tbsla_matrix* m, double* r, const double* v, double* buffer,
                   int vect_incr);

/* ---- column-stochastic preparation: get_col_sums / normalize_cols /
 *      make_stochastic (MatrixCSR.cpp:1192-1232, Matrix.cpp:33-38) ----------- */
/* s[j - f_col] += sum_i a_ij over the handle's values (s has ln_col entries). */
int tbsla_get_col_sums(tbsla_matrix* m, double* s);
/* a_ij /= s[j - f_col] where that is > 0; updates host and device values. */
int tbsla_normalize_cols(tbsla_matrix* m, const double* s);
/* s <- column sums (zeroed first), then normalize_cols(s). */
int tbsla_make_stochastic(tbsla_matrix* m, double* s);

/* ---- SpMM and the sparse-softmax helpers, CSR only ---------------------------
 * tbsla_dense_multiply: MatrixCSR::dense_multiply (MatrixCSR.cpp:1269-1281),
 * C (n_row x cols_B, row-major) = A B with B (n_col x cols_B) indexed by
 * the column as stored; C is overwritten.
 * tbsla_get_row_max_abs: get_row_max_abs (:1283-1312), max |a_ij| per local
 * row (0 for an empty row).
 * tbsla_apply_exponential: apply_exponential (:1315-1334), every nonzero a_ij
 * becomes exp(a_ij - max_abs[i]) (base <= 0) or base^(a_ij - max_abs[i]);
 * no shift when max_abs is NULL.
 * tbsla_get_row_sums: get_row_sums (:1147-1164), s[i] = sum of local row i
 * in entry order (s has ln_row entries).
 * tbsla_normalize_rows: normalize_rows (:1177-1190), a_ij /= s[i], or 0
 * where s[i] = 0 (the reference's safeguard). */
int tbsla_dense_multiply(const tbsla_matrix* m, const double* B, double* C, int cols_B);
int tbsla_get_row_max_abs(const tbsla_matrix* m, double* max_abs);
int tbsla_apply_exponential(tbsla_matrix* m, const double* max_abs, int base);
int tbsla_get_row_sums(const tbsla_matrix* m, double* s);
int tbsla_normalize_rows(tbsla_matrix* m, const double* s);

/* ---- PageRank (src/mpi/matrix/Matrix.cpp:540-602, 641-790), CSR only --------
 * A column-stochastic (zero columns = dangling nodes).  x_0 = 1/n and, with
 * each iterate normalised by its sum S_k before use,
 *   x_{k+1} = beta*A x_k/S_k + (1 - beta*M_k/S_k) * t,  t = 1/n,
 * M_k = sum_j w_j x_k[j], w_j = sum of column j of A as stored.  For exact
 * column-stochastic A this is the usual (1-beta) + beta*D_k/S_k dangling-node
 * redistribution (D_k = mass on dangling nodes); with FP32/BF16 storage it
 * also returns the mass the rounding loses.  Stops when
 * sum|x_{k+1} - x_k/S_k| < epsilon or after max_iterations; the result is
 * divided by its sum.  *iterations receives the count, *error the last L1
 * change.  Returns TBSLA_ERR_NOT_CONVERGED (result still written) when the
 * limit is hit first. */
int tbsla_page_rank(tbsla_matrix* m, double beta, double epsilon, int max_iterations,
                    double* result, int* iterations, double* error);
/* Personalised PageRank for nvec teleport vectors at once (one SpMM-style
 * matrix pass per iteration).  teleport and result are n x nvec row-major;
 * each teleport column must sum to 1.  Runs until every column's L1 change
 * is < epsilon or max_iterations.  nvec <= 32. */
int tbsla_page_rank_batched(tbsla_matrix* m, int nvec, const double* teleport, double beta,
                            double epsilon, int max_iterations, double* result,
                            int* iterations);

/* ---- CG (src/mpi/matrix/CG.cpp:32-73) ------------------------------------------
 * Solves A x = b for SPD CSR A from the start vector in x, stopping at
 * ||b - A x|| <= rel_tol * ||b||.  precond: 0 none, 1 Jacobi.  The SpMV runs
 * on the handle's value precision; with TBSLA_F32/TBSLA_BF16 storage the
 * residual is recomputed in FP64 from FP64 values every `refresh` iterations
 * (0 = never).  rel_residual receives the FP64 true residual at exit. */
int tbsla_cg(tbsla_matrix* m, const double* b, double* x, int max_iterations, double rel_tol,
             int precond, int refresh, int* iterations, double* rel_residual);

/* ---- batched CG: many SPD systems of uneven size solved together ------------------
 * (CG.cpp:32-73 per system).  tbsla_batch_create concatenates nsys square CSR
 * handles (f_col 0) into one block-diagonal device matrix, values in
 * `precision` plus an FP64 copy for the true residual, and the Jacobi
 * diagonal.  tbsla_batch_cg solves all systems from the start vectors in x;
 * rhs and x are the systems' vectors concatenated in order (offsets from
 * tbsla_batch_rows).  Each system stops on its own when its FP64 true
 * residual satisfies ||b - A x|| <= rel_tol ||b||; iterations[s] and
 * rel_residual[s] receive its count and final true relative residual.
 * precond: 0 none, 1 Jacobi, 2 the factors of tbsla_batch_set_factors
 * (z = L L^T r).  With FP32 / BF16 storage the iteration runs in FP32 as the
 * inner solver of FP64 iterative refinement: every `refresh` iterations
 * (and on apparent convergence) the correction is added to x in FP64, the
 * FP64 true residual b - A x replaces r and the iteration restarts.
 * graph_iters: iterations captured per CUDA graph replay of the
 * multi-launch engine (0: 10); the persistent engine runs the whole solve in
 * one launch.  Returns TBSLA_ERR_NOT_CONVERGED if some system hit
 * max_iterations, TBSLA_ERR_TIMEOUT if a bounded device wait ran out. */
typedef struct tbsla_batch tbsla_batch;
int tbsla_batch_create(tbsla_batch** b, tbsla_matrix* const* systems, int nsys, int precision);
int tbsla_batch_destroy(tbsla_batch* b);
int tbsla_batch_rows(const tbsla_batch* b, int* nsys, long* offsets);
int tbsla_batch_cg(tbsla_batch* b, const double* rhs, double* x, int max_iterations, double rel_tol,
                   int precond, int refresh, int graph_iters, int* iterations,
                   double* rel_residual);
/* After the last tbsla_batch_cg, per system: fallback[s] = 0 when it ran
 * with the preconditioner asked for, 1 when its factor failed the check made
 * before the first iteration (a non-finite value or a diagonal entry <= 0)
 * and it ran Jacobi-PCG instead, 2 when its factored iteration stopped making
 * progress (a refinement cycle that did not lower the FP64 true residual, a
 * cycle of 25 iterations or more that cut it by less than 10%, or r.z not
 * positive and finite) and it continued with Jacobi-PCG;
 * precond_used[s] = the preconditioner it ended with (0, 1, 2).  Either
 * pointer may be NULL.  Plain Jacobi-PCG is the fallback of the factored
 * preconditioner: the reference's CG (CG.cpp:32-73) has none. */
int tbsla_batch_fallbacks(const tbsla_batch* b, int* fallback, int* precond_used);
/* Bound, in nanoseconds, on one grid-wide wait of the persistent solver
 * (default 2e9).  A wait that runs out ends that solve on the GPU with
 * TBSLA_ERR_TIMEOUT; the batch stays usable. */
int tbsla_batch_set_wait_limit(tbsla_batch* b, long long ns);
/* Persistent engine tuning: rows per thread in the hot phases, 4 (the
 * default where every system's first row and size are multiples of 4 and the
 * iteration runs in FP32: 16-byte loads) or 1 (one row per thread, as for
 * every other batch).  The arithmetic of each row is the same either way. */
int tbsla_batch_set_rows_per_thread(tbsla_batch* b, int rows);
/* Persistent engine tuning: CTAs per SM of the cooperative launch (0,
 * the default: as many as fit, 3 for the FP32 iteration; at most that).
 * The work is handed out in warp units whatever the grid, so results agree
 * to the FP64 atomics' summation order. */
int tbsla_batch_set_ctas_per_sm(tbsla_batch* b, int ctas);
/* The persistent engine's current rows per thread and CTAs per SM (0: all
 * that fit); either pointer may be NULL. */
int tbsla_batch_tuning(const tbsla_batch* b, int* rows_per_thread, int* ctas_per_sm);
/* The engine of the last tbsla_batch_cg: persistent = 1 when the whole solve
 * was one cooperative launch (every system's entries on at most 8 diagonals,
 * at most 256 systems, a factor, if used, on at most 8 diagonals), 0 for the
 * multi-launch engine; graph = 1 when it was replayed from a CUDA graph;
 * seven_point = 1 when the persistent kernel ran in its seven-point form
 * (every system a 7-point stencil whose line and plane sizes are multiples
 * of 4, FP32 / BF16 storage: the neighbour alignments fixed when compiled).
 * Any pointer may be NULL. */
int tbsla_batch_engine(const tbsla_batch* b, int* persistent, int* graph, int* seven_point);
/* 1 (default): the seven-point form where it applies; 0: always the general
 * form (the same arithmetic in the same order). */
int tbsla_batch_set_seven_point(tbsla_batch* b, int on);
/* Factored preconditioner M^-1 = L L^T for every system of the batch (L:
 * lower-triangular CSR handles, one per system, same sizes), used by
 * tbsla_batch_cg with precond = 2.  Values are stored in `precision`
 * (TBSLA_F64 / F32 / BF16); M stays SPD whatever the rounding, since it is
 * L L^T of the rounded L with a positive diagonal.  z = L (L^T r) is
 * computed in FP32 arithmetic on r rounded to FP32; r.z and the CG vectors
 * stay FP64. */
int tbsla_batch_set_factors(tbsla_batch* b, tbsla_matrix* const* factors, int nsys, int precision);

/* ---- learned preconditioner (no reference counterpart) ------------------------
 * A message-passing network over the pattern of an SPD CSR matrix A that
 * emits L on the pattern of tril(A) with a positive diagonal, so that
 * M^-1 = L L^T is SPD; untrained it is Jacobi (L = D^-1/2).  6,467
 * parameters (3 layers, width 32), bfloat16 weights in the forward pass,
 * FP32 master weights and Adam state.  Trained on the GPU with the loss
 * sum (L L^T A Z - Z)^2 / (n P) over P Gaussian probes (P <= 16).  A must be
 * symmetric with a positive diagonal (TBSLA_ERR_BAD_MATRIX otherwise). */
typedef struct tbsla_mpnn tbsla_mpnn;
int tbsla_mpnn_create(tbsla_mpnn** net, unsigned long long seed);
int tbsla_mpnn_destroy(tbsla_mpnn* net);
/* FP32 master parameters (nparams = 6467); theta may be NULL. */
int tbsla_mpnn_params(const tbsla_mpnn* net, float* theta, int* nparams);
/* Loads parameters and resets the Adam state. */
int tbsla_mpnn_set_params(tbsla_mpnn* net, const float* theta, int nparams);
/* Loss and its gradient (FP32, 6467) on the probes Z (n x nprobes row-major). */
int tbsla_mpnn_loss_grad(tbsla_mpnn* net, const tbsla_matrix* A, int nprobes, const double* Z, double* loss,
                         float* grad);
/* One Adam step (betas 0.9 / 0.999) on A with nprobes probes drawn from `seed`. */
int tbsla_mpnn_train_step(tbsla_mpnn* net, const tbsla_matrix* A, int nprobes, unsigned long long seed, float lr,
                          double* loss);
/* Writes L (CSR: per row its strictly lower entries, then the diagonal)
 * into the CSR handle L. */
int tbsla_mpnn_factor(tbsla_mpnn* net, const tbsla_matrix* A, tbsla_matrix* L);
/* The network's factor for every system of a batch, computed on the GPU from
 * the batch's device copy of A and written straight into the batch's factor
 * storage (precision TBSLA_F32 or TBSLA_BF16; TBSLA_F64 is kept as F32, the
 * precision the factor is applied in): no host copy of A, L or L^T.  The
 * same L as tbsla_mpnn_factor on each system (entries of A stored as exact
 * zeros count as absent).  Requires a batch on the persistent engine
 * (TBSLA_ERR_UNSUPPORTED otherwise); then tbsla_batch_cg with precond = 2. */
int tbsla_batch_factor_mpnn(tbsla_batch* b, tbsla_mpnn* net, int precision);
/* The batch's factor in its diagonal-slot form, for inspection: *slots = the
 * slots per row (KL); deltas[s * 8 + q] = column - row of slot q of system s
 * (slot 0 the diagonal); values[q * n + i] = the stored value of row i on
 * slot q, widened to double (n = the batch's rows).  Any pointer may be NULL.
 * TBSLA_ERR_UNSUPPORTED when the batch holds no factor in that form. */
int tbsla_batch_factor_dia(const tbsla_batch* b, int* slots, int* deltas, double* values);

#ifdef __cplusplus
}
#endif

#endif /* TBSLA_GB300_H */
