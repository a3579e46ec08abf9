// Host-callable launchers of the SpMV-path kernels (one translation unit per
// kernel family).  All take device pointers and a stream; none synchronise.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tbsla_gpu {

enum Prec { kF64 = 0, kF32 = 1, kBF16 = 2 };

// Control block of the persistent kernels: [0] next work item, [1] CTAs
// finished; both return to 0 at the end of every launch (the last CTA
// resets them).
struct Ctl {
  unsigned* counter;
  double* partials;  // gridDim.x * nred doubles
  double* result;    // nred doubles
};

// ---- CSR (row-block adaptive) ------------------------------------------------
struct CsrArgs {
  const void* vals;
  int prec;
  const int* rowptr;
  const int* colidx;
  const int* blocks;  // nblocks + 1 row boundaries
  int nblocks;
  int f_col;
  int items;  // nnz budget per block / 256 (4, 8 or 16)
};
// y[row] = (A x)[row] for every row of the partition.
cudaError_t csr_spmv(const CsrArgs& a, const double* x, double* y, cudaStream_t s);
// Merge-path CSR SpMV (the default CSR kernel): tiles of 256*items items of
// the merged (row ends, entries) sequence; coord[ntiles+1] holds each tile's
// first row, carry_row / carry_val[ntiles] are per-tile scratch.
struct MergeArgs {
  const void* vals;
  int prec;
  const int* rowptr;
  const int* colidx;
  int n;
  long nnz;  // rowptr[n] - rowptr[0]
  int f_col;
  int items;  // 4, 8 or 16
  const int* coord;
  long ntiles;
  int* carry_row;
  double* carry_val;
};
long merge_tiles(int n, long nnz, int items);
cudaError_t csr_merge_setup(const int* rowptr, int n, long nnz, int items, int* coord, cudaStream_t s);
cudaError_t csr_merge_spmv(const MergeArgs& a, const double* x, double* y, cudaStream_t s);
// The merge-path SpMV (FP64 values, 8 items per thread) with its scratch in
// a file-scope device array: allocates nothing; n + nnz at most
// csr_merge_noalloc_max_items(); concurrent calls race on the scratch.
long csr_merge_noalloc_max_items();
cudaError_t csr_merge_spmv_noalloc(const double* vals, const int* rowptr, const int* colidx, int n, long nnz,
                                   int f_col, const double* x, double* y, cudaStream_t s);

// Sliced-ELL CSR SpMV (SELL-C-sigma with C = 32) for GB300's FP64 pipe,
// which costs one slot per warp-instruction whatever the active lanes.  A
// slice is 32 lanes, each row owning G = 2^g consecutive lanes (entry j of
// the row on lane j mod G of its group, at step j / G); its entries are
// stored step-major (step t, lane l at 32 * (offset + t) + l).  Rows of at
// most short_thr entries take one lane each and are sorted by length within
// windows of `sigma` consecutive rows; longer rows take the fewest lanes (up
// to 32) that keep their slice at most long_thr steps wide and are sorted by
// length over the whole block.  One warp per slice, fetched dynamically,
// widest slices first; lanes past their row's end issue no loads, so
// padding costs no traffic.
//
// The columns are split into blocks small enough for their part of x to
// stay in L2 while the block runs (x beyond ~60 MB misses L2 for most
// gathers on GB300); each block has its own plan and launch, the first
// writing y, the others adding to it in block order.
struct SellPlan {
  int n = 0;
  int col_lo = 0, col_hi = 0;  // the block's columns, relative to f_col
  int nwide = 0;               // slices sorted over the whole block (processed first)
  int nslices = 0;             // all slices of the block
  long sell_len = 0;           // elements of the block's slices
  int4* slice = nullptr;       // [nslices]: {step offset, width in steps, g, base}
  int* lane = nullptr;         // [32 * nslices]: base >= 0: (row - base) << 8 | len;
                               // base = -1: row; -1 for an unused lane
  int* lane_len = nullptr;     // [32 * nwide]: the row's entries in the block
  int row_lo = 0, row_hi = 0;  // rows the plan may hold (a part of the last block: its rows)
};
// Parts by rows of the last column block (when there are several blocks).
constexpr int kRowParts = 2;
// Host: plan of one column block from its per-row entry counts L[n]
// (arrays allocated with new[]); rows with no entry are left out when
// skip_empty; step offsets start at step0.
void sell_plan_build(const int* L, int n, int short_thr, int long_thr, int sigma, bool skip_empty, long step0,
                     SellPlan* p);
void sell_plan_free(SellPlan* p);
struct SellArgs {
  const void* vals;  // CSR copy (the slice arrays are filled from it)
  int prec;
  const int* rowptr;
  const int* colidx;
  int f_col;
  void* svals;  // slice arrays of all blocks
  int* scols;
  int unroll;               // steps per lane in flight: 4, 8 or 16
  int nblocks;              // column blocks
  const SellPlan* blocks;   // host array of plans holding device pointers
  // optional, per plan: the launch of plan b > 0 waits for ready[b] (its
  // part of x arriving on another stream), and after[b], when not null, is
  // recorded once plan b is launched
  const cudaEvent_t* ready = nullptr;
  const cudaEvent_t* after = nullptr;
  // Row parts: the last `parts` plans split the last column block by rows.
  // They do not depend on one another, so with side streams part k >= 1
  // runs on side[k - 1] (forked after the earlier blocks, joined back
  // before sell_spmv returns); the side streams have falling priorities,
  // so each part's CTAs fill the tail of the part before it.
  int parts = 1;
  const cudaStream_t* side = nullptr;  // [parts - 1]
  cudaEvent_t fork = nullptr;
  const cudaEvent_t* join = nullptr;   // [parts - 1]
};
// Fills the slice arrays of every block from the CSR device arrays.
cudaError_t sell_fill(const SellArgs& a, cudaStream_t s);
// y = A x, one launch per plan; counter: kSellCounterWords unsigned of
// zeroed scratch (a region per launch that may run at once), reset by each
// launch; a set *done (device) makes the launches no-ops.
constexpr int kSellCounterRegion = 1024;
constexpr int kSellCounterWords = kRowParts * kSellCounterRegion;
cudaError_t sell_spmv(const SellArgs& a, const double* x, double* y, unsigned* counter, cudaStream_t s,
                      const int* done = nullptr);

// Row-block partition of a CSR row pointer (host): blocks of consecutive
// rows with at most `tile` entries and at most 256 rows each; a row longer
// than `tile` forms a block on its own.  Returns the boundaries.
void csr_partition(const int* rowptr, int n_row, int tile, int** out, int* nblocks);

// PageRank step on CSR with the iterate carried unnormalised: with
// s = coef_in[0] = 1/S (S = sum x) and t = coef_in[1],
//   y_i = (beta * (A x)_i) * s + c_i,  c_i = t / n or t * tele_i.
// Reductions: L1 change sum |y - x s|, S' = sum y, M' = sum_i colw_i y_i
// (colw = column sums of A as stored; 0 for a dangling node); the last CTA
// writes coef_out = {1/S', 1 - beta M'/S'} and sets *done when the change is
// below eps (a done flag already set makes the launch a no-op).
struct PageRankArgs {
  double beta;
  double n_nodes;
  double eps;
  const double* tele;
  const double* colw;
  const double* coef_in;
  double* coef_out;
  int* done;
  int* iters;
};
cudaError_t csr_pagerank_step(const CsrArgs& a, const double* x, double* y,
                              const PageRankArgs& p, Ctl ctl, int grid, cudaStream_t s);
// One PageRank step on the sliced-ELL layout of a single column block (one
// plan, no row parts): y = the next iterate, its sums reduced in a fixed
// order, as csr_pagerank_step; ctl.partials holds 3 doubles for each of up
// to 8 CTAs per SM.  cudaErrorInvalidValue for a plan of several blocks.
cudaError_t sell_pagerank(const SellArgs& a, const double* x, double* y, const PageRankArgs& p, Ctl ctl,
                          cudaStream_t s);
// Batched personalised PageRank step: X, Y, T are n x nvec row-major
// (nvec <= 32); column k as above with s_k = coef_in[k], t_k =
// coef_in[32 + k] and c_i = t_k * T[i, k].  Reductions per column k:
// result[k] = L1 change, result[nvec + k] = S', result[2 nvec + k] = M';
// the last CTA writes coef_out[k], coef_out[32 + k] and sets *done when
// every column's change is < eps.
// The same in double-float (pairs of floats h + l, about 46 bits) for FP32 /
// BF16 values: X, Y, T (n x nvec) and W (the column sums, n) are float2
// arrays of the same byte size as FP64 ones; reductions are FP64.  gather:
// X-row gathers in flight per warp (8 or 16); stream: 0 a warp per row (the
// CTA's warps take a block's rows in turn), 1 a warp per row block, its
// entries walked as one stream across row boundaries.
cudaError_t csr_pagerank_batched_df_step(const CsrArgs& a, int nvec, const void* X, void* Y, const void* T,
                                         const void* W, const PageRankArgs& p, Ctl ctl, int grid, int gather,
                                         int stream, cudaStream_t s);
// FP64 <-> double-float (float2) conversions, element by element (the
// destination may be the source's own storage).
cudaError_t f64_to_df(const double* src, void* dst, long n, cudaStream_t s);
cudaError_t df_to_f64(const void* src, double* dst, long n, cudaStream_t s);
cudaError_t csr_pagerank_batched_step(const CsrArgs& a, int n_row, int nvec, const double* X,
                                      double* Y, const double* T, const PageRankArgs& p,
                                      Ctl ctl, int grid, cudaStream_t s);

// PageRank step after a separate SpMV t = A x (the sliced-ELL path): the
// same y, reductions and coefficients as csr_pagerank_step, over n rows, in
// `grid` CTAs (ctl sized for grid x 3 partials).
cudaError_t pagerank_epilogue(const double* t, const double* x, double* y, long n, const PageRankArgs& p,
                              Ctl ctl, int grid, cudaStream_t s);

// CTAs of the persistent PageRank kernels (resident capacity of the GPU).
int csr_pagerank_grid(int items, int prec);
int csr_pagerank_batched_grid(int prec, int gather, int stream);

// ---- batched CG over a block-diagonal concatenation of systems -------------------
// Per-system status: ACTIVE iterates; VERIFY has a recursive residual below
// the tolerance and waits for the FP64 true-residual check; DONE passed it;
// STOPPED hit the iteration limit.
enum CgStatus { kActive = 0, kVerify = 1, kDone = 2, kStopped = 3, kRestart = 4 };
struct CgBatch {
  int nsys;
  long n;
  const int* rowptr;
  const int* colidx;
  const void* vals;  // storage precision `prec` (the iteration's SpMV)
  int prec;
  const double* vals64;  // FP64 values (true residual)
  const int* blocks;     // SpMV row-block partition, no block spans two systems
  const int* block_sys;
  int nblocks;
  int items;
  const int* chunks;  // vector row chunks, no chunk spans two systems
  const int* chunk_sys;
  int nchunks;
  const double* dinv;  // Jacobi: 1/diag(A); nullptr = unpreconditioned
  // factored preconditioner z = L (L^T r) (nullptr lrowptr = none): L and
  // L^T as CSR, values in `lprec`, applied in FP32 arithmetic: rf = fp32(r),
  // tf = L^T rf, z = fp64(L tf)
  const int *lrowptr, *lcolidx, *trowptr, *tcolidx;
  const void *lvals, *tvals;
  int lprec;
  // ELL form of L and L^T (lslots > 0; then no CSR arrays): slot-major
  // values [slot * n + i] and column offsets from the row as int16, padded
  // with value 0 at offset 0
  const short *ldelta, *tdelta;
  int lslots, tslots;
  float *rf, *tf;  // set for a factored run
  float* zf;       // factored run: z in FP32 (computed in FP32, so exactly)
  const double* b;
  double *x, *r, *z, *p, *q;  // z == r when unpreconditioned
  // per-system scalars (rrt: squared FP64 true residual of the last check)
  double *rz, *rz_new, *pq, *rr, *bb, *beta, *rrt;
  int* status;
  int* iters;
  double tol2;
  int max_it;
};
// ---- persistent batched CG on diagonal-structured systems (cg_dia.cu) ----------
constexpr int kDiaMaxDiag = 8;   // diagonals per system (A and L)
constexpr int kDiaMaxSys = 256;  // systems per batch
enum DiaFallback { kFallbackNone = 0, kFallbackBadFactor = 1, kFallbackStagnation = 2 };
struct DiaCg {
  int nsys;
  long n;
  int K, KL;              // diagonal slots of A and of L (batch-wide, zero-padded)
  const long* sys_off;    // [nsys + 1] first row of each system
  const int* adelta;      // [nsys * kDiaMaxDiag] col - row of each slot of A (padding: 0, value 0)
  const void* avals;      // [K][n] in `prec` (the iteration's A)
  int prec;
  const double* a64;      // [K][n] FP64 (true residual)
  const float* dinv;      // [n] Jacobi
  const int* ldelta;      // [nsys * kDiaMaxDiag] L's deltas (<= 0), slot 0 the diagonal
  const void* lvals;      // [KL][n] in `lprec` (F32 or BF16)
  int lprec;
  const double* b;
  double* x;
  void *d, *r0, *r1, *p0, *p1, *q, *z, *t;  // FP32 (narrow storage) or FP64 vectors
  int* mode;              // [nsys] in: preconditioner per system; out: the one it ended with
  int* status;            // [nsys] out: kDone / kStopped
  int* iters;             // [nsys] out
  int* fallback;          // [nsys] out: DiaFallback
  double* relres;         // [nsys] out: FP64 true relative residual at exit
  double* acc;            // [3][4][nsys] rotating accumulator slots (zeroed before launch)
  unsigned* bar;          // [4] grid barrier: count, generation, error (zeroed before launch)
  double tol2;
  int max_it;
  int refresh;            // iterations per refinement cycle (narrow storage), 0 = never
  int vec4;               // every system's first row and size a multiple of 4, FP32 iteration:
                          // the hot phases take 4 rows per thread with 16-byte loads
  int st7;                // with vec4: every system in the seven-point form (dia_seven_point)
  long long wait_ns;      // bound on one grid-wide wait
};
// Co-resident CTAs of the persistent kernel for (prec, lprec, seven-point
// form) on this device.
int cg_dia_grid(int prec, int lprec, int st7);
// Host check of the seven-point form: every system has K = 7 slots whose
// deltas fall in the alignment classes of -n^2, -n, -1, 0, +1, +n, +n^2 with
// n^2 and n multiples of 4 (ascending slot order), and, with a factor
// (ldelta not null), KL = 4 slots in the classes of 0, -1, -n, -n^2.
bool dia_seven_point(const int* adelta, const int* ldelta, int nsys, int K, int KL);
// The whole batched solve, one cooperative launch of `grid` CTAs.
cudaError_t cg_dia_solve(const DiaCg& c, int grid, cudaStream_t s);
// out[k * n + i] = value of row i on slot k (zeroed by the caller).
cudaError_t dia_fill(const int* rowptr, const int* colidx, const double* vals, const int* row_sys,
                     const int* delta, int K, long n, double* out, cudaStream_t s);
cudaError_t dia_dinv(const double* a64, const int* row_sys, const int* delta, int K, long n, float* dinv,
                     cudaStream_t s);

cudaError_t cg_spmv_dot(const CgBatch& c, cudaStream_t s);   // q = A p; pq += p.q
cudaError_t cg_update(const CgBatch& c, cudaStream_t s);     // x += a p; r -= a q; z = M r; dots
cudaError_t cg_scalars(const CgBatch& c, cudaStream_t s);    // beta, status, iteration counts
cudaError_t cg_direction(const CgBatch& c, cudaStream_t s);  // p = z + beta p
// Factored preconditioner for the systems whose status is in `mask`:
// t = L^T r, z = L t, acc[sys] += r.z.
cudaError_t cg_factor_apply(const CgBatch& c, int mask, double* acc, cudaStream_t s);
// r = b - A64 x, z = M r, rr = r.r, rz = r.z for systems whose status is in
// `mask` (bit per status); then each VERIFY system becomes DONE (true residual
// within tolerance) or RESTART; with `init` every system is set from the result.
cudaError_t cg_true_residual(const CgBatch& c, int mask, bool init, cudaStream_t s);
// p = z for RESTART systems (then ACTIVE), or for every system with `all`.
cudaError_t cg_restart(const CgBatch& c, bool all, cudaStream_t s);
// bb = b.b per system.
cudaError_t cg_norms(const CgBatch& c, cudaStream_t s);
// Diagonal inverse of a CSR matrix (rows without a diagonal entry get 1).
cudaError_t csr_diag_inv(const int* rowptr, const int* colidx, const double* vals, long n,
                         double* dinv, cudaStream_t s);

// ---- ELL (column-major device copy) -------------------------------------------
cudaError_t ell_spmv(const void* vals, int prec, const int* cols, int ln_row, int max_col,
                     int f_col, const double* x, double* y, cudaStream_t s);

// ---- COO / SCOO (row-sorted device copy, reduce-by-key) ----------------------
// Triplets per warp chunk, and the carry scratch of a launch: per chunk the
// partial sums of its first / last row when that row crosses into a
// neighbouring chunk, and flags (int).
constexpr int kCooChunk = 256;
inline long coo_chunks(long nnz) { return (nnz + kCooChunk - 1) / kCooChunk; }
struct CooCarry {
  double* head;  // [chunks]
  double* tail;  // [chunks]
  int* flags;    // [chunks]
};
// y[row + row_off] += sum of vals * x[col + col_off] over entries of that
// row: one addition per row, the same from run to run.
cudaError_t coo_spmv(const void* vals, int prec, const int* rows, const int* cols, long nnz,
                     int row_off, int col_off, const double* x, double* y, const CooCarry& cc, cudaStream_t s);

// ---- DENSE (row-major GEMV, accumulating) -------------------------------------
cudaError_t dense_gemv(const void* vals, int prec, int ln_row, int ln_col, const double* x,
                       double* y, cudaStream_t s);
// FP32 / BF16 values in double-float arithmetic (FP32 pipes): x split into
// xs[0, ln_col) = xh and xs[ln_col, 2 ln_col) = xl; *bad (device int) is cleared, then set by the
// split when x leaves the [2^-40, 2^40] magnitude range, in which case the
// same launch computes in FP64.  The values must have passed
// dense_values_df_range, which checks them once (synchronises on s).
cudaError_t dense_gemv_df(const void* vals, int prec, int ln_row, int ln_col, const double* x, float* xs,
                          int* bad, double* y, cudaStream_t s);
cudaError_t dense_values_df_range(const void* vals, int prec, size_t n, int* flag, bool* ok, cudaStream_t s);

// ---- vector / preparation kernels ---------------------------------------------
cudaError_t vec_add(double* y, const double* x, long n, cudaStream_t s);  // y += x
cudaError_t vec_fill(double* y, double v, long n, cudaStream_t s);
// Column sums of a row-major n x ncol array (ncol <= 32) into out[ncol],
// two passes in a fixed order (deterministic); `partials` holds
// kSumBlocks * 32 doubles.
constexpr int kSumBlocks = 512;
cudaError_t mat_colsum(const double* x, long n, int ncol, double* partials, double* out,
                       cudaStream_t s);
// x[i*ncol + k] /= denom[k]
cudaError_t mat_scale_cols(double* x, long n, int ncol, const double* denom, cudaStream_t s);
// s[col - f_col] += value over all CSR entries (FP64 atomics).
cudaError_t csr_col_sums(const double* vals, const int* rowptr, const int* colidx, int n_row,
                         int f_col, double* s, cudaStream_t st);
// value /= s[col - f_col] where that is > 0.
cudaError_t csr_normalize_cols(double* vals, const int* rowptr, const int* colidx, int n_row,
                               int f_col, const double* s, cudaStream_t st);
// Stable LSD radix sort (8-bit digits) of (key, value) pairs over the low
// `bits` key bits; the result is in the *_alt arrays when *result_in_alt.
// scratch: radix_scratch(n) words.
long radix_scratch(long n);
cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* keys_alt, int* vals, int* vals_alt, long n, int bits,
                             unsigned* scratch, int* result_in_alt, cudaStream_t s);
// Exclusive scan in place; scratch: scan_scratch(n) words.
long scan_scratch(long n);
cudaError_t exclusive_scan(unsigned* a, long n, unsigned* scratch, cudaStream_t s);
// COO -> CSR ordering: perm = the entries sorted by (row, col), ties in
// storage order; rowcount (n_row + 1) becomes the row starts.  scratch:
// max(radix_scratch(n), scan_scratch(n_row + 1)) words.
cudaError_t coo_order(const int* row, const int* col, long n, int n_row, int n_col, uint64_t* keys,
                      uint64_t* keys_alt, int* perm, int* perm_alt, unsigned* rowcount, unsigned* scratch,
                      int* perm_in_alt, cudaStream_t s);
// dense[row * ln_col + col] = the sum, in storage order from 0, of the values
// at each (row, col), given perm from coo_order (dense zeroed by the caller).
cudaError_t coo_dense_scatter(const int* perm, const int* row, const int* col, const double* val, long n,
                              long ln_col, double* dense, cudaStream_t s);

// C = A B (MatrixCSR::dense_multiply): B (rows indexed by the stored
// column) and C row-major with k columns; C rows [0, n_row) written.
cudaError_t csr_dense_multiply(const void* vals, int prec, const int* rowptr, const int* colidx, int n_row,
                               const double* B, int k, double* Cm, cudaStream_t s);
// out[i] = max_j |a_ij| (0 for an empty row).
cudaError_t csr_row_max_abs(const double* vals, const int* rowptr, int n_row, double* out, cudaStream_t s);
// Row sums in entry order (FP64 values) and a_ij / s_i (0 where s_i = 0).
cudaError_t csr_row_sums(const double* vals, const int* rowptr, int n_row, double* out, cudaStream_t s);
cudaError_t csr_normalize_rows(double* vals, const int* rowptr, int n_row, const double* sums, cudaStream_t s);
// a_ij <- exp(a_ij - max_abs[i]) (base <= 0) or base^(a_ij - max_abs[i]) for
// every nonzero a_ij; no shift when max_abs is null.
cudaError_t csr_apply_exponential(double* vals, const int* rowptr, int n_row, const double* max_abs, int base,
                                  cudaStream_t s);

// Narrowing copy of FP64 values to the storage precision.
cudaError_t convert_values(const double* src, void* dst, int prec, long n, cudaStream_t s);
// Row-major -> column-major transpose of ELL arrays.
cudaError_t ell_transpose(const double* vals_rm, const int* cols_rm, void* vals_cm, int prec,
                          int* cols_cm, int ln_row, int max_col, cudaStream_t s);

}  // namespace tbsla_gpu
