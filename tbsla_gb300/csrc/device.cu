// Device copy of a matrix handle and the orchestration of the path's kernels.
//
// HBM layout per format (built once by dev_upload, dropped on host mutation):
//   CSR   rowptr int32[ln_row+1], colidx int32[nnz], values V[nnz],
//         row-block partition int32[nblocks+1], merge-path tile starts and
//         carries, and (default kernel) the sliced-ELL copy: per column
//         block a plan (slice descriptors, lane words) and the step-major
//         values / columns
//   ELL   columns int32[max_col*ln_row] and values V[max_col*ln_row],
//         slot-major (transposed from the reference's row-major)
//   COO/  rows, cols int32[nnz] and values V[nnz], stably sorted by row
//   SCOO
//   DENSE values V[ln_row*ln_col], row-major
// V is the storage precision (double / float / bfloat16); products and sums
// are always FP64.  Vectors are FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "device.hpp"
#include "host/parallel.hpp"
#include "kernels/kernels.hpp"

namespace tbsla_impl {

using namespace tbsla_gpu;

namespace {

int g_device = 0;

#define TRY(call)                                   \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return status_of(e_);    \
  } while (0)

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return TBSLA_OK;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return TBSLA_ERR_ALLOC;
  }
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TBSLA_ERR_NO_DEVICE;
  return TBSLA_ERR_CUDA;
}

int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return TBSLA_ERR_NO_DEVICE;
  }
  return TBSLA_OK;
}

size_t prec_size(int prec) { return prec == TBSLA_F64 ? 8 : prec == TBSLA_F32 ? 4 : 2; }

template <class T>
int dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) return TBSLA_OK;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return TBSLA_ERR_ALLOC;
  }
  return TBSLA_OK;
}

}  // namespace

struct DeviceMatrix {
  int device = 0;
  cudaStream_t stream = nullptr;
  int prec = TBSLA_F64;
  size_t bytes = 0;
  void* vals = nullptr;
  int* idx0 = nullptr;
  int* idx1 = nullptr;
  int* blocks = nullptr;  // CSR row-block partition
  int nblocks = 0;
  int items = 8;
  int algo = 0;            // CSR: 0 merge path, 1 row blocks, 2 sliced ELL
  int* coord = nullptr;    // CSR merge path: first row of each tile
  int* carry_row = nullptr;
  double* carry_val = nullptr;
  long ntiles = 0;
  int merge_items = 8;
  std::vector<SellPlan> sell;  // CSR sliced-ELL layout, one plan per column block (device pointers)
  void* svals = nullptr;
  int* scols = nullptr;
  unsigned* sell_counter = nullptr;
  int sell_parts = 1;  // trailing plans that split the last column block by rows
  std::vector<cudaStream_t> side;  // row parts 1..: falling priorities
  cudaEvent_t fork_ev = nullptr;
  std::vector<cudaEvent_t> join_ev;
  cudaStream_t xstream = nullptr;   // host entry point: x of column blocks 1.. copied here
  std::vector<cudaEvent_t> xready;  // [block]: that block's x has arrived
  double* colw = nullptr;  // PageRank: column sums of the stored values
  bool colw_ok = false;
  double colw_s0 = 0, colw_m0 = 0;  // S and M of the start vector 1/n
  long nnz = 0;  // entries on the device
  int min_row = 0, max_row = -1;
  double* coo_carry = nullptr;  // COO / SCOO: head, tail carries (double) and flags (int) per chunk
  // batched PageRank: two iterates and the teleport vectors (n x nvec), the
  // double-float column sums (n), coefficients and flags, kept between solves
  double *bx0 = nullptr, *bx1 = nullptr, *btele = nullptr, *bw = nullptr, *bcoef = nullptr;
  size_t bx0_len = 0, bx1_len = 0, btele_len = 0, bw_len = 0, bcoef_len = 0;
  double* x = nullptr;
  size_t x_len = 0;
  double* y = nullptr;
  size_t y_len = 0;
  double* t = nullptr;
  size_t t_len = 0;
  bool dense_df = false;     // DENSE, every value within the double-float range (any precision)
  float* xdf = nullptr;      // DENSE double-float: x split into xh[ln_col], xl[ln_col]
  int* df_flag = nullptr;    // DENSE double-float: x out of range in this call
  double* pr_ctl = nullptr;  // PageRank: coefficients [0, 4) and flags (2 int) at [4]
  size_t pr_ctl_len = 0;
  // persistent-kernel control and reduction scratch
  unsigned* counter = nullptr;
  double* partials = nullptr;
  size_t partials_len = 0;
  double* result = nullptr;

  ~DeviceMatrix() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : {vals, (void*)idx0, (void*)idx1, (void*)blocks, (void*)x, (void*)y, (void*)t, (void*)pr_ctl,
                    (void*)counter, (void*)partials, (void*)result, (void*)coord, (void*)carry_row,
                    (void*)carry_val, svals, (void*)scols, (void*)sell_counter, (void*)colw, (void*)xdf,
                    (void*)df_flag, (void*)coo_carry, (void*)bx0, (void*)bx1, (void*)btele, (void*)bw,
                    (void*)bcoef})
      if (p) cudaFree(p);
    for (SellPlan& p : sell)
      for (void* q : {(void*)p.slice, (void*)p.lane, (void*)p.lane_len})
        if (q) cudaFree(q);
    for (cudaEvent_t e : xready)
      if (e) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (cudaEvent_t e : join_ev)
      if (e) cudaEventDestroy(e);
    for (cudaStream_t q : side)
      if (q) cudaStreamDestroy(q);
    if (xstream) cudaStreamDestroy(xstream);
    if (stream) cudaStreamDestroy(stream);
  }

  int vec(double** p, size_t* len, size_t need) {
    if (*len >= need && *p) return TBSLA_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *len = 0;
    int st = dalloc(p, std::max<size_t>(need, 1));
    if (st == TBSLA_OK) *len = need;
    return st;
  }
  int ctl(size_t nred_per_cta, int grid) {
    if (!counter) {
      int st = dalloc(&counter, 4);
      if (st) return st;
      TRY(cudaMemsetAsync(counter, 0, 4 * sizeof(unsigned), stream));
      st = dalloc(&result, 256);
      if (st) return st;
    }
    size_t need = std::max<size_t>(nred_per_cta * grid, (size_t)kSumBlocks * 32);
    return vec(&partials, &partials_len, need);
  }
};

void device_release(DeviceMatrix* d) { delete d; }

int dev_select(int device) {
  int st = check_device();
  if (st) return st;
  int n = 0;
  cudaGetDeviceCount(&n);
  if (device < 0 || device >= n) return TBSLA_ERR_INVALID_ARG;
  g_device = device;
  return status_of(cudaSetDevice(device));
}

int dev_host_alloc(void** p, size_t bytes) {
  int st = check_device();
  if (st) return st;
  cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return TBSLA_ERR_ALLOC;
  }
  return TBSLA_OK;
}

int dev_host_free(void* p) { return status_of(cudaFreeHost(p)); }

namespace {

// Stable counting sort of COO/SCOO triplets by row (device copy order).
void sort_by_row(const tbsla_matrix* m, long nnz, int rmin, int rmax, std::vector<int>& rows,
                 std::vector<int>& cols, std::vector<double>& vals) {
  const int* r = m->idx0.data();
  const int* c = m->idx1.data();
  const double* v = m->values.data();
  size_t span = (size_t)(rmax - rmin) + 1;
  std::vector<long> pos(span + 1, 0);
  for (long k = 0; k < nnz; k++) pos[r[k] - rmin + 1]++;
  for (size_t i = 0; i < span; i++) pos[i + 1] += pos[i];
  rows.resize(nnz);
  cols.resize(nnz);
  vals.resize(nnz);
  for (long k = 0; k < nnz; k++) {
    long p = pos[r[k] - rmin]++;
    rows[p] = r[k];
    cols[p] = c[k];
    vals[p] = v[k];
  }
}

// Host <-> device copies of the large arrays go straight from and to the
// caller's pageable memory: on a Grace host (GB300 on the C2C link) the
// driver moves pageable memory at the link's rate, measured at 195 GB/s
// either way for 1 GiB (5.5 ms),
// the same as from pinned memory, while staging through pinned buffers adds
// a host memcpy (1 GiB in 76 ms on one core).
int h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  return status_of(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
}

// FP64 host values -> device storage precision.
int upload_values(DeviceMatrix* d, const double* host, size_t n) {
  if (n == 0) return TBSLA_OK;
  void* dst = nullptr;
  cudaError_t e = cudaMalloc(&dst, n * prec_size(d->prec));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return TBSLA_ERR_ALLOC;
  }
  d->vals = dst;
  d->bytes += n * prec_size(d->prec);
  if (d->prec == TBSLA_F64) return h2d(dst, host, n * 8, d->stream);
  double* tmp = nullptr;
  int st = dalloc(&tmp, n);
  if (st) return st;
  if ((st = h2d(tmp, host, n * 8, d->stream))) return st;
  TRY(convert_values(tmp, dst, d->prec, (long)n, d->stream));
  TRY(cudaStreamSynchronize(d->stream));
  cudaFree(tmp);
  return TBSLA_OK;
}

int upload_ints(DeviceMatrix* d, int** dst, const int* host, size_t n) {
  int st = dalloc(dst, n);
  if (st) return st;
  d->bytes += n * 4;
  if (n == 0) return TBSLA_OK;
  return h2d(*dst, host, n * 4, d->stream);
}

template <class T>
int upload_array(DeviceMatrix* d, T** dst, const T* src, size_t n) {
  int st = dalloc(dst, std::max<size_t>(n, 1));
  if (st) return st;
  d->bytes += n * sizeof(T);
  if (n == 0) return TBSLA_OK;
  return status_of(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, d->stream));
}

SellArgs sell_args(const tbsla_matrix* m, const DeviceMatrix* d) {
  SellArgs a;
  a.vals = d->vals;
  a.prec = d->prec;
  a.rowptr = d->idx0;
  a.colidx = d->idx1;
  a.f_col = m->info.f_col;
  a.svals = d->svals;
  a.scols = d->scols;
  // automatic: 8 steps in flight (the column blocks keep x in L2, where
  // 16 costs more in occupancy than it gains in latency)
  a.unroll = m->sell_unroll > 0 ? m->sell_unroll : 8;
  a.nblocks = (int)d->sell.size();
  a.blocks = d->sell.data();
  a.parts = d->sell_parts;
  a.side = d->side.empty() ? nullptr : d->side.data();
  a.fork = d->fork_ev;
  a.join = d->join_ev.empty() ? nullptr : d->join_ev.data();
  return a;
}

// Sliced-ELL device layout of a CSR matrix: the columns are split into
// blocks of at most `sell_colblock` columns (0: 8,388,608, 64 MiB of x), the
// plans (row classes, slices, offsets) are made on the host
// from the per-block row lengths, and the slice arrays are filled on the
// device from the CSR copy.
int build_sell(const tbsla_matrix* m, DeviceMatrix* d) {
  using tbsla_impl::parallel_for;
  const tbsla_info& I = m->info;
  const int n = I.ln_row, nc = std::max(I.ln_col, 1);
  const long cb = m->sell_colblock > 0 ? m->sell_colblock : 8388608L;
  const int P = (int)std::max<long>(1, (nc + cb - 1) / cb);
  const int W = (int)(((long)nc + P - 1) / P);
  const int* rp = m->idx0.data();
  const int* ci = m->idx1.data();
  std::vector<int> lens((size_t)P * n, 0);
  if (P == 1) {
    for (int i = 0; i < n; i++) lens[i] = rp[i + 1] - rp[i];
  } else {
    parallel_for(n, [&](long b, long e) {
      for (long i = b; i < e; i++)
        for (int j = rp[i]; j < rp[i + 1]; j++) {
          const int k = std::min(P - 1, std::max(0, (ci[j] - I.f_col) / W));
          lens[(size_t)k * n + i]++;
        }
    });
  }
  // With column blocks, the last block is planned in kRowParts parts by
  // rows: after a part's launch its rows of y are final, so the host entry
  // point copies them out while the next part runs.
  const int R = P > 1 ? kRowParts : 1;
  // automatic thresholds: with several column blocks a row's entries are
  // spread over the blocks, so the per-block lengths the thresholds act on
  // are about halved; for FP64 values (whose kernel keeps the next group's
  // columns in flight) doubling the thresholds then pays: at n = 2^24 128 /
  // 128 is 2.4% faster than 64 / 64.  With one block, or FP32 / BF16 values,
  // 64 / 64 measured best.
  const int sthr = m->sell_short > 0 ? m->sell_short : (P > 1 && d->prec == TBSLA_F64 ? 128 : 64);
  const int lthr = m->sell_long > 0 ? m->sell_long : sthr;
  long steps = 0;
  d->sell.assign(P - 1 + R, SellPlan{});
  int st = TBSLA_OK;
  std::vector<int> part;
  for (int k = 0; k < P - 1 + R && !st; k++) {
    const int blk = std::min(k, P - 1), r = k - blk;
    const int* L = lens.data() + (size_t)blk * n;
    const int r0 = (int)((long)n * r / R), r1 = (int)((long)n * (r + 1) / R);
    if (R > 1 && blk == P - 1) {
      part.assign(n, 0);
      std::copy(L + r0, L + r1, part.begin() + r0);
      L = part.data();
    }
    SellPlan hp;
    sell_plan_build(L, n, sthr, lthr, m->sell_sigma, blk > 0, steps, &hp);
    hp.col_lo = blk * W;
    hp.col_hi = blk == P - 1 ? INT_MAX : (blk + 1) * W;
    hp.row_lo = blk == P - 1 ? r0 : 0;
    hp.row_hi = blk == P - 1 ? r1 : n;
    SellPlan& dp = d->sell[k];
    dp = hp;
    dp.slice = nullptr;
    dp.lane = nullptr;
    dp.lane_len = nullptr;
    st = upload_array(d, &dp.slice, hp.slice, (size_t)hp.nslices);
    if (!st) st = upload_array(d, &dp.lane, hp.lane, 32 * (size_t)hp.nslices);
    if (!st) st = upload_array(d, &dp.lane_len, hp.lane_len, 32 * (size_t)hp.nwide);
    if (!st) st = status_of(cudaStreamSynchronize(d->stream));  // host plan arrays are freed next
    sell_plan_free(&hp);
    steps += dp.sell_len / 32;
  }
  d->sell_parts = R;
  if (!st && R > 1 && d->side.empty()) {
    // part k on priority greatest + k (numerically larger = lower), at most
    // the least priority; the matrix stream has the greatest
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    d->side.assign(R - 1, nullptr);
    d->join_ev.assign(R - 1, nullptr);
    for (int k = 1; k < R && !st; k++) {
      const int prio = std::min(least, greatest + k);
      st = status_of(cudaStreamCreateWithPriority(&d->side[k - 1], cudaStreamNonBlocking, prio));
      if (!st) st = status_of(cudaEventCreateWithFlags(&d->join_ev[k - 1], cudaEventDisableTiming));
    }
    if (!st) st = status_of(cudaEventCreateWithFlags(&d->fork_ev, cudaEventDisableTiming));
  }
  if (st) return st;
  const size_t len = (size_t)steps * 32;
  if (cudaMalloc(&d->svals, std::max<size_t>(len, 1) * prec_size(d->prec)) != cudaSuccess) {
    cudaGetLastError();
    return TBSLA_ERR_ALLOC;
  }
  if ((st = dalloc(&d->scols, std::max<size_t>(len, 1))) || (st = dalloc(&d->sell_counter, kSellCounterWords)))
    return st;
  d->bytes += len * (prec_size(d->prec) + 4);
  TRY(cudaMemsetAsync(d->sell_counter, 0, kSellCounterWords * sizeof(unsigned), d->stream));
  TRY(sell_fill(sell_args(m, d), d->stream));
  return TBSLA_OK;
}

int build(const tbsla_matrix* m, DeviceMatrix* d) {
  const tbsla_info& I = m->info;
  // the matrix's own stream at the greatest priority, so that work forked
  // onto a least-priority side stream only fills its tails
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  TRY(cudaStreamCreateWithPriority(&d->stream, cudaStreamNonBlocking, greatest));
  switch (m->format) {
    case TBSLA_CSR: {
      if (I.nnz == 0) return TBSLA_OK;
      const int* rp = m->idx0.data();
      long end = rp[I.ln_row];
      d->nnz = end;
      int st = upload_ints(d, &d->idx0, rp, (size_t)I.ln_row + 1);
      if (!st) st = upload_ints(d, &d->idx1, m->idx1.data(), (size_t)end);
      if (!st) st = upload_values(d, m->values.data(), (size_t)end);
      if (st) return st;
      int tile = std::max(256, std::min(4096, m->csr_tile));
      d->items = tile <= 1024 ? 4 : tile <= 2048 ? 8 : 16;
      int* blocks = nullptr;
      csr_partition(rp, I.ln_row, 256 * d->items, &blocks, &d->nblocks);
      st = upload_ints(d, &d->blocks, blocks, (size_t)d->nblocks + 1);
      delete[] blocks;
      if (st) return st;
      // merge-path tiles and their carry scratch
      const long enz = end - rp[0];
      // automatic kernel: row blocks for small matrices, whose SpMV is one
      // short launch where the sliced-ELL kernel's chain of dependent loads
      // per slice shows (10^5 entries: 6.2 against 10.3 us); the sliced-ELL
      // kernel from 2^19 entries on (10^7: 48 against 107 us)
      d->algo = m->csr_algo >= 0 ? m->csr_algo : (enz < (1L << 19) ? TBSLA_CSR_ROWBLOCK : TBSLA_CSR_SELL);
      d->merge_items = m->merge_items;
      d->ntiles = merge_tiles(I.ln_row, enz, d->merge_items);
      if ((st = dalloc(&d->coord, (size_t)d->ntiles + 1)) || (st = dalloc(&d->carry_row, (size_t)d->ntiles)) ||
          (st = dalloc(&d->carry_val, (size_t)d->ntiles)))
        return st;
      d->bytes += (size_t)d->ntiles * 16 + 4;
      TRY(csr_merge_setup(d->idx0, I.ln_row, enz, d->merge_items, d->coord, d->stream));
      if (d->algo == 2) {
        st = build_sell(m, d);
        if (st) return st;
      }
      return status_of(cudaStreamSynchronize(d->stream));
    }
    case TBSLA_ELL: {
      if (I.nnz == 0 || I.max_col == 0) return TBSLA_OK;
      size_t n = (size_t)I.ln_row * I.max_col;
      double* tv = nullptr;
      int* tc = nullptr;
      int st = dalloc(&tv, n);
      if (!st) st = dalloc(&tc, n);
      if (!st) st = dalloc(&d->idx0, n);
      if (st) return st;
      void* vcm = nullptr;
      if (cudaMalloc(&vcm, n * prec_size(d->prec)) != cudaSuccess) {
        cudaGetLastError();
        return TBSLA_ERR_ALLOC;
      }
      d->vals = vcm;
      d->bytes += n * (4 + prec_size(d->prec));
      TRY(cudaMemcpyAsync(tv, m->values.data(), n * 8, cudaMemcpyHostToDevice, d->stream));
      TRY(cudaMemcpyAsync(tc, m->idx0.data(), n * 4, cudaMemcpyHostToDevice, d->stream));
      TRY(ell_transpose(tv, tc, vcm, d->prec, d->idx0, I.ln_row, I.max_col, d->stream));
      TRY(cudaStreamSynchronize(d->stream));
      cudaFree(tv);
      cudaFree(tc);
      return TBSLA_OK;
    }
    case TBSLA_COO:
    case TBSLA_SCOO: {
      long nnz = I.nnz;
      d->nnz = nnz;
      if (nnz == 0) return TBSLA_OK;
      const int* r = m->idx0.data();
      int rmin = r[0], rmax = r[0];
      for (long k = 1; k < nnz; k++) {
        rmin = std::min(rmin, r[k]);
        rmax = std::max(rmax, r[k]);
      }
      d->min_row = rmin;
      d->max_row = rmax;
      std::vector<int> rows, cols;
      std::vector<double> vals;
      sort_by_row(m, nnz, rmin, rmax, rows, cols, vals);
      int st = upload_ints(d, &d->idx0, rows.data(), nnz);
      if (!st) st = upload_ints(d, &d->idx1, cols.data(), nnz);
      if (!st) st = upload_values(d, vals.data(), nnz);
      const long nch = coo_chunks(nnz);
      if (!st) st = dalloc(&d->coo_carry, (size_t)(2 * nch + (nch + 1) / 2));
      if (!st) d->bytes += (size_t)nch * 20;
      if (!st) st = status_of(cudaStreamSynchronize(d->stream));
      return st;
    }
    case TBSLA_DENSE: {
      if (I.nnz == 0) return TBSLA_OK;
      const size_t n = (size_t)I.ln_row * I.ln_col;
      int st = upload_values(d, m->values.data(), n);
      if (!st) st = status_of(cudaStreamSynchronize(d->stream));
      if (st) return st;
      // the double-float GEMV when every value is in its range (FP64 values
      // split on load into two floats; FP32 / BF16 values exact in one)
      if ((st = dalloc(&d->df_flag, 1))) return st;
      bool ok = false;
      TRY(dense_values_df_range(d->vals, d->prec, n, d->df_flag, &ok, d->stream));
      if (ok) {
        if (cudaMalloc(&d->xdf, (size_t)I.ln_col * 2 * sizeof(float)) != cudaSuccess) {
          cudaGetLastError();
          return TBSLA_ERR_ALLOC;
        }
        d->bytes += (size_t)I.ln_col * 2 * sizeof(float) + 4;
        d->dense_df = true;
      }
      return TBSLA_OK;
    }
  }
  return TBSLA_ERR_INVALID_ARG;
}

size_t in_len(const tbsla_matrix* m) {
  return m->format == TBSLA_COO ? (size_t)m->info.n_col : (size_t)m->info.ln_col;
}
size_t out_len(const tbsla_matrix* m) {
  return m->format == TBSLA_COO ? (size_t)m->info.n_row : (size_t)m->info.ln_row;
}
bool accumulates(int format) {
  return format == TBSLA_COO || format == TBSLA_SCOO || format == TBSLA_DENSE;
}
// CSR / ELL / DENSE return without touching r when empty (MatrixCSR.cpp:210,
// MatrixELL.cpp:182, MatrixDENSE.cpp:78).
bool skips_empty(const tbsla_matrix* m) {
  const tbsla_info& I = m->info;
  switch (m->format) {
    case TBSLA_CSR: return I.nnz == 0;
    case TBSLA_ELL: return I.nnz == 0 || I.max_col == 0;
    case TBSLA_DENSE: return I.nnz == 0;
    case TBSLA_SCOO: return I.nnz == 0;
  }
  return false;
}

DeviceMatrix* ensure(const tbsla_matrix* m, int* st) {
  *st = TBSLA_OK;
  if (m->dev) {
    cudaSetDevice(m->dev->device);
    return m->dev;
  }
  *st = validate(m);  // bad arrays are reported before any device work
  if (*st) return nullptr;
  *st = check_device();
  if (*st) return nullptr;
  cudaSetDevice(g_device);
  auto* d = new DeviceMatrix();
  d->device = g_device;
  d->prec = m->precision;
  *st = build(m, d);
  if (*st) {
    delete d;
    return nullptr;
  }
  m->dev = d;
  return d;
}

CsrArgs csr_args(const tbsla_matrix* m, DeviceMatrix* d) {
  CsrArgs a;
  a.vals = d->vals;
  a.prec = d->prec;
  a.rowptr = d->idx0;
  a.colidx = d->idx1;
  a.blocks = d->blocks;
  a.nblocks = d->nblocks;
  a.f_col = m->info.f_col;
  a.items = d->items;
  return a;
}

// r (device) op= A v (device) on stream s, following the format's Ax semantics.
int ax_device(const tbsla_matrix* m, DeviceMatrix* d, double* r, const double* v, int vect_incr,
              cudaStream_t s) {
  const tbsla_info& I = m->info;
  if (skips_empty(m)) return TBSLA_OK;
  switch (m->format) {
    case TBSLA_CSR:
      if (d->algo == 1) return status_of(csr_spmv(csr_args(m, d), v, r, s));
      if (d->algo == 2) return status_of(sell_spmv(sell_args(m, d), v, r, d->sell_counter, s));
      {
        MergeArgs a{d->vals, d->prec, d->idx0, d->idx1, I.ln_row, d->nnz - m->idx0[0], I.f_col,
                    d->merge_items, d->coord, d->ntiles, d->carry_row, d->carry_val};
        return status_of(csr_merge_spmv(a, v, r, s));
      }
    case TBSLA_ELL:
      return status_of(ell_spmv(d->vals, d->prec, d->idx0, I.ln_row, I.max_col, I.f_col, v, r, s));
    case TBSLA_COO:
    case TBSLA_SCOO: {
      if (d->nnz == 0) return TBSLA_OK;
      bool scoo = m->format == TBSLA_SCOO;
      long off = (long)vect_incr - (scoo ? I.f_row : 0);
      long len = scoo ? I.ln_row : I.n_row;
      if (d->min_row + off < 0 || d->max_row + off >= len) return TBSLA_ERR_INVALID_ARG;
      const long nch = coo_chunks(d->nnz);
      CooCarry cc{d->coo_carry, d->coo_carry + nch, reinterpret_cast<int*>(d->coo_carry + 2 * nch)};
      return status_of(coo_spmv(d->vals, d->prec, d->idx0, d->idx1, d->nnz, (int)off,
                                scoo ? -I.f_col : 0, v, r, cc, s));
    }
    case TBSLA_DENSE:
      if (d->dense_df)
        return status_of(dense_gemv_df(d->vals, d->prec, I.ln_row, I.ln_col, v, d->xdf, d->df_flag, r, s));
      return status_of(dense_gemv(d->vals, d->prec, I.ln_row, I.ln_col, v, r, s));
  }
  return TBSLA_ERR_INVALID_ARG;
}

}  // namespace

int dev_upload(const tbsla_matrix* m) {
  int st;
  ensure(m, &st);
  return st;
}

int dev_bytes(const tbsla_matrix* m, size_t* bytes) {
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  *bytes = d->bytes;
  return TBSLA_OK;
}

int dev_launches(const tbsla_matrix* m, int* launches) {
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  int k = 0;
  if (skips_empty(m))
    k = 0;
  else if (m->format == TBSLA_COO || m->format == TBSLA_SCOO)
    k = d->nnz > 0;
  else if (m->format == TBSLA_DENSE)
    k = d->dense_df ? 2 : 1;  // double-float: the split of x, then the GEMV
  else if (m->format != TBSLA_CSR)
    k = 1;
  else if (d->algo == 2)
    for (const SellPlan& p : d->sell) k += p.nslices > 0;
  else
    k = d->algo == 1 ? 1 : 2;
  *launches = k;
  return TBSLA_OK;
}

namespace {
// Host entry point of the sliced-ELL kernel with column blocks.  The host
// link of a GB300 moves about 0.2 TB/s each way, so the copies are hidden
// under launches where the data allows:
// - x of block 0 goes over on the matrix stream, x of the later blocks on a
//   second stream, and each later launch waits only for its own part of x;
// - the last block runs in parts by rows; once a part's launch ends its
//   rows of y are final and go back on the second stream while the next
//   part runs.
// Results are those of dev_ax's plain path.
int ax_host_blocks(const tbsla_matrix* m, DeviceMatrix* d, double* r, const double* v, int vect_incr,
                   bool zero_first) {
  (void)vect_incr;  // CSR ignores it (MatrixCSR.cpp:209-233)
  const size_t nx = in_len(m);
  const int NP = (int)d->sell.size(), parts = d->sell_parts;
  cudaStream_t s = d->stream;
  if (!d->xstream) TRY(cudaStreamCreateWithFlags(&d->xstream, cudaStreamNonBlocking));
  // [0, NP): x of plan b has arrived; [NP, 2 NP): plan b launched; 2 NP: start
  while ((int)d->xready.size() < 2 * NP + 1) {
    cudaEvent_t e = nullptr;
    TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    d->xready.push_back(e);
  }
  cudaEvent_t* ev = d->xready.data();
  // the copies into d->x start after the matrix stream's earlier work
  TRY(cudaEventRecord(ev[2 * NP], s));
  TRY(cudaStreamWaitEvent(d->xstream, ev[2 * NP], 0));
  for (int b = 0; b < NP; b++) {
    const SellPlan& p = d->sell[b];
    if (b == 0 || p.col_lo != d->sell[b - 1].col_lo) {
      const size_t lo = std::min<size_t>((size_t)p.col_lo, nx);
      const size_t hi = p.col_hi == INT_MAX ? nx : std::min<size_t>((size_t)p.col_hi, nx);
      if (hi > lo)
        TRY(cudaMemcpyAsync(d->x + lo, v + lo, (hi - lo) * sizeof(double), cudaMemcpyHostToDevice,
                            b == 0 ? s : d->xstream));
    }
    if (b > 0) TRY(cudaEventRecord(ev[b], d->xstream));
  }
  if (zero_first) TRY(cudaMemsetAsync(d->y, 0, out_len(m) * sizeof(double), s));
  std::vector<cudaEvent_t> after(NP, nullptr);
  for (int b = NP - parts; b < NP - 1; b++) after[b] = ev[NP + b];
  SellArgs a = sell_args(m, d);
  a.ready = ev;
  a.after = after.data();
  TRY(sell_spmv(a, d->x, d->y, d->sell_counter, s));
  for (int b = NP - parts; b < NP; b++) {
    const SellPlan& p = d->sell[b];
    const size_t n = (size_t)(p.row_hi - p.row_lo);
    cudaStream_t cs = b < NP - 1 ? d->xstream : s;
    if (b < NP - 1) TRY(cudaStreamWaitEvent(cs, ev[NP + b], 0));
    if (n) TRY(cudaMemcpyAsync(r + p.row_lo, d->y + p.row_lo, n * sizeof(double), cudaMemcpyDeviceToHost, cs));
  }
  TRY(cudaEventRecord(ev[2 * NP], d->xstream));
  TRY(cudaStreamWaitEvent(s, ev[2 * NP], 0));
  return status_of(cudaStreamSynchronize(s));
}
}  // namespace

int dev_ax(const tbsla_matrix* m, double* r, const double* v, int vect_incr, bool zero_first,
           bool host, void* stream) {
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  if (!host) {
    cudaStream_t s = stream ? (cudaStream_t)stream : d->stream;
    if (zero_first) TRY(cudaMemsetAsync(r, 0, out_len(m) * sizeof(double), s));
    return ax_device(m, d, r, v, vect_incr, s);
  }
  if (!zero_first && skips_empty(m)) return TBSLA_OK;
  size_t nx = in_len(m), ny = out_len(m);
  if ((st = d->vec(&d->x, &d->x_len, nx)) || (st = d->vec(&d->y, &d->y_len, ny))) return st;
  cudaStream_t s = d->stream;
  if (m->format == TBSLA_CSR && d->algo == 2 && d->sell.size() > 1 && nx && !skips_empty(m))
    return ax_host_blocks(m, d, r, v, vect_incr, zero_first);
  if (nx) TRY(cudaMemcpyAsync(d->x, v, nx * sizeof(double), cudaMemcpyHostToDevice, s));
  if (zero_first) TRY(cudaMemsetAsync(d->y, 0, ny * sizeof(double), s));
  else if (accumulates(m->format) && ny) TRY(cudaMemcpyAsync(d->y, r, ny * sizeof(double), cudaMemcpyHostToDevice, s));
  st = ax_device(m, d, d->y, d->x, vect_incr, s);
  if (st) return st;
  if (ny) TRY(cudaMemcpyAsync(r, d->y, ny * sizeof(double), cudaMemcpyDeviceToHost, s));
  return status_of(cudaStreamSynchronize(s));
}

int dev_a_axpx(const tbsla_matrix* m, double* r, const double* v, int vect_incr) {
  // Matrix::a_axpx_, Matrix.cpp:5-14: r = spmv(v); r += v; return spmv(r).
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  size_t nx = in_len(m), ny = out_len(m);
  if (nx != ny) return TBSLA_ERR_INVALID_ARG;
  if ((st = d->vec(&d->x, &d->x_len, nx)) || (st = d->vec(&d->y, &d->y_len, ny)) ||
      (st = d->vec(&d->t, &d->t_len, ny)))
    return st;
  cudaStream_t s = d->stream;
  TRY(cudaMemcpyAsync(d->x, v, nx * 8, cudaMemcpyHostToDevice, s));
  TRY(cudaMemsetAsync(d->t, 0, ny * 8, s));
  if ((st = ax_device(m, d, d->t, d->x, vect_incr, s))) return st;
  TRY(vec_add(d->t, d->x, (long)nx, s));
  TRY(cudaMemsetAsync(d->y, 0, ny * 8, s));
  if ((st = ax_device(m, d, d->y, d->t, vect_incr, s))) return st;
  TRY(cudaMemcpyAsync(r, d->y, ny * 8, cudaMemcpyDeviceToHost, s));
  return status_of(cudaStreamSynchronize(s));
}

int dev_aaxpax(const tbsla_matrix* m, double* r, const double* v, double* buffer, int vect_incr,
               bool plus_x) {
  // Matrix::AAxpAx / AAxpAxpx, Matrix.cpp:16-31: Ax(buffer, v); buffer += v;
  // Ax(r, buffer) [; r += v].  Buffer and r keep the format's Ax semantics.
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  size_t nx = in_len(m), ny = out_len(m);
  if (nx != ny) return TBSLA_ERR_INVALID_ARG;
  if ((st = d->vec(&d->x, &d->x_len, nx)) || (st = d->vec(&d->y, &d->y_len, ny)) ||
      (st = d->vec(&d->t, &d->t_len, ny)))
    return st;
  cudaStream_t s = d->stream;
  TRY(cudaMemcpyAsync(d->x, v, nx * 8, cudaMemcpyHostToDevice, s));
  TRY(cudaMemcpyAsync(d->t, buffer, ny * 8, cudaMemcpyHostToDevice, s));
  TRY(cudaMemcpyAsync(d->y, r, ny * 8, cudaMemcpyHostToDevice, s));
  if ((st = ax_device(m, d, d->t, d->x, vect_incr, s))) return st;
  TRY(vec_add(d->t, d->x, (long)nx, s));
  if ((st = ax_device(m, d, d->y, d->t, vect_incr, s))) return st;
  if (plus_x) TRY(vec_add(d->y, d->x, (long)nx, s));
  TRY(cudaMemcpyAsync(buffer, d->t, ny * 8, cudaMemcpyDeviceToHost, s));
  TRY(cudaMemcpyAsync(r, d->y, ny * 8, cudaMemcpyDeviceToHost, s));
  return status_of(cudaStreamSynchronize(s));
}

// ---- column-stochastic preparation -----------------------------------------------

namespace {
// FP64 device copy of the CSR values (the device storage may be narrower).
int values64(const tbsla_matrix* m, DeviceMatrix* d, double** out, bool* owned) {
  long n = d->nnz;
  if (d->prec == TBSLA_F64) {
    *out = (double*)d->vals;
    *owned = false;
    return TBSLA_OK;
  }
  int st = dalloc(out, (size_t)n);
  if (st) return st;
  *owned = true;
  return status_of(cudaMemcpyAsync(*out, m->values.data(), n * 8, cudaMemcpyHostToDevice, d->stream));
}
}  // namespace

int dev_col_sums(tbsla_matrix* m, double* s, bool zero_first) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  if (I.nnz == 0) {  // MatrixCSR.cpp:1194-1197: nothing to add
    if (zero_first) std::memset(s, 0, sizeof(double) * I.ln_col);
    return TBSLA_OK;
  }
  size_t nc = I.ln_col;
  if ((st = d->vec(&d->t, &d->t_len, nc))) return st;
  cudaStream_t str = d->stream;
  if (zero_first) TRY(cudaMemsetAsync(d->t, 0, nc * 8, str));
  else TRY(cudaMemcpyAsync(d->t, s, nc * 8, cudaMemcpyHostToDevice, str));
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  TRY(csr_col_sums(v64, d->idx0, d->idx1, I.ln_row, I.f_col, d->t, str));
  TRY(cudaMemcpyAsync(s, d->t, nc * 8, cudaMemcpyDeviceToHost, str));
  TRY(cudaStreamSynchronize(str));
  if (owned) cudaFree(v64);
  return TBSLA_OK;
}

int dev_normalize_cols(tbsla_matrix* m, const double* s) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  if (I.nnz == 0) return TBSLA_OK;
  size_t nc = I.ln_col;
  if ((st = d->vec(&d->t, &d->t_len, nc))) return st;
  cudaStream_t str = d->stream;
  TRY(cudaMemcpyAsync(d->t, s, nc * 8, cudaMemcpyHostToDevice, str));
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  TRY(csr_normalize_cols(v64, d->idx0, d->idx1, I.ln_row, I.f_col, d->t, str));
  // keep the host arrays (the reference layout) in step with the device
  TRY(cudaMemcpyAsync(m->values.data(), v64, d->nnz * 8, cudaMemcpyDeviceToHost, str));
  if (owned) TRY(convert_values(v64, d->vals, d->prec, d->nnz, str));
  if (d->algo == 2 && d->svals) TRY(sell_fill(sell_args(m, d), str));  // slice copy
  d->colw_ok = false;
  TRY(cudaStreamSynchronize(str));
  if (owned) cudaFree(v64);
  return TBSLA_OK;
}

int dev_row_sums(const tbsla_matrix* m, double* s) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  if (I.ln_row <= 0) return TBSLA_OK;
  if (I.nnz == 0) {  // MatrixCSR.cpp:1152-1154: zeroed, nothing to add
    std::memset(s, 0, sizeof(double) * I.ln_row);
    return TBSLA_OK;
  }
  cudaStream_t str = d->stream;
  if ((st = d->vec(&d->t, &d->t_len, (size_t)I.ln_row))) return st;
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  st = status_of(csr_row_sums(v64, d->idx0, I.ln_row, d->t, str));
  if (!st) st = status_of(cudaMemcpyAsync(s, d->t, (size_t)I.ln_row * 8, cudaMemcpyDeviceToHost, str));
  if (!st) st = status_of(cudaStreamSynchronize(str));
  if (owned) cudaFree(v64);
  return st;
}

int dev_normalize_rows(tbsla_matrix* m, const double* s) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  if (I.nnz == 0 || I.ln_row <= 0) return TBSLA_OK;
  cudaStream_t str = d->stream;
  if ((st = d->vec(&d->t, &d->t_len, (size_t)I.ln_row))) return st;
  TRY(cudaMemcpyAsync(d->t, s, (size_t)I.ln_row * 8, cudaMemcpyHostToDevice, str));
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  TRY(csr_normalize_rows(v64, d->idx0, I.ln_row, d->t, str));
  // keep the host arrays (the reference layout) in step with the device
  TRY(cudaMemcpyAsync(m->values.data(), v64, d->nnz * 8, cudaMemcpyDeviceToHost, str));
  if (owned) TRY(convert_values(v64, d->vals, d->prec, d->nnz, str));
  if (d->algo == 2 && d->svals) TRY(sell_fill(sell_args(m, d), str));  // slice copy
  d->colw_ok = false;
  TRY(cudaStreamSynchronize(str));
  if (owned) cudaFree(v64);
  return TBSLA_OK;
}

int dev_make_stochastic(tbsla_matrix* m, double* s) {
  int st = dev_col_sums(m, s, true);
  if (st) return st;
  return dev_normalize_cols(m, s);
}

// ---- SpMM and the sparse-softmax helpers ---------------------------------------------

int dev_dense_multiply(const tbsla_matrix* m, const double* B, double* Cm, int cols) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  const size_t nb = (size_t)I.n_col * cols, nc = (size_t)I.n_row * cols;
  cudaStream_t s = d->stream;
  double *db = nullptr, *dc = nullptr;
  if ((st = dalloc(&db, std::max<size_t>(nb, 1))) || (st = dalloc(&dc, std::max<size_t>(nc, 1)))) {
    cudaFree(db);
    return st;
  }
  st = status_of(cudaMemcpyAsync(db, B, nb * 8, cudaMemcpyHostToDevice, s));
  if (!st) st = status_of(cudaMemsetAsync(dc, 0, nc * 8, s));  // MatrixCSR.cpp:1270
  if (!st) st = status_of(csr_dense_multiply(d->vals, d->prec, d->idx0, d->idx1, I.ln_row, db, cols, dc, s));
  if (!st) st = status_of(cudaMemcpyAsync(Cm, dc, nc * 8, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  cudaFree(db);
  cudaFree(dc);
  return st;
}

int dev_row_max_abs(const tbsla_matrix* m, double* max_abs) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  cudaStream_t s = d->stream;
  if ((st = d->vec(&d->t, &d->t_len, std::max<size_t>(I.ln_row, 1)))) return st;
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  st = status_of(csr_row_max_abs(v64, d->idx0, I.ln_row, d->t, s));
  if (!st) st = status_of(cudaMemcpyAsync(max_abs, d->t, (size_t)I.ln_row * 8, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  if (owned) cudaFree(v64);
  return st;
}

int dev_apply_exponential(tbsla_matrix* m, const double* max_abs, int base) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const tbsla_info& I = m->info;
  if (I.nnz == 0) return TBSLA_OK;
  cudaStream_t str = d->stream;
  if ((st = d->vec(&d->t, &d->t_len, std::max<size_t>(I.ln_row, 1)))) return st;
  if (max_abs) TRY(cudaMemcpyAsync(d->t, max_abs, (size_t)I.ln_row * 8, cudaMemcpyHostToDevice, str));
  double* v64;
  bool owned;
  if ((st = values64(m, d, &v64, &owned))) return st;
  TRY(csr_apply_exponential(v64, d->idx0, I.ln_row, max_abs ? d->t : nullptr, base, str));
  // keep the host arrays (the reference layout) in step with the device
  TRY(cudaMemcpyAsync(m->values.data(), v64, d->nnz * 8, cudaMemcpyDeviceToHost, str));
  if (owned) TRY(convert_values(v64, d->vals, d->prec, d->nnz, str));
  if (d->algo == 2 && d->svals) TRY(sell_fill(sell_args(m, d), str));
  d->colw_ok = false;
  TRY(cudaStreamSynchronize(str));
  if (owned) cudaFree(v64);
  return TBSLA_OK;
}

// ---- PageRank ------------------------------------------------------------------------

namespace {
// A value as the device stores it at precision `prec`, widened back: FP32
// rounds to nearest even; BF16 rounds the double's bits to 8 significant
// bits (ties to even), as the device narrowing does.
double stored_value(double v, int prec) {
  if (prec == TBSLA_F32) return (double)(float)v;
  if (prec != TBSLA_BF16) return v;
  uint64_t b;
  std::memcpy(&b, &v, 8);
  if ((b & 0x7ff0000000000000ull) != 0x7ff0000000000000ull) {
    b += (1ull << 44) - 1 + ((b >> 45) & 1);
    b &= ~((1ull << 45) - 1);
  }
  double r;
  std::memcpy(&r, &b, 8);
  float f = (float)r;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u &= 0xffff0000u;
  std::memcpy(&f, &u, 4);
  return f;
}

// PageRank column weights w_j = sum of column j of A as stored (0 for a
// dangling node), summed on the host in entry order -- deterministic, and
// the order the oracle uses -- then kept on the device until the values
// change.
int column_weights(const tbsla_matrix* m, DeviceMatrix* d) {
  if (d->colw_ok) return TBSLA_OK;
  const tbsla_info& I = m->info;
  std::vector<double> w(I.ln_col, 0.0);
  const int* rp = m->idx0.data();
  const int* ci = m->idx1.data();
  for (int i = 0; i < I.ln_row; i++)
    for (int j = rp[i]; j < rp[i + 1]; j++) w[ci[j] - I.f_col] += stored_value(m->values[j], d->prec);
  if (!d->colw) {
    int st = dalloc(&d->colw, std::max<size_t>(I.ln_col, 1));
    if (st) return st;
  }
  int st = status_of(cudaMemcpyAsync(d->colw, w.data(), w.size() * 8, cudaMemcpyHostToDevice, d->stream));
  if (!st) st = status_of(cudaStreamSynchronize(d->stream));
  if (st) return st;
  // S and M of x_0 = 1/n, summed in index order as the oracle forms them
  const double x_init = 1.0 / I.ln_row;
  double S = 0, M = 0;
  for (int i = 0; i < I.ln_row; i++) {
    S += x_init;
    M += w[i] * x_init;
  }
  d->colw_s0 = S;
  d->colw_m0 = M;
  d->colw_ok = true;
  return TBSLA_OK;
}

// Scale and teleport weight of step 0 from x_0 = 1/n.
void initial_coefficients(const DeviceMatrix* d, double beta, double c[2]) {
  c[0] = 1.0 / d->colw_s0;
  c[1] = 1.0 - beta * d->colw_m0 * c[0];
}
}  // namespace

int dev_page_rank(tbsla_matrix* m, double beta, double eps, int max_it, double* result,
                  int* iterations, double* error) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  const tbsla_info& I = m->info;
  if (I.n_row != I.n_col || I.ln_row != I.n_row || I.f_col != 0 || max_it < 0)
    return TBSLA_ERR_INVALID_ARG;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const int n = I.n_row;
  cudaStream_t s = d->stream;
  // the sliced-ELL kernel (FP64-efficient on skewed rows) with a separate
  // epilogue pass, or the row-block kernel with the epilogue fused
  const bool sell = d->algo == 2;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device);
  int grid = sell ? 8 * sms : (I.nnz > 0 ? csr_pagerank_grid(d->items, d->prec) : 1);
  // the two iterates and the control words stay with the device copy, so
  // repeated solves allocate (and synchronise on frees) nothing
  if ((st = d->vec(&d->x, &d->x_len, (size_t)n)) || (st = d->vec(&d->y, &d->y_len, (size_t)n)) ||
      (st = d->vec(&d->pr_ctl, &d->pr_ctl_len, 8)) || (st = d->ctl(3, grid)) || (st = column_weights(m, d)) ||
      (sell && (st = d->vec(&d->t, &d->t_len, (size_t)n))))
    return st;
  double *x0 = d->x, *x1 = d->y, *coef = d->pr_ctl;
  int* flags = reinterpret_cast<int*>(d->pr_ctl + 4);  // [0] done, [1] iterations
  const double x_init = 1.0 / n;
  double c0[2];
  initial_coefficients(d, beta, c0);
  vec_fill(x0, x_init, n, s);
  cudaMemcpyAsync(coef, c0, 16, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
  CsrArgs a = csr_args(m, d);
  // one column block: the epilogue runs inside the sliced-ELL kernel
  // (sell_pagerank); several: a separate pass over t = A x
  SellArgs sa{};
  bool fused = false;
  if (sell && I.nnz > 0) {
    sa = sell_args(m, d);
    fused = sa.nblocks == 1 && sa.parts == 1 && m->pr_fused;
  }
  PageRankArgs p{beta, (double)n, eps, nullptr, d->colw, coef, coef + 2, flags, flags + 1};
  Ctl ctl{d->counter, d->partials, d->result};
  int launched = 0, hflags[2] = {0, 0};
  const int chunk = 8;
  while (launched < max_it && !hflags[0]) {
    int k = std::min(chunk, max_it - launched);
    for (int j = 0; j < k; j++, launched++) {
      const bool even = (launched % 2) == 0;
      p.coef_in = coef + (even ? 0 : 2);
      p.coef_out = coef + (even ? 2 : 0);
      cudaError_t e = cudaErrorInvalidValue;
      if (I.nnz > 0 && sell && fused) {
        e = sell_pagerank(sa, even ? x0 : x1, even ? x1 : x0, p, ctl, s);
      } else if (I.nnz > 0 && sell) {
        e = sell_spmv(sa, even ? x0 : x1, d->t, d->sell_counter, s, flags);
        if (e == cudaSuccess) e = pagerank_epilogue(d->t, even ? x0 : x1, even ? x1 : x0, n, p, ctl, grid, s);
      } else if (I.nnz > 0) {
        e = csr_pagerank_step(a, even ? x0 : x1, even ? x1 : x0, p, ctl, grid, s);
      }
      if (e != cudaSuccess) return I.nnz > 0 ? status_of(e) : TBSLA_ERR_BAD_MATRIX;
    }
    if (cudaMemcpyAsync(hflags, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return TBSLA_ERR_CUDA;
  }
  const int iters = hflags[1];
  double* fin = (iters % 2 == 1) ? x1 : x0;
  // final normalisation x /= sum(x) (Matrix.cpp:149-171)
  double* sum = d->result + 8;
  st = status_of(mat_colsum(fin, n, 1, d->partials, sum, s));
  if (!st) st = status_of(mat_scale_cols(fin, n, 1, sum, s));
  if (!st) st = status_of(cudaMemcpyAsync(result, fin, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  double herr = 0;
  if (!st) st = status_of(cudaMemcpyAsync(&herr, d->result, 8, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  if (st) return st;
  if (iterations) *iterations = iters;
  if (error) *error = herr;
  return hflags[0] ? TBSLA_OK : TBSLA_ERR_NOT_CONVERGED;
}

int dev_page_rank_batched(tbsla_matrix* m, int nvec, const double* tele, double beta, double eps,
                          int max_it, double* result, int* iterations) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  const tbsla_info& I = m->info;
  if (I.n_row != I.n_col || I.ln_row != I.n_row || I.f_col != 0 || nvec < 1 || nvec > 32 ||
      max_it < 0 || I.nnz == 0)
    return TBSLA_ERR_INVALID_ARG;
  int st;
  DeviceMatrix* d = ensure(m, &st);
  if (st) return st;
  const int n = I.n_row;
  const size_t nn = (size_t)n * nvec;
  cudaStream_t s = d->stream;
  // FP32 / BF16 values: the iterates, teleport vectors and column sums in
  // double-float (float pairs, the bytes of FP64), products and sums on the
  // FP32 pipe; FP64 values keep FP64 arithmetic
  const bool df = d->prec != TBSLA_F64;
  const int gather = m->pr_gather == 16 ? 16 : 8;
  // the row-block stream form keeps X row offsets in 32 bits
  const int stream = m->pr_stream && (long)I.n_col * nvec <= 0x7fffffffL ? 1 : 0;
  int grid = csr_pagerank_batched_grid(d->prec, gather, stream);
  // the buffers stay with the device copy: repeated solves allocate (and
  // synchronise on frees) nothing
  if ((st = d->vec(&d->bx0, &d->bx0_len, nn)) || (st = d->vec(&d->bx1, &d->bx1_len, nn)) ||
      (st = d->vec(&d->btele, &d->btele_len, nn)) || (st = d->vec(&d->bcoef, &d->bcoef_len, 130)) ||
      (st = d->ctl(96, grid)) || (st = column_weights(m, d)) || (df && (st = d->vec(&d->bw, &d->bw_len, (size_t)n))))
    return st;
  double *X0 = d->bx0, *X1 = d->bx1, *T = d->btele, *coef = d->bcoef, *W = d->bw;
  int* flags = reinterpret_cast<int*>(d->bcoef + 128);
  const double x_init = 1.0 / n;
  double cc[2];
  initial_coefficients(d, beta, cc);
  std::vector<double> c0(64, 0.0);
  for (int k = 0; k < nvec; k++) {
    c0[k] = cc[0];
    c0[32 + k] = cc[1];
  }
  vec_fill(X0, x_init, (long)nn, s);
  if ((st = h2d(T, tele, nn * 8, s))) return st;
  cudaMemcpyAsync(coef, c0.data(), 64 * 8, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
  if (df && ((st = status_of(f64_to_df(X0, X0, (long)nn, s))) || (st = status_of(f64_to_df(T, T, (long)nn, s))) ||
             (st = status_of(f64_to_df(d->colw, W, (long)n, s)))))
    return st;
  CsrArgs a = csr_args(m, d);
  PageRankArgs p{beta, (double)n, eps, nullptr, d->colw, coef, coef + 64, flags, flags + 1};
  Ctl ctl{d->counter, d->partials, d->result};
  int launched = 0, hflags[2] = {0, 0};
  while (launched < max_it && !hflags[0]) {
    int k = std::min(8, max_it - launched);
    for (int j = 0; j < k; j++, launched++) {
      const bool even = (launched % 2) == 0;
      p.coef_in = coef + (even ? 0 : 64);
      p.coef_out = coef + (even ? 64 : 0);
      cudaError_t e = df ? csr_pagerank_batched_df_step(a, nvec, even ? X0 : X1, even ? X1 : X0, T, W, p, ctl, grid,
                                                        gather, stream, s)
                         : csr_pagerank_batched_step(a, n, nvec, even ? X0 : X1, even ? X1 : X0, T, p, ctl, grid, s);
      if (e != cudaSuccess) return status_of(e);
    }
    if (cudaMemcpyAsync(hflags, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return TBSLA_ERR_CUDA;
  }
  const int iters = hflags[1];
  double* fin = (iters % 2 == 1) ? X1 : X0;
  if (df) {  // to FP64 in the other iterate's storage
    double* out = (iters % 2 == 1) ? X0 : X1;
    if ((st = status_of(df_to_f64(fin, out, (long)nn, s)))) return st;
    fin = out;
  }
  double* sums = d->result + 128;
  st = status_of(mat_colsum(fin, n, nvec, d->partials, sums, s));
  if (!st) st = status_of(mat_scale_cols(fin, n, nvec, sums, s));
  if (!st) st = status_of(cudaMemcpyAsync(result, fin, nn * 8, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  if (st) return st;
  if (iterations) *iterations = iters;
  return hflags[0] ? TBSLA_OK : TBSLA_ERR_NOT_CONVERGED;
}

// ---- autotuner ------------------------------------------------------------------------

namespace {
void apply_tuning(tbsla_matrix* m, const tbsla_tuning& t) {
  const bool rebuild = m->csr_algo != t.algorithm ||
                       (t.algorithm == TBSLA_CSR_MERGE && m->merge_items != t.items) ||
                       (t.algorithm == TBSLA_CSR_ROWBLOCK && m->csr_tile != t.tile) ||
                       (t.algorithm == TBSLA_CSR_SELL &&
                        (m->sell_short != t.short_thr || m->sell_long != t.long_thr ||
                         m->sell_sigma != t.sigma || m->sell_colblock != t.col_block));
  if (rebuild) m->invalidate();
  m->csr_algo = t.algorithm;
  if (t.algorithm == TBSLA_CSR_MERGE) m->merge_items = t.items;
  if (t.algorithm == TBSLA_CSR_ROWBLOCK) m->csr_tile = t.tile;
  if (t.algorithm == TBSLA_CSR_SELL) {
    m->sell_unroll = t.items;
    m->sell_short = t.short_thr;
    m->sell_long = t.long_thr;
    m->sell_sigma = t.sigma;
    m->sell_colblock = t.col_block;
  }
}
}  // namespace

int dev_autotune(tbsla_matrix* m, int reps, tbsla_tuning* best, tbsla_tuning* trials, int max_trials,
                 int* ntrials) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  const tbsla_info& I = m->info;
  reps = std::max(reps, 1);
  // candidates, grouped so that consecutive ones share a device layout
  std::vector<tbsla_tuning> cand;
  std::vector<int> blocks = {0};
  if (I.ln_col > 8388608) blocks.push_back(I.ln_col);  // one block
  if (I.ln_col > 4194304) blocks.push_back(4194304);
  const int thr[4][2] = {{64, 64}, {128, 128}, {32, 32}, {64, 255}};
  for (int cb : blocks)
    for (auto& t : thr)
      for (int u : {8, 16}) cand.push_back({TBSLA_CSR_SELL, u, t[0], t[1], 16384, cb, m->csr_tile, 0.0});
  const tbsla_tuning keep{m->csr_algo, m->csr_algo == TBSLA_CSR_MERGE ? m->merge_items : m->sell_unroll,
                          m->sell_short, m->sell_long, m->sell_sigma, m->sell_colblock, m->csr_tile, 0.0};
  cand.push_back({TBSLA_CSR_MERGE, 8, keep.short_thr, keep.long_thr, keep.sigma, keep.col_block, keep.tile, 0});
  cand.push_back({TBSLA_CSR_ROWBLOCK, 0, keep.short_thr, keep.long_thr, keep.sigma, keep.col_block, 2048, 0});
  double *x = nullptr, *y = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = TBSLA_OK;
  if ((st = check_device())) return st;
  cudaSetDevice(g_device);
  if ((st = dalloc(&x, std::max(I.ln_col, 1))) || (st = dalloc(&y, std::max(I.ln_row, 1)))) {
    cudaFree(x);
    return st;
  }
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int bestk = -1, count = 0;
  for (size_t k = 0; k < cand.size() && !st; k++) {
    apply_tuning(m, cand[k]);
    DeviceMatrix* d = ensure(m, &st);
    if (st) break;
    cudaStream_t s = d->stream;
    if ((st = status_of(vec_fill(x, 1.0, I.ln_col, s)))) break;
    if ((st = ax_device(m, d, y, x, 0, s))) break;  // warm-up
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && !st; r++) st = ax_device(m, d, y, x, 0, s);
    cudaEventRecord(e1, s);
    if (!st) st = status_of(cudaEventSynchronize(e1));
    if (st) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cand[k].ms = ms / reps;
    if (trials && count < max_trials) trials[count] = cand[k];
    count++;
    if (bestk < 0 || cand[k].ms < cand[bestk].ms) bestk = (int)k;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  if (ntrials) *ntrials = std::min(count, std::max(max_trials, 0));
  if (st || bestk < 0) {
    apply_tuning(m, keep);
    return st ? st : TBSLA_ERR_CUDA;
  }
  apply_tuning(m, cand[bestk]);
  if (best) *best = cand[bestk];
  ensure(m, &st);
  return st;
}

int dev_coo_order(const int* row, const int* col, long n, int n_row, int n_col, long* start, long* perm) {
  int st = check_device();
  if (st) return st;
  if (n >= (1L << 31) - 1) return TBSLA_ERR_INVALID_ARG;
  cudaSetDevice(g_device);
  cudaStream_t s = nullptr;
  int *drow = nullptr, *dcol = nullptr, *p0 = nullptr, *p1 = nullptr;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  unsigned *cnt = nullptr, *scr = nullptr;
  const size_t ns = std::max<size_t>(1, std::max(radix_scratch(n), scan_scratch((long)n_row + 1)));
  auto cleanup = [&]() {
    for (void* q : {(void*)drow, (void*)dcol, (void*)p0, (void*)p1, (void*)k0, (void*)k1, (void*)cnt, (void*)scr})
      if (q) cudaFree(q);
    if (s) cudaStreamDestroy(s);
  };
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || (st = dalloc(&drow, n)) ||
      (st = dalloc(&dcol, n)) || (st = dalloc(&p0, n)) || (st = dalloc(&p1, n)) || (st = dalloc(&k0, n)) ||
      (st = dalloc(&k1, n)) || (st = dalloc(&cnt, (size_t)n_row + 1)) || (st = dalloc(&scr, ns))) {
    cleanup();
    return st ? st : TBSLA_ERR_CUDA;
  }
  int alt = 0;
  std::vector<int> hp(n);
  std::vector<unsigned> hs((size_t)n_row + 1);
  st = n ? status_of(cudaMemcpyAsync(drow, row, n * 4, cudaMemcpyHostToDevice, s)) : TBSLA_OK;
  if (!st && n) st = status_of(cudaMemcpyAsync(dcol, col, n * 4, cudaMemcpyHostToDevice, s));
  if (!st) st = status_of(coo_order(drow, dcol, n, n_row, n_col, k0, k1, p0, p1, cnt, scr, &alt, s));
  if (!st && n) st = status_of(cudaMemcpyAsync(hp.data(), alt ? p1 : p0, n * 4, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaMemcpyAsync(hs.data(), cnt, hs.size() * 4, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  cleanup();
  if (st) return st;
  for (size_t i = 0; i < hs.size(); i++) start[i] = hs[i];
  for (long k = 0; k < n; k++) perm[k] = hp[k];
  return TBSLA_OK;
}

int dev_coo_to_dense(const int* row, const int* col, const double* val, long n, int ln_row, int ln_col,
                     double* dense_host) {
  int st = check_device();
  if (st) return st;
  if (n >= (1L << 31) - 1) return TBSLA_ERR_INVALID_ARG;
  cudaSetDevice(g_device);
  const size_t cells = (size_t)ln_row * ln_col;
  cudaStream_t s = nullptr;
  int *drow = nullptr, *dcol = nullptr, *p0 = nullptr, *p1 = nullptr;
  double *dval = nullptr, *dense = nullptr;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  unsigned *cnt = nullptr, *scr = nullptr;
  const size_t ns = std::max<size_t>(1, std::max(radix_scratch(n), scan_scratch((long)ln_row + 1)));
  auto cleanup = [&]() {
    for (void* q : {(void*)drow, (void*)dcol, (void*)p0, (void*)p1, (void*)dval, (void*)dense, (void*)k0, (void*)k1,
                    (void*)cnt, (void*)scr})
      if (q) cudaFree(q);
    if (s) cudaStreamDestroy(s);
  };
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || (st = dalloc(&drow, n)) ||
      (st = dalloc(&dcol, n)) || (st = dalloc(&dval, n)) || (st = dalloc(&p0, n)) || (st = dalloc(&p1, n)) ||
      (st = dalloc(&k0, n)) || (st = dalloc(&k1, n)) || (st = dalloc(&cnt, (size_t)ln_row + 1)) ||
      (st = dalloc(&scr, ns)) || (st = dalloc(&dense, cells))) {
    cleanup();
    return st ? st : TBSLA_ERR_CUDA;
  }
  int alt = 0;
  if (cells) st = status_of(cudaMemsetAsync(dense, 0, cells * 8, s));
  if (!st && n) st = h2d(drow, row, n * 4, s);
  if (!st && n) st = h2d(dcol, col, n * 4, s);
  if (!st && n) st = h2d(dval, val, n * 8, s);
  if (!st) st = status_of(coo_order(drow, dcol, n, ln_row, ln_col, k0, k1, p0, p1, cnt, scr, &alt, s));
  if (!st) st = status_of(coo_dense_scatter(alt ? p1 : p0, drow, dcol, dval, n, ln_col, dense, s));
  if (!st && cells) st = status_of(cudaMemcpyAsync(dense_host, dense, cells * 8, cudaMemcpyDeviceToHost, s));
  if (!st) st = status_of(cudaStreamSynchronize(s));
  cleanup();
  return st;
}

int dev_ready(int* device) {
  const int st = check_device();
  if (!st) *device = g_device;
  return st;
}

long dev_noalloc_max_items() { return csr_merge_noalloc_max_items(); }

int dev_csr_ax_noalloc(int n_row, long nnz, int f_col, const int* rowptr, const int* colidx,
                       const double* values, const double* v, double* r, void* stream) {
  return status_of(csr_merge_spmv_noalloc(values, rowptr, colidx, n_row, nnz, f_col, v, r,
                                          static_cast<cudaStream_t>(stream)));
}

}  // namespace tbsla_impl
