// COO / SCOO SpMV as a segmented reduction over a row-sorted device copy.
//
// Replaces tbsla::cpp::MatrixCOO::Ax (src/cpp/matrix/MatrixCOO.cpp:135-142)
// and tbsla::cpp::MatrixSCOO::Ax (src/cpp/matrix/MatrixSCOO.cpp:154-164):
// r[row + row_off] += values * v[col + col_off] for every triplet, where the
// reference uses an OpenMP array reduction (one private copy of r per
// thread).  Here the triplets are stably sorted by row once at upload, and
// each CTA reduces a tile of 256*ITEMS consecutive triplets by key:
//  1. striped, coalesced loads of (row, col, value); products with the
//     gathered x staged in shared memory;
//  2. each thread scans its ITEMS consecutive products; a block-wide
//     segmented scan of the per-thread (has-segment-start, tail-sum) pairs
//     gives every thread the partial sum carried into its range;
//  3. each segment is written once by the thread that sees its end: a
//     segment that starts and ends inside the tile owns its row outright
//     (plain read-modify-write), while the tile's first and last segments may
//     continue in the neighbouring tiles and are added with FP64 atomics.
// No per-thread copy of r, no atomics except at tile boundaries.
#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;

template <class V, int ITEMS>
__global__ void __launch_bounds__(NT) k_coo(const int* __restrict__ rows, const int* __restrict__ cols,
                                           const V* __restrict__ vals, long nnz, int row_off,
                                           int col_off, const double* __restrict__ x,
                                           double* __restrict__ y) {
  constexpr int TILE = NT * ITEMS;
  __shared__ double s_prod[TILE];
  __shared__ int s_row[TILE];
  __shared__ int s_wf[NT / kWarp];
  __shared__ double s_wv[NT / kWarp];
  __shared__ int s_first_head;
  const int tid = threadIdx.x, lane = tid % kWarp, warp = tid / kWarp;
  const long base = (long)blockIdx.x * TILE;
  const int cnt = (int)min((long)TILE, nnz - base);
  const uint64_t pol = policy_evict_first();
  if (tid == 0) s_first_head = TILE;

  int r[ITEMS], c[ITEMS];
  V v[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    const int i = k * NT + tid;
    if (i < cnt) {
      r[k] = ld_stream(rows + base + i, pol);
      c[k] = ld_stream(cols + base + i, pol);
      v[k] = ld_stream(vals + base + i, pol);
    }
  }
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    const int i = k * NT + tid;
    if (i < cnt) {
      s_row[i] = r[k];
      s_prod[i] = mul_rn(widen(v[k]), ld_gather(x + c[k] + col_off));
    }
  }
  __syncthreads();

  // Per-thread pair (f, t): f = a segment starts inside [lo, hi) (at k > 0),
  // t = sum of the products after the last such start (all of them if none).
  const int lo = tid * ITEMS, hi = min(lo + ITEMS, cnt);
  int f = 0;
  double t = 0;
  for (int k = lo; k < hi; k++) {
    if (k > 0 && s_row[k] != s_row[k - 1]) {
      if (!f) atomicMin(&s_first_head, k);
      f = 1;
      t = 0;
    }
    t = add_rn(t, s_prod[k]);
  }
  // Inclusive segmented scan over the warp: (fa,ta) then (fb,tb) combine to
  // (fa|fb, fb ? tb : ta + tb).
  int fi = f;
  double ti = t;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const int fu = __shfl_up_sync(0xffffffffu, fi, o);
    const double tu = __shfl_up_sync(0xffffffffu, ti, o);
    if (lane >= o) {
      ti = fi ? ti : add_rn(tu, ti);
      fi |= fu;
    }
  }
  if (lane == kWarp - 1) {
    s_wf[warp] = fi;
    s_wv[warp] = ti;
  }
  const int fl = __shfl_up_sync(0xffffffffu, fi, 1);
  const double tl = __shfl_up_sync(0xffffffffu, ti, 1);
  __syncthreads();
  // Exclusive prefix for this thread: earlier warps, then earlier lanes.
  double carry = 0;
  for (int w = 0; w < warp; w++) carry = s_wf[w] ? s_wv[w] : add_rn(carry, s_wv[w]);
  if (lane > 0) carry = fl ? tl : add_rn(carry, tl);
  const int first_head = s_first_head;

  double acc = carry;
  for (int k = lo; k < hi; k++) {
    if (k > 0 && s_row[k] != s_row[k - 1]) {
      double* dst = y + (s_row[k - 1] + row_off);
      if (k == first_head) atomicAdd(dst, acc);  // first segment: may span the previous tile
      else *dst = add_rn(*dst, acc);              // interior segment: owned by this CTA
      acc = 0;
    }
    acc = add_rn(acc, s_prod[k]);
  }
  if (lo < cnt && hi == cnt) atomicAdd(y + (s_row[cnt - 1] + row_off), acc);  // last segment
}

template <class V>
cudaError_t launch(const void* vals, const int* rows, const int* cols, long nnz, int row_off,
                   int col_off, const double* x, double* y, cudaStream_t s) {
  constexpr int ITEMS = 8;
  const long tiles = (nnz + NT * ITEMS - 1) / (NT * ITEMS);
  k_coo<V, ITEMS><<<(unsigned)tiles, NT, 0, s>>>(rows, cols, static_cast<const V*>(vals), nnz,
                                                 row_off, col_off, x, y);
  return cudaGetLastError();
}

}  // namespace

cudaError_t coo_spmv(const void* vals, int prec, const int* rows, const int* cols, long nnz,
                     int row_off, int col_off, const double* x, double* y, cudaStream_t s) {
  if (nnz <= 0) return cudaSuccess;
  switch (prec) {
    case kF64: return launch<double>(vals, rows, cols, nnz, row_off, col_off, x, y, s);
    case kF32: return launch<float>(vals, rows, cols, nnz, row_off, col_off, x, y, s);
    case kBF16: return launch<__nv_bfloat16>(vals, rows, cols, nnz, row_off, col_off, x, y, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tbsla_gpu
