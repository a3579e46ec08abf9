// Shared device code of the CSR traversal: the row-block worker used by the
// SpMV, PageRank and CG kernels, and the persistent-kernel helpers (dynamic
// block fetch, per-CTA partial sums reduced by the last CTA to finish).
#pragma once

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {
namespace csr {

constexpr int NT = 256;

template <class V>
__device__ __forceinline__ double row_dot_cta(const V* vals, const int* colidx, int s, int e,
                                              const double* x, int f_col, uint64_t pol) {
  double acc = 0;
  int j = s + (int)threadIdx.x;
  for (; j + 3 * NT < e; j += 4 * NT) {
    int c0 = ld_stream(colidx + j, pol), c1 = ld_stream(colidx + j + NT, pol);
    int c2 = ld_stream(colidx + j + 2 * NT, pol), c3 = ld_stream(colidx + j + 3 * NT, pol);
    V v0 = ld_stream(vals + j, pol), v1 = ld_stream(vals + j + NT, pol);
    V v2 = ld_stream(vals + j + 2 * NT, pol), v3 = ld_stream(vals + j + 3 * NT, pol);
    double x0 = ld_gather(x + c0 - f_col), x1 = ld_gather(x + c1 - f_col);
    double x2 = ld_gather(x + c2 - f_col), x3 = ld_gather(x + c3 - f_col);
    acc = fma_rn(widen(v0), x0, acc);
    acc = fma_rn(widen(v1), x1, acc);
    acc = fma_rn(widen(v2), x2, acc);
    acc = fma_rn(widen(v3), x3, acc);
  }
  for (; j < e; j += NT)
    acc = fma_rn(widen(ld_stream(vals + j, pol)), ld_gather(x + ld_stream(colidx + j, pol) - f_col), acc);
  return acc;
}

struct Smem {
  int rp[NT + 1];
  double red[NT / kWarp];
  int blk;
  int flag;
};

// Dynamic shared memory of a stream block: x[NT*ITEMS] doubles then
// values[NT*ITEMS] in the storage precision.
template <class V, int ITEMS>
constexpr size_t stage_bytes() { return (size_t)NT * ITEMS * (sizeof(double) + sizeof(V)); }

// One block of the partition; epi.emit(row, sum, red) per row.
template <class V, int ITEMS, class Epi>
__device__ __forceinline__ void csr_block(const CsrArgs& a, int b, const double* x, const Epi& epi,
                                          double* red, unsigned char* stage, Smem& sm, uint64_t pol) {
  const V* vals = static_cast<const V*>(a.vals);
  double* s_x = reinterpret_cast<double*>(stage);
  V* s_v = reinterpret_cast<V*>(stage + (size_t)NT * ITEMS * sizeof(double));
  const int r0 = a.blocks[b], r1 = a.blocks[b + 1];
  const int nrows = r1 - r0;
  const int tid = threadIdx.x;
  if (nrows == 1) {
    const int s = a.rowptr[r0], e = a.rowptr[r0 + 1];
    double acc = row_dot_cta(vals, a.colidx, s, e, x, a.f_col, pol);
    acc = block_sum<NT>(acc, sm.red);
    if (tid == 0) epi.emit(r0, acc, red);
    return;
  }
  for (int i = tid; i <= nrows; i += NT) sm.rp[i] = ld_stream(a.rowptr + r0 + i, pol);
  __syncthreads();
  const int s = sm.rp[0];
  const int cnt = sm.rp[nrows] - s;
  int cidx[ITEMS];
  V vv[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    const int i = k * NT + tid;
    if (i < cnt) {
      cidx[k] = ld_stream(a.colidx + s + i, pol);
      vv[k] = ld_stream(vals + s + i, pol);
    }
  }
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    const int i = k * NT + tid;
    if (i < cnt) {
      s_x[i] = ld_gather(x + cidx[k] - a.f_col);
      s_v[i] = vv[k];
    }
  }
  __syncthreads();
  const int G = nrows <= 8 ? 32 : nrows <= 16 ? 16 : nrows <= 32 ? 8 : nrows <= 64 ? 4 : nrows <= 128 ? 2 : 1;
  const int g = tid / G, lane = tid % G;
  double acc = 0;
  if (g < nrows) {
    const int lo = sm.rp[g] - s, hi = sm.rp[g + 1] - s;
    for (int j = lo + lane; j < hi; j += G) acc = fma_rn(widen(s_v[j]), s_x[j], acc);
  }
  for (int o = G >> 1; o > 0; o >>= 1) acc = add_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
  if (g < nrows && lane == 0) epi.emit(r0 + g, acc, red);
  __syncthreads();  // stage / rp reused by the next block
}


// ---- persistent variant with reductions --------------------------------------

__device__ __forceinline__ int next_block(Ctl ctl, Smem& sm) {
  __syncthreads();
  if (threadIdx.x == 0) sm.blk = (int)atomicAdd(ctl.counter, 1u);
  __syncthreads();
  return sm.blk;
}

// Per-CTA partials, then the last CTA to finish sums them in CTA order
// (deterministic), calls epi.finalize(result) and resets the counters.
template <int NRED, class Fin>
__device__ __forceinline__ void reduce_and_finish(Ctl ctl, double* red, Smem& sm, Fin fin) {
  for (int k = 0; k < NRED; k++) {
    double v = block_sum<NT>(red[k], sm.red);
    if (threadIdx.x == 0) ctl.partials[(size_t)blockIdx.x * NRED + k] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(ctl.counter + 1, 1u);
    sm.flag = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!sm.flag) return;
  __threadfence();
  for (int k = 0; k < NRED; k++) {
    double acc = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT)
      acc = add_rn(acc, __ldcg(ctl.partials + (size_t)i * NRED + k));
    acc = block_sum<NT>(acc, sm.red);
    if (threadIdx.x == 0) ctl.result[k] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    fin(ctl.result);
    ctl.counter[0] = 0;
    ctl.counter[1] = 0;
    __threadfence();
  }
}


// ---- PageRank step epilogue ----------------------------------------------------

// x is used normalised by its sum S (scale s = 1/S, carried from the
// previous step): y_i = (beta * (A x)_i) * s + c_i with c_i = t / n or
// t * tele_i and t = 1 - (beta * M) * s, M = sum_j w_j x_j (w = column sums
// of A as stored), so that y sums to 1.  Reductions: L1 change, sum y and
// sum w y (the next step's S and M).
// Four FP64 operations per row (GB300's FP64 pipe is the epilogue's
// bound): yn = fma(beta s, sum, c), the change fma(-x, s, yn), S += yn,
// M = fma(w, yn, M).
struct EpiPageRank {
  double* y;
  const double* x;
  const double* colw;
  const double* tele;
  double bs, s, t, c_uniform;  // bs = beta * s, formed once per thread
  __device__ __forceinline__ void emit(int row, double sum, double* red) const {
    const double c = tele ? mul_rn(t, tele[row]) : c_uniform;
    const double yn = fma_rn(bs, sum, c);
    red[0] = add_rn(red[0], fabs(fma_rn(-x[row], s, yn)));
    red[1] = add_rn(red[1], yn);
    red[2] = fma_rn(colw[row], yn, red[2]);
    y[row] = yn;
  }
};

// t of the next step from its S (r1) and M (r2): 1 - (beta * M) / S.
__device__ __forceinline__ double teleport_weight(double beta, double s1, double m) {
  return add_rn(1.0, -mul_rn(mul_rn(beta, m), s1));
}

// The last CTA's step: the next coefficients from the sums r = {L1 change,
// S, M}, the iteration count and the done flag.
struct PageRankFinish {
  double beta, eps;
  double* coef_out;
  int* done;
  int* iters;
  static __device__ __forceinline__ PageRankFinish of(const PageRankArgs& p) {
    return PageRankFinish{p.beta, p.eps, p.coef_out, p.done, p.iters};
  }
  __device__ __forceinline__ void operator()(const double* r) const {
    const double s1 = 1.0 / r[1];
    coef_out[0] = s1;
    coef_out[1] = teleport_weight(beta, s1, r[2]);
    *iters += 1;
    if (r[0] < eps) *done = 1;
  }
};

}  // namespace csr
}  // namespace tbsla_gpu
