// CSR SpMV, row-block adaptive (the CSR-Stream / CSR-Vector scheme of
// Greathouse & Daga, SC'14, built here for sm_103a), and the PageRank steps
// that reuse its traversal with a fused epilogue.
//
// Replaces tbsla::cpp::MatrixCSR::Ax (src/cpp/matrix/MatrixCSR.cpp:209-233):
// y_i = sum_j values_j * v[colidx_j - f_col], overwriting y.
//
// Layout: the reference CSR arrays as they are (int32 rowptr / colidx, values
// in the storage precision) plus a row-block partition built once per
// matrix (csr_partition).  A block is either
//  - a run of <= 256 consecutive rows holding <= 256*ITEMS entries
//    ("stream" block): the CTA reads the block's values and column indices
//    with coalesced loads, gathers x, stages (value, x) pairs in shared
//    memory, then sums each row with a group of G lanes, G = the largest
//    power of two with G * rows <= 256 (capped at 32), one fused
//    multiply-add per entry in entry order;
//  - one row longer than 256*ITEMS ("vector" block): the whole CTA strides
//    over it and reduces.
// GB300's FP64 pipe is narrow, so the kernel spends exactly one FP64
// instruction (DFMA) per entry, widens FP32 / BF16 values on the integer
// pipes, and keeps reductions to one add per row-group lane.
// Matrix values, indices and row pointers are read once, through the
// non-allocating read-only path with an L2 evict-first policy; x is gathered
// through L1 so that it owns L2.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "df.cuh"
#include "csr_block.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

using namespace csr;

struct EpiStore {
  double* y;
  __device__ __forceinline__ void emit(int row, double s, double*) const { y[row] = s; }
};

template <class V, int ITEMS>
__global__ void __launch_bounds__(NT) k_csr_spmv(CsrArgs a, const double* __restrict__ x,
                                                double* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ Smem sm;
  const uint64_t pol = policy_evict_first();
  EpiStore epi{y};
  csr_block<V, ITEMS>(a, blockIdx.x, x, epi, nullptr, stage, sm, pol);
}

template <class V, int ITEMS>
__global__ void __launch_bounds__(NT) k_csr_pagerank(CsrArgs a, const double* __restrict__ x,
                                                    double* __restrict__ y, PageRankArgs p,
                                                    Ctl ctl) {
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ Smem sm;
  if (*(volatile int*)p.done) return;  // converged in an earlier launch: no-op
  const uint64_t pol = policy_evict_first();
  const double s = p.coef_in[0], t = p.coef_in[1];
  EpiPageRank epi{y, x, p.colw, p.tele, mul_rn(p.beta, s), s, t, t / p.n_nodes};
  double red[3] = {0, 0, 0};
  for (int b = next_block(ctl, sm); b < a.nblocks; b = next_block(ctl, sm))
    csr_block<V, ITEMS>(a, b, x, epi, red, stage, sm, pol);
  reduce_and_finish<3>(ctl, red, sm, PageRankFinish::of(p));
}

// PageRank epilogue over a separately computed t = A x: the EpiPageRank
// step of every row (grid-stride, fixed grid, so the reduction order is
// fixed), then the deterministic CTA reduction and the next coefficients.
__global__ void __launch_bounds__(NT) k_pagerank_epilogue(const double* __restrict__ t,
                                                         const double* __restrict__ x, double* __restrict__ y,
                                                         long n, PageRankArgs p, Ctl ctl) {
  __shared__ Smem sm;
  if (*(volatile int*)p.done) return;
  const double s = p.coef_in[0], tw = p.coef_in[1];
  EpiPageRank epi{y, x, p.colw, p.tele, mul_rn(p.beta, s), s, tw, tw / p.n_nodes};
  double red[3] = {0, 0, 0};
  for (long i = blockIdx.x * (long)NT + threadIdx.x; i < n; i += (long)gridDim.x * NT)
    epi.emit((int)i, t[i], red);
  reduce_and_finish<3>(ctl, red, sm, PageRankFinish::of(p));
}

// The end of a batched PageRank step: per-column CTA sums over warps (in
// warp order), per-CTA partials, and the last CTA's sums in CTA order
// (deterministic), coefficients of the next step and the done flag.
__device__ __forceinline__ void batched_finish(double err, double sum, double dsum, int nvec,
                                               double (*s_red)[3 * kWarp], Smem& sm, const PageRankArgs& p,
                                               Ctl ctl) {
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  s_red[warp][lane] = err;
  s_red[warp][kWarp + lane] = sum;
  s_red[warp][2 * kWarp + lane] = dsum;
  __syncthreads();
  if (threadIdx.x < 3 * kWarp) {
    double acc = 0;
    for (int w = 0; w < NT / kWarp; w++) acc = add_rn(acc, s_red[w][threadIdx.x]);
    ctl.partials[(size_t)blockIdx.x * 3 * kWarp + threadIdx.x] = acc;
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
  if (threadIdx.x < 3 * kWarp) {
    double acc = 0;
#pragma unroll 8
    for (int i = 0; i < (int)gridDim.x; i++)
      acc = add_rn(acc, __ldcg(ctl.partials + (size_t)i * 3 * kWarp + threadIdx.x));
    s_red[0][threadIdx.x] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int all = 1;
    for (int k = 0; k < nvec; k++) {
      const double e = s_red[0][k], sm_ = s_red[0][kWarp + k], d = s_red[0][2 * kWarp + k];
      ctl.result[k] = e;
      ctl.result[nvec + k] = sm_;
      ctl.result[2 * nvec + k] = d;
      const double s1 = 1.0 / sm_;
      p.coef_out[k] = s1;
      p.coef_out[kWarp + k] = teleport_weight(p.beta, s1, d);
      if (!(e < p.eps)) all = 0;
    }
    *p.iters += 1;
    if (all) *p.done = 1;
    ctl.counter[0] = 0;
    ctl.counter[1] = 0;
    __threadfence();
  }
}


__device__ __forceinline__ DF df_ld(const float2* p) {
  const float2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ float as_f32(float v) { return v; }
__device__ __forceinline__ float as_f32(__nv_bfloat16 v) { return __bfloat162float(v); }

// The batched step in double-float, for FP32 / BF16 values (exact in one
// float): X, Y, T and the column sums w are stored as float pairs; each
// lane sums its row's products a_ij X[j, k] in entry order as a compensated
// dot product (Dot2: about twice FP32 precision), and the epilogue forms the
// single-vector epilogue's quantities (y = beta s acc + t T, |y - x s|, y,
// w y) in the same arithmetic: the difference y - x s, which cancels as the
// iteration converges, with the full double-float addition, the sums of
// terms of one sign (y's two terms, the three running sums) with the
// same-sign one.  The CTA and grid reductions run in FP64 (batched_finish).
template <class V, int GB>
__global__ void __launch_bounds__(NT) k_csr_pagerank_batched_df(CsrArgs a, int nvec, const float2* __restrict__ X,
                                                               float2* __restrict__ Y, const float2* __restrict__ T,
                                                               const float2* __restrict__ W, PageRankArgs p,
                                                               Ctl ctl) {
  __shared__ Smem sm;
  __shared__ double s_red[NT / kWarp][3 * kWarp];
  if (*(volatile int*)p.done) return;
  const uint64_t pol = policy_evict_first();
  const V* vals = static_cast<const V*>(a.vals);
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const bool active = lane < nvec;
  const double scd = active ? p.coef_in[lane] : 0.0;
  const DF sc = df_of(scd), tc = df_of(active ? p.coef_in[kWarp + lane] : 0.0), bsc = df_of(mul_rn(p.beta, scd));
  DF err{0.f, 0.f}, sum{0.f, 0.f}, dsum{0.f, 0.f};
  for (int b = next_block(ctl, sm); b < a.nblocks; b = next_block(ctl, sm)) {
    const int r0 = a.blocks[b], r1 = a.blocks[b + 1];
    for (int row = r0 + warp; row < r1; row += NT / kWarp) {
      const int s = a.rowptr[row], e = a.rowptr[row + 1];
      float as = 0.f, ac = 0.f;  // compensated sum of the row's products
      for (int base = s; base < e; base += kWarp) {
        const int j = base + lane;
        int c = 0;
        float v = 0.f;
        if (j < e) {
          c = ld_stream(a.colidx + j, pol);
          v = as_f32(ld_stream(vals + j, pol));
        }
        const int m = min(kWarp, e - base);
        // GB entries' gathers of X in flight (8 or 16, a tuning choice),
        // then their products added in entry order; a short tail runs as a
        // masked batch (a dead slot adds 0 * 0, which leaves s and c as they
        // are), so a row of a few entries waits for one gather latency, not
        // one per entry
        for (int t = 0; t < m; t += GB) {
          DF xv[GB];
          float vv[GB];
#pragma unroll
          for (int u = 0; u < GB; u++) {
            const bool live = t + u < m;
            const int ct = __shfl_sync(0xffffffffu, c, (t + u) & (kWarp - 1));
            const float vu = __shfl_sync(0xffffffffu, v, (t + u) & (kWarp - 1));
            vv[u] = live ? vu : 0.f;
            xv[u] = (active && live) ? df_ld(X + (size_t)(ct - a.f_col) * nvec + lane) : DF{0.f, 0.f};
          }
#pragma unroll
          for (int u = 0; u < GB; u++) dot2_step(as, ac, vv[u], xv[u]);
        }
      }
      if (active) {
        const DF acc = fast_two_sum(as, ac);
        const size_t o = (size_t)row * nvec + lane;
        const DF yn = df_add_same_sign(df_mul(bsc, acc), df_mul(tc, df_ld(T + o)));
        DF dx = df_add(yn, df_neg(df_mul(df_ld(X + o), sc)));
        if (dx.h < 0) dx = df_neg(dx);
        err = df_add_same_sign(err, dx);
        sum = df_add_same_sign(sum, yn);
        dsum = df_add_same_sign(dsum, df_mul(df_ld(W + row), yn));
        Y[o] = make_float2(yn.h, yn.l);
      }
    }
  }
  batched_finish(df_val(err), df_val(sum), df_val(dsum), nvec, s_red, sm, p, ctl);
}

// The same step in an entry-stream form: each warp claims whole row blocks
// of the partition and walks the block's entries as one stream, GB X-row
// gathers in flight whatever the row boundaries, finishing each row (the
// same epilogue) where its last entry is added.  Each row's products are
// added in entry order with the same Dot2 steps as above, so Y is the same
// bit for bit; only the order in which rows enter the norms' partial sums
// differs.  Rows of a few entries (most rows of a power-law graph) then
// share one gather latency instead of paying one each, and a row's
// epilogue operands (T, X, w) are loaded when the previous row finishes.
//
// The kernel is bound by instruction issue and by how many warps hide the
// gathers, so the per-entry work is kept small: each lane turns its entry
// of a 32-entry chunk into (X row offset, value) once and leaves it in
// shared memory, where every lane reads it back with one broadcast load
// (the offset is 32-bit: the host takes this form only when
// n_col * nvec < 2^31); a batch of GB whole entries that no row ends inside
// runs without the per-entry row-end test; and the register cap keeps four
// CTAs (32 warps) on an SM for GB = 8 (two for GB = 16).
template <class V, int GB>
__global__ void __launch_bounds__(NT, GB <= 8 ? 4 : 2)
    k_csr_pagerank_batched_dfs(CsrArgs a, int nvec, const float2* __restrict__ X, float2* __restrict__ Y,
                               const float2* __restrict__ T, const float2* __restrict__ W, PageRankArgs p, Ctl ctl) {
  __shared__ Smem sm;
  __shared__ double s_red[NT / kWarp][3 * kWarp];
  __shared__ int2 s_ent[NT / kWarp][kWarp];  // per warp: its chunk's (X row offset, value bits)
  if (*(volatile int*)p.done) return;
  constexpr unsigned full = 0xffffffffu;
  const uint64_t pol = policy_evict_first();
  const V* vals = static_cast<const V*>(a.vals);
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const bool active = lane < nvec;
  const float2* __restrict__ Xl = X + lane;
  int2* const ent = s_ent[warp];
  const double scd = active ? p.coef_in[lane] : 0.0;
  const DF sc = df_of(scd), tc = df_of(active ? p.coef_in[kWarp + lane] : 0.0), bsc = df_of(mul_rn(p.beta, scd));
  DF err{0.f, 0.f}, sum{0.f, 0.f}, dsum{0.f, 0.f};
  for (;;) {
    int b = 0;
    if (lane == 0) b = (int)atomicAdd(ctl.counter, 1u);
    b = __shfl_sync(full, b, 0);
    if (b >= a.nblocks) break;
    const int r0 = a.blocks[b], r1 = a.blocks[b + 1];
    const int s0 = a.rowptr[r0], e0 = a.rowptr[r1];
    // ends of rows [rw, rw + 32): lane k holds rowptr[rw + k + 1]
    int rw = r0;
    int rpw = rw + 1 + lane <= r1 ? a.rowptr[rw + 1 + lane] : 0;
    int row = r0;
    int row_end = __shfl_sync(full, rpw, 0);
    DF tn{0.f, 0.f}, xn{0.f, 0.f}, wn;
    auto load_ops = [&](int r) {
      if (active) {
        const size_t o = (size_t)r * nvec + lane;
        tn = df_ld(T + o);
        xn = df_ld(X + o);
      }
      wn = df_ld(W + r);
    };
    load_ops(row);
    float as = 0.f, ac = 0.f;
    // the epilogue of `row`, then the next row's end and operands
    auto finish = [&]() {
      if (active) {
        const DF acc = fast_two_sum(as, ac);
        const DF yn = df_add_same_sign(df_mul(bsc, acc), df_mul(tc, tn));
        DF dx = df_add(yn, df_neg(df_mul(xn, sc)));
        if (dx.h < 0) dx = df_neg(dx);
        err = df_add_same_sign(err, dx);
        sum = df_add_same_sign(sum, yn);
        dsum = df_add_same_sign(dsum, df_mul(wn, yn));
        Y[(size_t)row * nvec + lane] = make_float2(yn.h, yn.l);
      }
      as = ac = 0.f;
      row++;
      if (row < r1) {
        if (row - rw >= kWarp) {
          rw += kWarp;
          rpw = rw + 1 + lane <= r1 ? a.rowptr[rw + 1 + lane] : 0;
        }
        row_end = __shfl_sync(full, rpw, row - rw);
        load_ops(row);
      }
    };
    for (int base = s0; base < e0; base += kWarp) {
      const int j = base + lane;
      int xo = 0;
      float v = 0.f;
      if (j < e0) {
        xo = (ld_stream(a.colidx + j, pol) - a.f_col) * nvec;
        v = as_f32(ld_stream(vals + j, pol));
      }
      __syncwarp();
      ent[lane] = make_int2(xo, __float_as_int(v));
      __syncwarp();
      const int m = min(kWarp, e0 - base);
      int t = 0;
      for (; t + GB <= m; t += GB) {
        DF xv[GB];
        float vv[GB];
#pragma unroll
        for (int u = 0; u < GB; u++) {
          const int2 ev = ent[t + u];
          vv[u] = __int_as_float(ev.y);
          xv[u] = active ? df_ld(Xl + ev.x) : DF{0.f, 0.f};
        }
        if (base + t + GB <= row_end) {  // no row ends inside the batch
#pragma unroll
          for (int u = 0; u < GB; u++) dot2_step(as, ac, vv[u], xv[u]);
        } else {
#pragma unroll
          for (int u = 0; u < GB; u++) {
            while (base + t + u >= row_end) finish();  // rows ending before this entry (empty ones too)
            dot2_step(as, ac, vv[u], xv[u]);
          }
        }
      }
      if (t < m) {  // the block's last, partial batch (its dead slots neither load nor add)
        DF xv[GB];
        float vv[GB];
#pragma unroll
        for (int u = 0; u < GB; u++) {
          const bool live = t + u < m;
          const int2 ev = ent[(t + u) & (kWarp - 1)];
          vv[u] = live ? __int_as_float(ev.y) : 0.f;
          xv[u] = (active && live) ? df_ld(Xl + ev.x) : DF{0.f, 0.f};
        }
#pragma unroll
        for (int u = 0; u < GB; u++) {
          if (t + u < m) {
            while (base + t + u >= row_end) finish();
            dot2_step(as, ac, vv[u], xv[u]);
          }
        }
      }
    }
    while (row < r1) finish();  // the last row with entries and the empty rows after it
  }
  batched_finish(df_val(err), df_val(sum), df_val(dsum), nvec, s_red, sm, p, ctl);
}

__global__ void k_f64_to_df(const double* src, float2* dst, long n) {  // may run in place
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const DF v = df_of(src[i]);
    dst[i] = make_float2(v.h, v.l);
  }
}

__global__ void k_df_to_f64(const float2* src, double* dst, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float2 v = src[i];
    dst[i] = (double)v.x + (double)v.y;
  }
}

// Batched personalised PageRank: lanes of a warp are the nvec vectors; the
// warps of the CTA take the rows of a block in turn.  Each lane sums its
// row's products in entry order.
template <class V>
__global__ void __launch_bounds__(NT) k_csr_pagerank_batched(CsrArgs a, int nvec,
                                                            const double* __restrict__ X,
                                                            double* __restrict__ Y,
                                                            const double* __restrict__ T,
                                                            PageRankArgs p, Ctl ctl) {
  __shared__ Smem sm;
  __shared__ double s_red[NT / kWarp][3 * kWarp];
  if (*(volatile int*)p.done) return;
  const uint64_t pol = policy_evict_first();
  const V* vals = static_cast<const V*>(a.vals);
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const bool active = lane < nvec;
  const double sc = active ? p.coef_in[lane] : 0.0;        // 1 / sum of the vector
  const double tc = active ? p.coef_in[kWarp + lane] : 0.0;  // teleport weight
  const double bsc = mul_rn(p.beta, sc);
  double err = 0, sum = 0, dsum = 0;  // L1 change, sum y, sum w y
  for (int b = next_block(ctl, sm); b < a.nblocks; b = next_block(ctl, sm)) {
    const int r0 = a.blocks[b], r1 = a.blocks[b + 1];
    for (int row = r0 + warp; row < r1; row += NT / kWarp) {
      const int s = a.rowptr[row], e = a.rowptr[row + 1];
      double acc = 0;
      for (int base = s; base < e; base += kWarp) {
        const int j = base + lane;
        int c = 0;
        double v = 0;
        if (j < e) {
          c = ld_stream(a.colidx + j, pol);
          v = widen(ld_stream(vals + j, pol));
        }
        const int m = min(kWarp, e - base);
        int t = 0;
        // 8 entries' gathers of X in flight, then their multiply-adds in
        // entry order
        for (; t + 8 <= m; t += 8) {
          double xv[8], vv[8];
#pragma unroll
          for (int u = 0; u < 8; u++) {
            const int ct = __shfl_sync(0xffffffffu, c, t + u);
            vv[u] = __shfl_sync(0xffffffffu, v, t + u);
            xv[u] = active ? ld_gather(X + (size_t)(ct - a.f_col) * nvec + lane) : 0.0;
          }
#pragma unroll
          for (int u = 0; u < 8; u++) acc = fma_rn(vv[u], xv[u], acc);
        }
        for (; t < m; t++) {
          const int ct = __shfl_sync(0xffffffffu, c, t);
          const double vt = __shfl_sync(0xffffffffu, v, t);
          if (active) acc = fma_rn(vt, ld_gather(X + (size_t)(ct - a.f_col) * nvec + lane), acc);
        }
      }
      if (active) {
        const size_t o = (size_t)row * nvec + lane;
        // the single-vector epilogue's operations (EpiPageRank), per column:
        // six FP64 instructions per row and vector
        const double yn = fma_rn(bsc, acc, mul_rn(tc, T[o]));
        err = add_rn(err, fabs(fma_rn(-X[o], sc, yn)));
        sum = add_rn(sum, yn);
        dsum = fma_rn(p.colw[row], yn, dsum);
        Y[o] = yn;
      }
    }
  }
  batched_finish(err, sum, dsum, nvec, s_red, sm, p, ctl);
}

template <class V, int ITEMS>
cudaError_t launch_spmv(const CsrArgs& a, const double* x, double* y, cudaStream_t s) {
  constexpr size_t smem = stage_bytes<V, ITEMS>();
  cudaError_t ready = smem_opt_in<k_csr_spmv<V, ITEMS>>(smem);
  if (ready != cudaSuccess) return ready;
  k_csr_spmv<V, ITEMS><<<a.nblocks, NT, smem, s>>>(a, x, y);
  return cudaGetLastError();
}

template <class V>
cudaError_t spmv_items(const CsrArgs& a, const double* x, double* y, cudaStream_t s) {
  switch (a.items) {
    case 4: return launch_spmv<V, 4>(a, x, y, s);
    case 8: return launch_spmv<V, 8>(a, x, y, s);
    case 16: return launch_spmv<V, 16>(a, x, y, s);
  }
  return cudaErrorInvalidValue;
}

template <class V, int ITEMS>
cudaError_t launch_pr(const CsrArgs& a, const double* x, double* y, const PageRankArgs& p, Ctl c,
                      int grid, cudaStream_t s) {
  constexpr size_t smem = stage_bytes<V, ITEMS>();
  cudaError_t ready = smem_opt_in<k_csr_pagerank<V, ITEMS>>(smem);
  if (ready != cudaSuccess) return ready;
  k_csr_pagerank<V, ITEMS><<<grid, NT, smem, s>>>(a, x, y, p, c);
  return cudaGetLastError();
}

template <class V>
cudaError_t pr_items(const CsrArgs& a, const double* x, double* y, const PageRankArgs& p, Ctl c,
                     int grid, cudaStream_t s) {
  switch (a.items) {
    case 4: return launch_pr<V, 4>(a, x, y, p, c, grid, s);
    case 8: return launch_pr<V, 8>(a, x, y, p, c, grid, s);
    case 16: return launch_pr<V, 16>(a, x, y, p, c, grid, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

void csr_partition(const int* rowptr, int n_row, int tile, int** out, int* nblocks) {
  std::vector<int> b;
  b.reserve((size_t)n_row / 64 + 16);
  b.push_back(0);
  int r = 0;
  while (r < n_row) {
    const long len = (long)rowptr[r + 1] - rowptr[r];
    if (len > tile) {
      r++;
      b.push_back(r);
      continue;
    }
    const int start = r;
    const long base = rowptr[r];
    while (r < n_row && r - start < NT && (long)rowptr[r + 1] - base <= tile) r++;
    b.push_back(r);
  }
  *nblocks = (int)b.size() - 1;
  *out = new int[b.size()];
  std::copy(b.begin(), b.end(), *out);
}

namespace {
template <auto Kernel>
int resident_grid(size_t smem = 0) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (smem) smem_opt_in<Kernel>(smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, Kernel, NT, smem);
  return std::max(1, sms * std::max(1, per));
}
}  // namespace

int csr_pagerank_grid(int items, int prec) {
  switch (prec * 100 + items) {
    case kF64 * 100 + 4: return resident_grid<k_csr_pagerank<double, 4>>(stage_bytes<double, 4>());
    case kF64 * 100 + 8: return resident_grid<k_csr_pagerank<double, 8>>(stage_bytes<double, 8>());
    case kF64 * 100 + 16: return resident_grid<k_csr_pagerank<double, 16>>(stage_bytes<double, 16>());
    case kF32 * 100 + 4: return resident_grid<k_csr_pagerank<float, 4>>(stage_bytes<float, 4>());
    case kF32 * 100 + 8: return resident_grid<k_csr_pagerank<float, 8>>(stage_bytes<float, 8>());
    case kF32 * 100 + 16: return resident_grid<k_csr_pagerank<float, 16>>(stage_bytes<float, 16>());
    case kBF16 * 100 + 4: return resident_grid<k_csr_pagerank<__nv_bfloat16, 4>>(stage_bytes<__nv_bfloat16, 4>());
    case kBF16 * 100 + 8: return resident_grid<k_csr_pagerank<__nv_bfloat16, 8>>(stage_bytes<__nv_bfloat16, 8>());
    case kBF16 * 100 + 16: return resident_grid<k_csr_pagerank<__nv_bfloat16, 16>>(stage_bytes<__nv_bfloat16, 16>());
  }
  return 152;
}

int csr_pagerank_batched_grid(int prec, int gather, int stream) {
  const bool wide = gather == 16;
  switch (prec) {
    case kF64: return resident_grid<k_csr_pagerank_batched<double>>();
    case kF32:
      if (stream)
        return wide ? resident_grid<k_csr_pagerank_batched_dfs<float, 16>>()
                    : resident_grid<k_csr_pagerank_batched_dfs<float, 8>>();
      return wide ? resident_grid<k_csr_pagerank_batched_df<float, 16>>()
                  : resident_grid<k_csr_pagerank_batched_df<float, 8>>();
    case kBF16:
      if (stream)
        return wide ? resident_grid<k_csr_pagerank_batched_dfs<__nv_bfloat16, 16>>()
                    : resident_grid<k_csr_pagerank_batched_dfs<__nv_bfloat16, 8>>();
      return wide ? resident_grid<k_csr_pagerank_batched_df<__nv_bfloat16, 16>>()
                  : resident_grid<k_csr_pagerank_batched_df<__nv_bfloat16, 8>>();
  }
  return 152;
}

cudaError_t csr_pagerank_batched_df_step(const CsrArgs& a, int nvec, const void* X, void* Y, const void* T,
                                         const void* W, const PageRankArgs& p, Ctl ctl, int grid, int gather,
                                         int stream, cudaStream_t s) {
  if (nvec < 1 || nvec > kWarp) return cudaErrorInvalidValue;
  const float2 *x = static_cast<const float2*>(X), *t = static_cast<const float2*>(T),
               *w = static_cast<const float2*>(W);
  float2* y = static_cast<float2*>(Y);
  const bool wide = gather == 16;
  switch (a.prec * 4 + (wide ? 2 : 0) + (stream ? 1 : 0)) {
    case kF32 * 4 + 0: k_csr_pagerank_batched_df<float, 8><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl); break;
    case kF32 * 4 + 1: k_csr_pagerank_batched_dfs<float, 8><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl); break;
    case kF32 * 4 + 2: k_csr_pagerank_batched_df<float, 16><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl); break;
    case kF32 * 4 + 3: k_csr_pagerank_batched_dfs<float, 16><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl); break;
    case kBF16 * 4 + 0:
      k_csr_pagerank_batched_df<__nv_bfloat16, 8><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl);
      break;
    case kBF16 * 4 + 1:
      k_csr_pagerank_batched_dfs<__nv_bfloat16, 8><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl);
      break;
    case kBF16 * 4 + 2:
      k_csr_pagerank_batched_df<__nv_bfloat16, 16><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl);
      break;
    case kBF16 * 4 + 3:
      k_csr_pagerank_batched_dfs<__nv_bfloat16, 16><<<grid, NT, 0, s>>>(a, nvec, x, y, t, w, p, ctl);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t f64_to_df(const double* src, void* dst, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_f64_to_df<<<(int)std::min<long>((n + 255) / 256, 152L * 16), 256, 0, s>>>(src, static_cast<float2*>(dst), n);
  return cudaGetLastError();
}

cudaError_t df_to_f64(const void* src, double* dst, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_df_to_f64<<<(int)std::min<long>((n + 255) / 256, 152L * 16), 256, 0, s>>>(static_cast<const float2*>(src), dst,
                                                                           n);
  return cudaGetLastError();
}

cudaError_t csr_spmv(const CsrArgs& a, const double* x, double* y, cudaStream_t s) {
  if (a.nblocks == 0) return cudaSuccess;
  switch (a.prec) {
    case kF64: return spmv_items<double>(a, x, y, s);
    case kF32: return spmv_items<float>(a, x, y, s);
    case kBF16: return spmv_items<__nv_bfloat16>(a, x, y, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t csr_pagerank_step(const CsrArgs& a, const double* x, double* y,
                              const PageRankArgs& p, Ctl ctl, int grid, cudaStream_t s) {
  switch (a.prec) {
    case kF64: return pr_items<double>(a, x, y, p, ctl, grid, s);
    case kF32: return pr_items<float>(a, x, y, p, ctl, grid, s);
    case kBF16: return pr_items<__nv_bfloat16>(a, x, y, p, ctl, grid, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t pagerank_epilogue(const double* t, const double* x, double* y, long n, const PageRankArgs& p,
                              Ctl ctl, int grid, cudaStream_t s) {
  k_pagerank_epilogue<<<grid, NT, 0, s>>>(t, x, y, n, p, ctl);
  return cudaGetLastError();
}

cudaError_t csr_pagerank_batched_step(const CsrArgs& a, int n_row, int nvec, const double* X,
                                      double* Y, const double* T, const PageRankArgs& p,
                                      Ctl ctl, int grid, cudaStream_t s) {
  (void)n_row;
  if (nvec < 1 || nvec > kWarp) return cudaErrorInvalidValue;
  switch (a.prec) {
    case kF64: k_csr_pagerank_batched<double><<<grid, NT, 0, s>>>(a, nvec, X, Y, T, p, ctl); break;
    case kF32: k_csr_pagerank_batched<float><<<grid, NT, 0, s>>>(a, nvec, X, Y, T, p, ctl); break;
    case kBF16: k_csr_pagerank_batched<__nv_bfloat16><<<grid, NT, 0, s>>>(a, nvec, X, Y, T, p, ctl); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
