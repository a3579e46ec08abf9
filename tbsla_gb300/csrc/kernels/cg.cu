// Batched conjugate gradients on a block-diagonal concatenation of SPD CSR
// systems of uneven sizes.
//
// Follows tbsla::mpi::Matrix::CG (src/mpi/matrix/CG.cpp:32-73) with its
// vector helpers (:7-30), restated: the SpMV is q = A p (CG.cpp:61 passes
// the arguments in the other order), alpha = r.z / p.q, beta = r_new.z_new /
// r.z, optional Jacobi preconditioning z = D^-1 r, and a relative stop test
// ||r|| <= tol ||b|| confirmed on the FP64 true residual b - A x.
//
// Every system keeps its own scalars; one iteration over the whole batch is
// four launches (SpMV + p.q, update + r.z / r.r, scalars, direction) that
// skip the rows of systems which are not ACTIVE, so systems of 16^3 and 96^3
// rows run side by side and drop out as they converge.  The host captures a
// number of iterations in a CUDA graph and replays it.  With FP32 / BF16
// matrix storage the residual is recomputed in FP64 from the FP64 values
// every `refresh` iterations (residual replacement) and on every apparent
// convergence.
#include "common.cuh"
#include "csr_block.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

using namespace csr;

struct EpiDot {
  double* q;
  const double* p;
  __device__ __forceinline__ void emit(int row, double s, double* red) const {
    q[row] = s;
    red[0] = fma_rn(p[row], s, red[0]);
  }
};

struct EpiResidual {
  const double* b;
  double* r;
  double* z;  // nullptr when unpreconditioned
  const double* dinv;
  float* rf;  // factored preconditioner: r in FP32
  __device__ __forceinline__ void emit(int row, double s, double* red) const {
    const double ri = b[row] - s;
    r[row] = ri;
    if (rf) rf[row] = (float)ri;
    const double zi = dinv ? dinv[row] * ri : ri;
    if (dinv) z[row] = zi;
    red[0] = fma_rn(ri, ri, red[0]);
    red[1] = fma_rn(ri, zi, red[1]);
  }
};

// Row blocks per CTA of the SpMV: p.q is summed over the CTA's consecutive
// blocks of one system and reduced once.  The reduction (a warp butterfly
// and the warps' sums, all FP64) cost about as much FP64 pipe time per
// 256-row block as the block's 7 multiply-adds per row.  64 diffusion
// systems, Jacobi-PCG: 584-619 ms with one block per CTA, 558 ms with 4,
// 547 ms with 8.  The kernel also serves the learned-preconditioner solve,
// whose factor passes it does not shorten: the learned / Jacobi time ratio
// on the 128^3 systems was 0.454-0.469 with 1, 0.467 with 4, 0.478 with 8.
constexpr int kDotBlocksPerCta = 4;

template <class V, int ITEMS>
__global__ void __launch_bounds__(NT) k_cg_spmv_dot(CgBatch c) {
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ Smem sm;
  const int b0 = blockIdx.x * kDotBlocksPerCta;
  const int b1 = min(b0 + kDotBlocksPerCta, c.nblocks);
  const uint64_t pol = policy_evict_first();
  CsrArgs a{c.vals, c.prec, c.rowptr, c.colidx, c.blocks, c.nblocks, 0, c.items};
  EpiDot epi{c.q, c.p};
  double red[1] = {0};
  int cur = c.block_sys[b0];
  bool any = false;
  for (int b = b0; b < b1; b++) {  // uniform over the CTA
    const int sys = c.block_sys[b];
    if (sys != cur) {
      if (any) {
        const double v = block_sum<NT>(red[0], sm.red);
        if (threadIdx.x == 0) atomicAdd(c.pq + cur, v);
      }
      red[0] = 0;
      any = false;
      cur = sys;
    }
    if (c.status[sys] != kActive) continue;
    csr_block<V, ITEMS>(a, b, c.p, epi, red, stage, sm, pol);
    any = true;
  }
  if (any) {
    const double v = block_sum<NT>(red[0], sm.red);
    if (threadIdx.x == 0) atomicAdd(c.pq + cur, v);
  }
}

template <int ITEMS>
__global__ void __launch_bounds__(NT) k_cg_residual(CgBatch c, int mask) {
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ Smem sm;
  const int b = blockIdx.x;
  const int sys = c.block_sys[b];
  if (!((mask >> c.status[sys]) & 1)) return;
  const uint64_t pol = policy_evict_first();
  CsrArgs a{c.vals64, kF64, c.rowptr, c.colidx, c.blocks, c.nblocks, 0, c.items};
  EpiResidual epi{c.b, c.r, c.dinv ? c.z : nullptr, c.dinv, c.rf};
  double red[2] = {0, 0};
  csr_block<double, ITEMS>(a, b, c.x, epi, red, stage, sm, pol);
  const double rr = block_sum<NT>(red[0], sm.red);
  const double rz = block_sum<NT>(red[1], sm.red);
  if (threadIdx.x == 0) {
    atomicAdd(c.rrt + sys, rr);
    if (!c.rf) atomicAdd(c.rz + sys, rz);  // factored: r.z comes with z
  }
}

__global__ void __launch_bounds__(NT) k_cg_update(CgBatch c) {
  __shared__ double red_s[NT / kWarp];
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (c.status[sys] != kActive) return;
  const double pq = c.pq[sys];
  const double alpha = pq != 0 ? c.rz[sys] / pq : 0.0;
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  double rz = 0, rr = 0;
  for (int i = r0 + threadIdx.x; i < r1; i += NT) {
    const double pi = c.p[i], qi = c.q[i];
    c.x[i] = fma_rn(alpha, pi, c.x[i]);
    const double ri = fma_rn(-alpha, qi, c.r[i]);
    c.r[i] = ri;
    double zi = ri;
    if (c.dinv) {
      zi = c.dinv[i] * ri;
      c.z[i] = zi;
    }
    if (!c.rf) rz = fma_rn(ri, zi, rz);  // factored: r.z comes with z
    else c.rf[i] = (float)ri;
    rr = fma_rn(ri, ri, rr);
  }
  rz = block_sum<NT>(rz, red_s);
  rr = block_sum<NT>(rr, red_s);
  if (threadIdx.x == 0) {
    atomicAdd(c.rz_new + sys, rz);
    atomicAdd(c.rr + sys, rr);
  }
}

__global__ void k_cg_scalars(CgBatch c) {
  for (int s = threadIdx.x; s < c.nsys; s += blockDim.x) {
    if (c.status[s] != kActive) continue;
    c.iters[s] += 1;
    const double rzn = c.rz_new[s];
    c.beta[s] = c.rz[s] != 0 ? rzn / c.rz[s] : 0.0;
    c.rz[s] = rzn;
    if (c.rr[s] <= c.tol2 * c.bb[s]) c.status[s] = kVerify;
    else if (c.iters[s] >= c.max_it) c.status[s] = kStopped;
    c.pq[s] = 0;
    c.rz_new[s] = 0;
    c.rr[s] = 0;
  }
}

__global__ void __launch_bounds__(NT) k_cg_direction(CgBatch c) {
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (c.status[sys] != kActive) return;
  const double beta = c.beta[sys];
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  if (c.zf) {
    for (int i = r0 + threadIdx.x; i < r1; i += NT) c.p[i] = fma_rn(beta, c.p[i], (double)c.zf[i]);
  } else {
    const double* z = c.z;
    for (int i = r0 + threadIdx.x; i < r1; i += NT) c.p[i] = fma_rn(beta, c.p[i], z[i]);
  }
}

// Zero the true-residual accumulators of the masked systems.
__global__ void k_cg_pre_residual(CgBatch c, int mask) {
  for (int s = threadIdx.x; s < c.nsys; s += blockDim.x)
    if ((mask >> c.status[s]) & 1) {
      c.rrt[s] = 0;
      c.rz[s] = 0;
    }
}

__global__ void k_cg_post_residual(CgBatch c, int mask, int init) {
  for (int s = threadIdx.x; s < c.nsys; s += blockDim.x) {
    if (!((mask >> c.status[s]) & 1)) continue;
    const bool ok = c.rrt[s] <= c.tol2 * c.bb[s];
    if (init) {
      c.iters[s] = 0;
      c.pq[s] = c.rz_new[s] = c.rr[s] = 0;
      c.status[s] = ok ? kDone : kRestart;
    } else if (c.status[s] == kVerify) {
      c.status[s] = ok ? kDone : (c.iters[s] >= c.max_it ? kStopped : kRestart);
    } else if (c.status[s] == kActive) {
      // Periodic refresh of a system iterating on a narrowed matrix: the
      // FP64 residual belongs to another operator than the directions, so
      // the iteration restarts from it (one step of iterative refinement).
      c.status[s] = ok ? kDone : kRestart;
    }
  }
}

__global__ void __launch_bounds__(NT) k_cg_restart(CgBatch c, int all) {
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (!all && c.status[sys] != kRestart) return;
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  if (c.zf) {
    for (int i = r0 + threadIdx.x; i < r1; i += NT) c.p[i] = (double)c.zf[i];
  } else {
    const double* z = c.z;
    for (int i = r0 + threadIdx.x; i < r1; i += NT) c.p[i] = z[i];
  }
}

__device__ __forceinline__ float to_f32(double v) { return (float)v; }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }

// tf = L^T rf over the chunks of the masked systems (FP32 arithmetic).
template <class V>
__global__ void __launch_bounds__(NT) k_cg_factor_t(CgBatch c, int mask) {
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (!((mask >> c.status[sys]) & 1)) return;
  const V* v = static_cast<const V*>(c.tvals);
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  for (int i = r0 + threadIdx.x; i < r1; i += NT) {
    float s = 0.f;
    for (int k = c.trowptr[i]; k < c.trowptr[i + 1]; k++) s = fmaf(to_f32(v[k]), c.rf[c.tcolidx[k]], s);
    c.tf[i] = s;
  }
}

// z = L tf (FP32 arithmetic, stored in FP32: zf) and acc[sys] += r . z (FP64).
template <class V>
__global__ void __launch_bounds__(NT) k_cg_factor_l(CgBatch c, int mask, double* acc) {
  __shared__ double red_s[NT / kWarp];
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (!((mask >> c.status[sys]) & 1)) return;
  const V* v = static_cast<const V*>(c.lvals);
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  double d = 0;
  for (int i = r0 + threadIdx.x; i < r1; i += NT) {
    float s = 0.f;
    for (int k = c.lrowptr[i]; k < c.lrowptr[i + 1]; k++) s = fmaf(to_f32(v[k]), c.tf[c.lcolidx[k]], s);
    const double zi = widen(s);
    c.zf[i] = s;
    d = fma_rn(c.r[i], zi, d);
  }
  d = block_sum<NT>(d, red_s);
  if (threadIdx.x == 0) atomicAdd(acc + sys, d);
}

// The same two passes over the ELL form: slot k of row i is its k-th entry
// (same FP32 operations in the same order as the CSR passes; a padded slot
// adds 0 * x[i]).  No row pointer, 2-byte column offsets, every load of a
// slot coalesced.  The slots are unrolled up to KMAX (4, or 8 for longer
// rows), so a row's offset and value loads go out together and then its
// gathers: two memory latencies per row instead of two per slot.  One row
// per thread at a time keeps the registers low and the SM full of rows.
template <class V, int KMAX>
__device__ __forceinline__ float ell_row(const V* __restrict__ v, const short* __restrict__ dl,
                                         const float* __restrict__ x, long n, int K, int i) {
  short d[KMAX];
  V a[KMAX];
#pragma unroll
  for (int k = 0; k < KMAX; k++) {
    const long o = k * n + i;
    d[k] = k < K ? dl[o] : (short)0;
    a[k] = k < K ? v[o] : V(0.0f);
  }
  float g[KMAX];
#pragma unroll
  for (int k = 0; k < KMAX; k++) g[k] = k < K ? x[i + d[k]] : 0.f;
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < KMAX; k++)
    if (k < K) s = fmaf(to_f32(a[k]), g[k], s);
  return s;
}

template <class V, int KMAX>
__global__ void __launch_bounds__(NT) k_cg_factor_t_ell(CgBatch c, int mask) {
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (!((mask >> c.status[sys]) & 1)) return;
  const V* __restrict__ v = static_cast<const V*>(c.tvals);
  const int K = c.tslots, r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  for (int i = r0 + threadIdx.x; i < r1; i += NT) c.tf[i] = ell_row<V, KMAX>(v, c.tdelta, c.rf, c.n, K, i);
}

template <class V, int KMAX>
__global__ void __launch_bounds__(NT) k_cg_factor_l_ell(CgBatch c, int mask, double* acc) {
  __shared__ double red_s[NT / kWarp];
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  if (!((mask >> c.status[sys]) & 1)) return;
  const V* __restrict__ v = static_cast<const V*>(c.lvals);
  const int K = c.lslots, r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  double d = 0;
  for (int i = r0 + threadIdx.x; i < r1; i += NT) {
    const float zs = ell_row<V, KMAX>(v, c.ldelta, c.tf, c.n, K, i);
    c.zf[i] = zs;
    d = fma_rn(c.r[i], widen(zs), d);
  }
  d = block_sum<NT>(d, red_s);
  if (threadIdx.x == 0) atomicAdd(acc + sys, d);
}

__global__ void k_cg_activate(CgBatch c) {
  for (int s = threadIdx.x; s < c.nsys; s += blockDim.x)
    if (c.status[s] == kRestart) c.status[s] = kActive;
}

__global__ void __launch_bounds__(NT) k_cg_norms(CgBatch c) {
  __shared__ double red_s[NT / kWarp];
  const int ch = blockIdx.x;
  const int sys = c.chunk_sys[ch];
  const int r0 = c.chunks[ch], r1 = c.chunks[ch + 1];
  double bb = 0;
  for (int i = r0 + threadIdx.x; i < r1; i += NT) bb = fma_rn(c.b[i], c.b[i], bb);
  bb = block_sum<NT>(bb, red_s);
  if (threadIdx.x == 0) atomicAdd(c.bb + sys, bb);
}

__global__ void k_diag_inv(const int* __restrict__ rowptr, const int* __restrict__ colidx,
                           const double* __restrict__ vals, long n, double* __restrict__ dinv) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double d = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
      if (colidx[j] == i) d += vals[j];
    dinv[i] = d != 0 ? 1.0 / d : 1.0;
  }
}

template <class V, int ITEMS>
cudaError_t launch_dot(const CgBatch& c, cudaStream_t s) {
  constexpr size_t smem = stage_bytes<V, ITEMS>();
  cudaError_t ready = smem_opt_in<k_cg_spmv_dot<V, ITEMS>>(smem);
  if (ready != cudaSuccess) return ready;
  k_cg_spmv_dot<V, ITEMS><<<(c.nblocks + kDotBlocksPerCta - 1) / kDotBlocksPerCta, NT, smem, s>>>(c);
  return cudaGetLastError();
}

template <int ITEMS>
cudaError_t launch_res(const CgBatch& c, int mask, cudaStream_t s) {
  constexpr size_t smem = stage_bytes<double, ITEMS>();
  cudaError_t ready = smem_opt_in<k_cg_residual<ITEMS>>(smem);
  if (ready != cudaSuccess) return ready;
  k_cg_residual<ITEMS><<<c.nblocks, NT, smem, s>>>(c, mask);
  return cudaGetLastError();
}

}  // namespace

cudaError_t cg_spmv_dot(const CgBatch& c, cudaStream_t s) {
  if (c.nblocks == 0) return cudaSuccess;
  const int key = c.prec * 100 + c.items;
  switch (key) {
    case kF64 * 100 + 4: return launch_dot<double, 4>(c, s);
    case kF64 * 100 + 8: return launch_dot<double, 8>(c, s);
    case kF32 * 100 + 4: return launch_dot<float, 4>(c, s);
    case kF32 * 100 + 8: return launch_dot<float, 8>(c, s);
    case kBF16 * 100 + 4: return launch_dot<__nv_bfloat16, 4>(c, s);
    case kBF16 * 100 + 8: return launch_dot<__nv_bfloat16, 8>(c, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t cg_update(const CgBatch& c, cudaStream_t s) {
  if (c.nchunks == 0) return cudaSuccess;
  k_cg_update<<<c.nchunks, NT, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t cg_scalars(const CgBatch& c, cudaStream_t s) {
  k_cg_scalars<<<1, 256, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t cg_direction(const CgBatch& c, cudaStream_t s) {
  if (c.nchunks == 0) return cudaSuccess;
  k_cg_direction<<<c.nchunks, NT, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t cg_true_residual(const CgBatch& c, int mask, bool init, cudaStream_t s) {
  k_cg_pre_residual<<<1, 256, 0, s>>>(c, mask);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (c.nblocks) {
    e = c.items == 4 ? launch_res<4>(c, mask, s) : launch_res<8>(c, mask, s);
    if (e != cudaSuccess) return e;
  }
  if (c.rf) {  // z = L L^T r, rz = r.z of the masked systems
    e = cg_factor_apply(c, mask, c.rz, s);
    if (e != cudaSuccess) return e;
  }
  k_cg_post_residual<<<1, 256, 0, s>>>(c, mask, init ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t cg_restart(const CgBatch& c, bool all, cudaStream_t s) {
  if (c.nchunks) k_cg_restart<<<c.nchunks, NT, 0, s>>>(c, all ? 1 : 0);
  k_cg_activate<<<1, 256, 0, s>>>(c);
  return cudaGetLastError();
}

template <class V>
cudaError_t factor_apply(const CgBatch& c, int mask, double* acc, cudaStream_t s) {
  if (c.lslots > 0 && c.lslots <= 4 && c.tslots <= 4) {
    k_cg_factor_t_ell<V, 4><<<c.nchunks, NT, 0, s>>>(c, mask);
    k_cg_factor_l_ell<V, 4><<<c.nchunks, NT, 0, s>>>(c, mask, acc);
  } else if (c.lslots > 0) {
    k_cg_factor_t_ell<V, 8><<<c.nchunks, NT, 0, s>>>(c, mask);
    k_cg_factor_l_ell<V, 8><<<c.nchunks, NT, 0, s>>>(c, mask, acc);
  } else {
    k_cg_factor_t<V><<<c.nchunks, NT, 0, s>>>(c, mask);
    k_cg_factor_l<V><<<c.nchunks, NT, 0, s>>>(c, mask, acc);
  }
  return cudaGetLastError();
}

cudaError_t cg_factor_apply(const CgBatch& c, int mask, double* acc, cudaStream_t s) {
  if (!c.rf || c.nchunks == 0) return cudaSuccess;
  switch (c.lprec) {
    case kF64: return factor_apply<double>(c, mask, acc, s);
    case kF32: return factor_apply<float>(c, mask, acc, s);
    case kBF16: return factor_apply<__nv_bfloat16>(c, mask, acc, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t cg_norms(const CgBatch& c, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(c.bb, 0, sizeof(double) * c.nsys, s);
  if (e != cudaSuccess || c.nchunks == 0) return e;
  k_cg_norms<<<c.nchunks, NT, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t csr_diag_inv(const int* rowptr, const int* colidx, const double* vals, long n,
                         double* dinv, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (int)std::min<long>((n + 255) / 256, 152L * 16);
  k_diag_inv<<<grid, 256, 0, s>>>(rowptr, colidx, vals, n, dinv);
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
