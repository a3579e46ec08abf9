// Batched CG: block-diagonal device copy of many SPD systems and the solve
// loop around the kernels of kernels/cg.cu.
//
// HBM layout of a batch: the systems' CSR arrays concatenated (rowptr
// int32[n+1], colidx int32[nnz] shifted to global columns, values in the
// storage precision and in FP64), the row-block partition of the SpMV and
// the row chunks of the vector kernels (neither crosses a system boundary,
// each carries its system id), the Jacobi diagonal, six FP64 vectors (b, x,
// r, z, p, q) and per-system scalars.
//
// Two engines solve a batch:
//  - persistent (kernels/cg_dia.cu): when every system's entries lie on at
//    most 8 diagonals (stencils) and there are at most 256 systems, the batch
//    also holds A slot-major per diagonal (values in the storage precision
//    and in FP64, a delta table per system), the FP32 Jacobi diagonal and
//    eight solve vectors in the iteration precision (FP32 for FP32 / BF16
//    storage); the whole solve is one cooperative launch, captured once in a
//    CUDA graph and replayed.  A factored preconditioner on at most 8
//    diagonals is kept the same way (slot 0 the diagonal).
//  - multi-launch (kernels/cg.cu): any other batch, and factors that are not
//    diagonal-structured: four to six launches per iteration, captured in
//    graphs of `graph_iters` iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "api_guard.hpp"
#include "device.hpp"
#include "host/parallel.hpp"
#include "kernels/kernels.hpp"

using namespace tbsla_gpu;

namespace {

constexpr int kChunkRows = 2048;
constexpr int kNScal = 7;  // rz, rz_new, pq, rr, bb, beta, rrt

int st_of(cudaError_t e) {
  if (e == cudaSuccess) return TBSLA_OK;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? TBSLA_ERR_ALLOC : TBSLA_ERR_CUDA;
}

#define CK(call)                              \
  do {                                        \
    int s_ = st_of(call);                     \
    if (s_ != TBSLA_OK) return s_;            \
  } while (0)

template <class T>
cudaError_t alloc(T** p, size_t n) {
  *p = nullptr;
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

}  // namespace

struct tbsla_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int nsys = 0;
  long n = 0, nnz = 0;
  std::vector<long> off;
  int prec = TBSLA_F64;
  int *rowptr = nullptr, *colidx = nullptr;
  void* vals = nullptr;
  double* vals64 = nullptr;
  int *blocks = nullptr, *block_sys = nullptr;
  int nblocks = 0;
  int *chunks = nullptr, *chunk_sys = nullptr;
  int nchunks = 0;
  double* dinv = nullptr;
  // factored preconditioner L L^T (block-diagonal over the systems)
  int *lrowptr = nullptr, *lcolidx = nullptr, *trowptr = nullptr, *tcolidx = nullptr;
  void *lvals = nullptr, *tvals = nullptr;
  int lprec = TBSLA_F64;
  short *ldelta = nullptr, *tdelta = nullptr;  // ELL form (lslots > 0)
  int lslots = 0, tslots = 0;
  float *rf = nullptr, *tf = nullptr, *zf = nullptr;
  double *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  double* scal = nullptr;
  int *status = nullptr, *iters = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_k = 0, graph_pre = -1, graph_max = -1;
  double graph_tol2 = -1;

  // persistent engine (DIA layout)
  bool dia = false;
  bool vec4 = false;              // FP32 iteration, every system's first row and size a multiple of 4
  bool vec4_off = false;          // tuning: one row per thread even where 4 would do
  bool st7_off = false;           // tuning: the general kernel even for seven-point batches
  int ctas_per_sm = 0;            // tuning: CTAs per SM of the persistent launch (0: all that fit)
  int K = 0;                      // diagonal slots of A
  std::vector<int> adelta_h;      // [nsys * kDiaMaxDiag]
  int* adelta = nullptr;
  long* sys_off = nullptr;
  int* row_sys = nullptr;
  void* avals_dia = nullptr;      // [K][n] storage precision
  double* a64_dia = nullptr;      // [K][n]
  float* dinv_f = nullptr;
  bool dia_factor = false;        // the factor is held in DIA form
  int KL = 0;
  std::vector<int> fdelta_h;      // [nsys * kDiaMaxDiag] deltas of the factor's slots
  int* fdelta = nullptr;
  void* lvals_dia = nullptr;      // [KL][n] in lprec_dia
  size_t lvals_cap = 0;           // bytes allocated at lvals_dia
  int lprec_dia = TBSLA_F32;
  void *dv = nullptr, *r0 = nullptr, *r1 = nullptr, *p0 = nullptr, *p1 = nullptr, *q2 = nullptr,
       *z2 = nullptr, *t2 = nullptr;
  int *mode_d = nullptr, *fallback_d = nullptr;
  double *relres_d = nullptr, *acc = nullptr;
  unsigned* bar = nullptr;
  long long wait_ns = 2000000000LL;  // bound on one grid-wide wait of the persistent kernel
  int pgrid = 0;
  cudaGraphExec_t pgraph = nullptr;
  DiaCg pkey{};                   // the arguments the graph was captured with
  int pkey_pre = -1;
  bool pgraph_ok = false;
  // last solve
  std::vector<int> fallback_h, mode_h;
  std::vector<int> factor_fb;     // per system: the factor failed the host check (multi-launch engine)
  int last_engine = 0, last_graph = 0, last_st7 = 0;

  ~tbsla_batch() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    if (graph) cudaGraphExecDestroy(graph);
    if (pgraph) cudaGraphExecDestroy(pgraph);
    void* ps[] = {rowptr, colidx, vals64, blocks, block_sys, chunks, chunk_sys, dinv, b, x, r, z, p, q,
                  scal, status, iters, lrowptr, lcolidx, trowptr, tcolidx, lvals, tvals, rf, tf,
                  ldelta, tdelta, zf, adelta, sys_off, row_sys, a64_dia, dinv_f, fdelta, lvals_dia,
                  dv, r0, r1, p0, p1, q2, z2, t2, mode_d, fallback_d, relres_d, acc, bar};
    for (void* v : ps)
      if (v) cudaFree(v);
    if (avals_dia && avals_dia != (void*)a64_dia) cudaFree(avals_dia);
    if (vals && vals != vals64) cudaFree(vals);
    if (stream) cudaStreamDestroy(stream);
  }

  // precond: 0 none, 1 Jacobi, 2 factored L L^T
  CgBatch view(int precond, double tol2, int max_it) const {
    CgBatch c{};
    c.nsys = nsys;
    c.n = n;
    c.rowptr = rowptr;
    c.colidx = colidx;
    c.vals = vals;
    c.prec = prec;
    c.vals64 = vals64;
    c.blocks = blocks;
    c.block_sys = block_sys;
    c.nblocks = nblocks;
    c.items = 8;
    c.chunks = chunks;
    c.chunk_sys = chunk_sys;
    c.nchunks = nchunks;
    c.dinv = precond == 1 ? dinv : nullptr;
    const bool f = precond == 2;
    c.lrowptr = f ? lrowptr : nullptr;
    c.lcolidx = f ? lcolidx : nullptr;
    c.trowptr = f ? trowptr : nullptr;
    c.tcolidx = f ? tcolidx : nullptr;
    c.lvals = f ? lvals : nullptr;
    c.tvals = f ? tvals : nullptr;
    c.lprec = lprec;
    c.ldelta = f ? ldelta : nullptr;
    c.tdelta = f ? tdelta : nullptr;
    c.lslots = f ? lslots : 0;
    c.tslots = f ? tslots : 0;
    c.rf = f ? rf : nullptr;
    c.zf = f ? zf : nullptr;
    c.tf = f ? tf : nullptr;
    c.b = b;
    c.x = x;
    c.r = r;
    c.z = precond ? z : r;
    c.p = p;
    c.q = q;
    c.rz = scal;
    c.rz_new = scal + nsys;
    c.pq = scal + 2 * nsys;
    c.rr = scal + 3 * nsys;
    c.bb = scal + 4 * nsys;
    c.beta = scal + 5 * nsys;
    c.rrt = scal + 6 * nsys;
    c.status = status;
    c.iters = iters;
    c.tol2 = tol2;
    c.max_it = max_it;
    return c;
  }
};

namespace {


// Diagonal structure of the concatenated CSR arrays: per system the sorted
// distinct col - row values (at most kDiaMaxDiag), false when a system has
// more, a row repeats a column, or the batch has more than kDiaMaxSys
// systems.  Systems are scanned in parallel.
bool dia_deltas(const tbsla_batch* B, const std::vector<int>& rp, const std::vector<int>& ci,
                std::vector<int>* delta, int* K) {
  const int nsys = B->nsys;
  if (nsys > kDiaMaxSys) return false;
  delta->assign((size_t)nsys * kDiaMaxDiag, 0);
  std::vector<int> cnt(nsys, 0);
  std::vector<char> ok(nsys, 1);
  tbsla_impl::parallel_for_items(nsys, [&](long b, long e) {
    for (long s = b; s < e; s++) {
      int* ds = delta->data() + s * kDiaMaxDiag;
      int c = 0, hint = 0;
      for (long i = B->off[s]; i < B->off[s + 1] && ok[s]; i++) {
        unsigned used = 0;
        for (int q = rp[i]; q < rp[i + 1]; q++) {
          const long d = (long)ci[q] - i;
          int k = -1;
          for (int t = 0; t < c; t++) {  // start at the slot after the last hit
            const int u = (hint + t) % c;
            if (ds[u] == d) {
              k = u;
              break;
            }
          }
          if (k < 0) {
            if (c == kDiaMaxDiag) {
              ok[s] = 0;
              break;
            }
            ds[c] = (int)d;
            k = c++;
          }
          if (used & (1u << k)) {  // the row repeats a column
            ok[s] = 0;
            break;
          }
          used |= 1u << k;
          hint = (k + 1) % std::max(c, 1);
        }
      }
      std::sort(ds, ds + c);
      cnt[s] = c;
    }
  });
  *K = 0;
  for (int s = 0; s < nsys; s++) {
    if (!ok[s]) return false;
    *K = std::max(*K, cnt[s]);
  }
  return *K > 0;
}

// The DIA copy of the batch and the persistent engine's vectors.
int build_dia(tbsla_batch* B, const std::vector<int>& delta, int K) {
  cudaStream_t st = B->stream;
  const long n = B->n;
  const int nsys = B->nsys;
  std::vector<int> rsys(n);
  tbsla_impl::parallel_for_items(nsys, [&](long b, long e) {
    for (long s = b; s < e; s++)
      for (long i = B->off[s]; i < B->off[s + 1]; i++) rsys[i] = (int)s;
  });
  CK(alloc(&B->adelta, delta.size()));
  CK(alloc(&B->sys_off, B->off.size()));
  CK(alloc(&B->row_sys, (size_t)n));
  CK(cudaMemcpyAsync(B->adelta, delta.data(), delta.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->sys_off, B->off.data(), B->off.size() * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->row_sys, rsys.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
  CK(alloc(&B->a64_dia, (size_t)K * n));
  CK(cudaMemsetAsync(B->a64_dia, 0, (size_t)K * n * 8, st));
  CK(dia_fill(B->rowptr, B->colidx, B->vals64, B->row_sys, B->adelta, K, n, B->a64_dia, st));
  if (B->prec == TBSLA_F64) {
    B->avals_dia = B->a64_dia;
  } else {
    CK(cudaMalloc(&B->avals_dia, std::max<size_t>((size_t)K * n, 1) * (B->prec == TBSLA_F32 ? 4 : 2)));
    CK(convert_values(B->a64_dia, B->avals_dia, B->prec, (long)K * n, st));
  }
  CK(alloc(&B->dinv_f, (size_t)n));
  CK(dia_dinv(B->a64_dia, B->row_sys, B->adelta, K, n, B->dinv_f, st));
  const size_t es = B->prec == TBSLA_F64 ? 8 : 4;
  for (void** v : {&B->dv, &B->r0, &B->r1, &B->p0, &B->p1, &B->q2, &B->z2, &B->t2})
    CK(cudaMalloc(v, std::max<size_t>((size_t)n, 1) * es));
  CK(alloc(&B->mode_d, nsys));
  CK(alloc(&B->fallback_d, nsys));
  CK(alloc(&B->relres_d, nsys));
  CK(alloc(&B->acc, (size_t)12 * nsys));
  CK(alloc(&B->bar, 4));
  B->vec4 = B->prec != TBSLA_F64;
  for (int s = 0; s <= nsys; s++) B->vec4 = B->vec4 && B->off[s] % 4 == 0;
  B->adelta_h = delta;
  B->K = K;
  B->dia = true;
  B->fallback_h.assign(nsys, 0);
  B->mode_h.assign(nsys, 0);
  return TBSLA_OK;
}

int build_batch(tbsla_batch* B, tbsla_matrix* const* sys, int nsys, int prec) {
  using namespace tbsla_impl;
  B->nsys = nsys;
  B->prec = prec;
  B->off.assign(nsys + 1, 0);
  long nnz = 0;
  for (int s = 0; s < nsys; s++) {
    const tbsla_matrix* m = sys[s];
    const tbsla_info& I = m->info;
    if (m->format != TBSLA_CSR || I.n_row != I.n_col || I.ln_row != I.n_row || I.ln_col != I.n_col ||
        I.f_col != 0 || I.f_row != 0 || I.nnz <= 0)
      return TBSLA_ERR_INVALID_ARG;
    int v = validate(m);
    if (v) return v;
    B->off[s + 1] = B->off[s] + I.n_row;
    nnz += (long)m->idx0[I.n_row] - m->idx0[0];
  }
  B->n = B->off[nsys];
  B->nnz = nnz;
  if (B->n > INT_MAX - 1 || nnz > INT_MAX) return TBSLA_ERR_INVALID_ARG;
  std::vector<int> rp(B->n + 1), ci(nnz);
  std::vector<double> va(nnz);
  std::vector<int> blocks{0}, bsys, chunks{0}, csys;
  long k = 0;
  for (int s = 0; s < nsys; s++) {
    const tbsla_matrix* m = sys[s];
    const int ns = m->info.n_row;
    const int* mrp = m->idx0.data();
    const long o = B->off[s];
    for (int i = 0; i < ns; i++) {
      rp[o + i] = (int)k;
      for (int j = mrp[i]; j < mrp[i + 1]; j++, k++) {
        ci[k] = m->idx1[j] + (int)o;
        va[k] = m->values[j];
      }
    }
    int* pb = nullptr;
    int nb = 0;
    csr_partition(mrp, ns, 2048, &pb, &nb);
    for (int t = 1; t <= nb; t++) {
      blocks.push_back((int)o + pb[t]);
      bsys.push_back(s);
    }
    delete[] pb;
    for (int r0 = 0; r0 < ns; r0 += kChunkRows) {
      chunks.push_back((int)o + std::min(ns, r0 + kChunkRows));
      csys.push_back(s);
    }
  }
  rp[B->n] = (int)k;
  B->nblocks = (int)bsys.size();
  B->nchunks = (int)csys.size();
  cudaStream_t st = B->stream;
  CK(alloc(&B->rowptr, rp.size()));
  CK(alloc(&B->colidx, ci.size()));
  CK(alloc(&B->vals64, va.size()));
  CK(alloc(&B->blocks, blocks.size()));
  CK(alloc(&B->block_sys, bsys.size()));
  CK(alloc(&B->chunks, chunks.size()));
  CK(alloc(&B->chunk_sys, csys.size()));
  CK(cudaMemcpyAsync(B->rowptr, rp.data(), rp.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->colidx, ci.data(), ci.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->vals64, va.data(), va.size() * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->blocks, blocks.data(), blocks.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->block_sys, bsys.data(), bsys.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->chunks, chunks.data(), chunks.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B->chunk_sys, csys.data(), csys.size() * 4, cudaMemcpyHostToDevice, st));
  if (prec == TBSLA_F64) {
    B->vals = B->vals64;
  } else {
    size_t es = prec == TBSLA_F32 ? 4 : 2;
    CK(cudaMalloc(&B->vals, std::max<size_t>(nnz, 1) * es));
    CK(convert_values(B->vals64, B->vals, prec, nnz, st));
  }
  CK(alloc(&B->dinv, B->n));
  CK(csr_diag_inv(B->rowptr, B->colidx, B->vals64, B->n, B->dinv, st));
  for (double** v : {&B->b, &B->x, &B->r, &B->z, &B->p, &B->q}) CK(alloc(v, B->n));
  CK(alloc(&B->scal, (size_t)kNScal * nsys));
  CK(alloc(&B->status, nsys));
  CK(alloc(&B->iters, nsys));
  std::vector<int> delta;
  int K = 0;
  if (dia_deltas(B, rp, ci, &delta, &K)) {
    int st2 = build_dia(B, delta, K);
    if (st2) return st2;
  }
  return st_of(cudaStreamSynchronize(st));
}

int capture(tbsla_batch* B, const CgBatch& c, int K) {
  cudaStream_t s = B->stream;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < K; i++) {
    cudaError_t e = cg_spmv_dot(c, s);
    if (e == cudaSuccess) e = cg_update(c, s);
    if (e == cudaSuccess) e = cg_factor_apply(c, 1 << kActive, c.rz_new, s);
    if (e == cudaSuccess) e = cg_scalars(c, s);
    if (e == cudaSuccess) e = cg_direction(c, s);
    if (e != cudaSuccess) {
      cudaStreamEndCapture(s, &g);
      return st_of(e);
    }
  }
  CK(cudaStreamEndCapture(s, &g));
  cudaError_t e = cudaGraphInstantiate(&B->graph, g, 0);
  cudaGraphDestroy(g);
  return st_of(e);
}



// The DIA factor's value array, grown on demand and kept (repeated factor
// builds of the same batch allocate nothing).
cudaError_t lvals_reserve(tbsla_batch* B, size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  if (B->lvals_dia && B->lvals_cap >= bytes) return cudaSuccess;
  if (B->lvals_dia) cudaFree(B->lvals_dia);
  B->lvals_dia = nullptr;
  B->lvals_cap = 0;
  cudaError_t e = cudaMalloc(&B->lvals_dia, bytes);
  if (e == cudaSuccess) B->lvals_cap = bytes;
  return e;
}

// A factor on at most kDiaMaxDiag diagonals per system, kept in DIA form for
// the persistent engine (slot 0 the diagonal, then the other deltas in
// descending order); TBSLA_ERR_UNSUPPORTED for any other factor.
int set_dia_factor(tbsla_batch* B, const std::vector<int>& rp, const std::vector<int>& ci,
                   const std::vector<double>& va, int precision) {
  const int nsys = B->nsys;
  const long n = B->n;
  std::vector<int> delta((size_t)nsys * kDiaMaxDiag, 0);
  int KL = 0;
  for (int s = 0; s < nsys; s++) {
    int* ds = delta.data() + (size_t)s * kDiaMaxDiag;
    int c = 1;  // ds[0] = 0, the diagonal
    for (long i = B->off[s]; i < B->off[s + 1]; i++) {
      unsigned used = 0;
      for (int q = rp[i]; q < rp[i + 1]; q++) {
        const int d = ci[q] - (int)i;
        int k = 0;
        while (k < c && ds[k] != d) k++;
        if (k == c) {
          if (c == kDiaMaxDiag) return TBSLA_ERR_UNSUPPORTED;
          ds[c++] = d;
        }
        if (used & (1u << k)) return TBSLA_ERR_UNSUPPORTED;  // repeated column
        used |= 1u << k;
      }
    }
    std::sort(ds + 1, ds + c, [](int a, int b) { return a > b; });
    KL = std::max(KL, c);
  }
  cudaSetDevice(B->device);
  cudaStream_t st = B->stream;
  int *rp_d = nullptr, *ci_d = nullptr;
  double *va_d = nullptr, *l64 = nullptr;
  auto release = [&]() {
    for (void* p : {(void*)rp_d, (void*)ci_d, (void*)va_d, (void*)l64})
      if (p) cudaFree(p);
  };
  auto fail = [&](cudaError_t e) {
    cudaStreamSynchronize(st);
    release();
    return st_of(e);
  };
  cudaError_t e;
  if ((e = alloc(&rp_d, rp.size())) || (e = alloc(&ci_d, std::max<size_t>(ci.size(), 1))) ||
      (e = alloc(&va_d, std::max<size_t>(va.size(), 1))) || (e = alloc(&l64, (size_t)KL * n)))
    return fail(e);
  if (!B->fdelta && (e = alloc(&B->fdelta, delta.size()))) return fail(e);
  const int lprec = precision == TBSLA_BF16 ? TBSLA_BF16 : TBSLA_F32;
  if ((e = lvals_reserve(B, (size_t)KL * n * (lprec == TBSLA_BF16 ? 2 : 4))) ||
      (e = cudaMemcpyAsync(rp_d, rp.data(), rp.size() * 4, cudaMemcpyHostToDevice, st)) ||
      (!ci.empty() && (e = cudaMemcpyAsync(ci_d, ci.data(), ci.size() * 4, cudaMemcpyHostToDevice, st))) ||
      (!va.empty() && (e = cudaMemcpyAsync(va_d, va.data(), va.size() * 8, cudaMemcpyHostToDevice, st))) ||
      (e = cudaMemcpyAsync(B->fdelta, delta.data(), delta.size() * 4, cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemsetAsync(l64, 0, (size_t)KL * n * 8, st)) ||
      (e = dia_fill(rp_d, ci_d, va_d, B->row_sys, B->fdelta, KL, n, l64, st)) ||
      (e = convert_values(l64, B->lvals_dia, lprec, (long)KL * n, st)) || (e = cudaStreamSynchronize(st)))
    return fail(e);
  release();
  B->fdelta_h = delta;
  B->KL = KL;
  B->lprec_dia = lprec;
  B->dia_factor = true;
  return TBSLA_OK;
}

// The persistent engine: H2D of b, x and the per-system modes, then the
// device part -- clearing the correction, accumulators and barrier words,
// and the one cooperative launch -- replayed from a CUDA graph captured once
// per argument set (a direct launch where capture is refused), then D2H of
// x and the per-system results.
int dia_solve(tbsla_batch* B, const double* rhs, double* x, int max_iterations, double rel_tol, int precond,
              int refresh, int* iterations, double* rel_residual) {
  cudaStream_t s = B->stream;
  const int ns = B->nsys;
  const long n = B->n;
  const int lprec = precond == 2 ? B->lprec_dia : TBSLA_F32;
  const bool vec4 = B->vec4 && !B->vec4_off;
  // the seven-point form of the kernel (neighbour alignments fixed at compile
  // time) where every system is a 7-point stencil with n, n^2 multiples of 4
  const bool st7 = vec4 && B->prec != TBSLA_F64 && !B->st7_off &&
                   B->adelta_h.size() >= (size_t)ns * kDiaMaxDiag &&
                   (precond != 2 || B->fdelta_h.size() >= (size_t)ns * kDiaMaxDiag) &&
                   dia_seven_point(B->adelta_h.data(), precond == 2 ? B->fdelta_h.data() : nullptr, ns, B->K,
                                   precond == 2 ? B->KL : 0);
  int grid = cg_dia_grid(B->prec, lprec, st7 ? 1 : 0);
  if (grid <= 0) return TBSLA_ERR_CUDA;
  if (B->ctas_per_sm > 0) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device);
    grid = std::min(grid, B->ctas_per_sm * sms);
  }
  DiaCg c;
  std::memset(&c, 0, sizeof c);  // padding too: the struct is the graph's cache key
  c.nsys = ns;
  c.n = n;
  c.K = B->K;
  c.KL = precond == 2 ? B->KL : 0;
  c.sys_off = B->sys_off;
  c.adelta = B->adelta;
  c.avals = B->avals_dia;
  c.prec = B->prec;
  c.a64 = B->a64_dia;
  c.dinv = B->dinv_f;
  c.ldelta = precond == 2 ? B->fdelta : nullptr;
  c.lvals = precond == 2 ? B->lvals_dia : nullptr;
  c.lprec = lprec;
  c.b = B->b;
  c.x = B->x;
  c.d = B->dv;
  c.r0 = B->r0;
  c.r1 = B->r1;
  c.p0 = B->p0;
  c.p1 = B->p1;
  c.q = B->q2;
  c.z = B->z2;
  c.t = B->t2;
  c.mode = B->mode_d;
  c.status = B->status;
  c.iters = B->iters;
  c.fallback = B->fallback_d;
  c.relres = B->relres_d;
  c.acc = B->acc;
  c.bar = B->bar;
  c.tol2 = rel_tol * rel_tol;
  c.max_it = max_iterations;
  c.refresh = B->prec != TBSLA_F64 ? refresh : 0;
  c.wait_ns = B->wait_ns;
  c.vec4 = vec4 ? 1 : 0;
  c.st7 = st7 ? 1 : 0;
  std::vector<int> mode(ns, precond);
  CK(cudaMemcpyAsync(B->b, rhs, n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->x, x, n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->mode_d, mode.data(), ns * sizeof(int), cudaMemcpyHostToDevice, s));
  const size_t es = B->prec == TBSLA_F64 ? 8 : 4;
  auto enqueue = [&](cudaStream_t st) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    // Jacobi builds its preconditioner (D^-1 from A's diagonal) inside every
    // solve, as the factored form builds L before its solve
    if (precond == 1) e = dia_dinv(B->a64_dia, B->row_sys, B->adelta, B->K, n, B->dinv_f, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->dv, 0, (size_t)n * es, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->acc, 0, (size_t)12 * ns * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->bar, 0, 4 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cg_dia_solve(c, grid, st);
    return e;
  };
  if (!B->pgraph || std::memcmp(&B->pkey, &c, sizeof c) != 0 || B->pkey_pre != precond) {
    if (B->pgraph) cudaGraphExecDestroy(B->pgraph);
    B->pgraph = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      e = enqueue(s);
      const cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&B->pgraph, g, 0);
      if (g) cudaGraphDestroy(g);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      if (B->pgraph) cudaGraphExecDestroy(B->pgraph);
      B->pgraph = nullptr;
    }
    B->pkey = c;
    B->pkey_pre = precond;
  }
  if (B->pgraph) CK(cudaGraphLaunch(B->pgraph, s));
  else CK(enqueue(s));
  std::vector<int> st(ns), it(ns);
  std::vector<double> rr(ns);
  unsigned err[4] = {0, 0, 0, 0};
  B->mode_h.assign(ns, 0);
  B->fallback_h.assign(ns, 0);
  CK(cudaMemcpyAsync(x, B->x, n * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(st.data(), B->status, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(it.data(), B->iters, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(rr.data(), B->relres_d, ns * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(B->mode_h.data(), B->mode_d, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(B->fallback_h.data(), B->fallback_d, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(err, B->bar, sizeof err, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  B->last_engine = 1;
  B->last_graph = B->pgraph ? 1 : 0;
  B->last_st7 = st7 ? 1 : 0;
  if (err[2]) return TBSLA_ERR_TIMEOUT;
  bool all = true;
  for (int k = 0; k < ns; k++) {
    if (iterations) iterations[k] = it[k];
    if (rel_residual) rel_residual[k] = rr[k];
    all &= st[k] == kDone;
  }
  return all ? TBSLA_OK : TBSLA_ERR_NOT_CONVERGED;
}

}  // namespace

extern "C" {

int tbsla_batch_create(tbsla_batch** out, tbsla_matrix* const* systems, int nsys, int precision) try {
  if (!out || !systems || nsys <= 0 || precision < TBSLA_F64 || precision > TBSLA_BF16)
    return TBSLA_ERR_INVALID_ARG;
  for (int s = 0; s < nsys; s++)
    if (!systems[s]) return TBSLA_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return TBSLA_ERR_NO_DEVICE;
  }
  std::unique_ptr<tbsla_batch> B(new tbsla_batch());  // freed if the build fails or throws
  cudaGetDevice(&B->device);
  int st = st_of(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  if (!st) st = build_batch(B.get(), systems, nsys, precision);
  if (st) return st;
  *out = B.release();
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_destroy(tbsla_batch* b) try {
  delete b;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_set_factors(tbsla_batch* B, tbsla_matrix* const* factors, int nsys, int precision) try {
  using namespace tbsla_impl;
  if (!B || !factors || nsys != B->nsys || precision < TBSLA_F64 || precision > TBSLA_BF16)
    return TBSLA_ERR_INVALID_ARG;
  // L concatenated block-diagonally, and L^T built by a counting sort
  std::vector<int> rp(B->n + 1, 0), ci;
  std::vector<double> va;
  for (int s = 0; s < nsys; s++) {
    const tbsla_matrix* m = factors[s];
    if (!m || m->format != TBSLA_CSR) return TBSLA_ERR_INVALID_ARG;
    const tbsla_info& I = m->info;
    const long o = B->off[s], ns = B->off[s + 1] - o;
    if (I.n_row != ns || I.n_col != ns || I.ln_row != ns || I.f_col != 0) return TBSLA_ERR_INVALID_ARG;
    int v = validate(m);
    if (v) return v;
    const int* mrp = m->idx0.data();
    for (long i = 0; i < ns; i++) {
      for (int j = mrp[i]; j < mrp[i + 1]; j++) {
        if (m->idx1[j] > i) return TBSLA_ERR_BAD_MATRIX;  // not lower-triangular
        ci.push_back(m->idx1[j] + (int)o);
        va.push_back(m->values[j]);
      }
      rp[o + i + 1] = (int)ci.size();
    }
  }
  // Per system, the check the persistent engine makes on the device before
  // its first iteration: every value finite, every diagonal entry > 0.
  B->factor_fb.assign(nsys, 0);
  for (int s = 0; s < nsys; s++)
    for (long i = B->off[s]; i < B->off[s + 1] && !B->factor_fb[s]; i++) {
      bool diag = false;
      for (int k = rp[i]; k < rp[i + 1]; k++) {
        if (!std::isfinite(va[k])) B->factor_fb[s] = kFallbackBadFactor;
        if (ci[k] == i) diag = va[k] > 0;
      }
      if (!diag) B->factor_fb[s] = kFallbackBadFactor;
    }
  if (B->dia) {
    const int st2 = set_dia_factor(B, rp, ci, va, precision);
    if (st2 != TBSLA_ERR_UNSUPPORTED) return st2;
  }
  B->dia_factor = false;
  if (std::count(B->factor_fb.begin(), B->factor_fb.end(), 0) != nsys) {
    // the multi-launch engine runs a system whose factor failed the check
    // with the Jacobi factor L = D^-1/2 (z = D^-1 r: Jacobi-PCG)
    std::vector<double> dinv(B->n);
    CK(cudaMemcpy(dinv.data(), B->dinv, B->n * 8, cudaMemcpyDeviceToHost));
    std::vector<int> rp2(B->n + 1, 0), ci2;
    std::vector<double> va2;
    ci2.reserve(ci.size());
    va2.reserve(va.size());
    for (int s = 0; s < nsys; s++)
      for (long i = B->off[s]; i < B->off[s + 1]; i++) {
        if (B->factor_fb[s]) {
          ci2.push_back((int)i);
          va2.push_back(std::sqrt(dinv[i]));
        } else {
          for (int k = rp[i]; k < rp[i + 1]; k++) {
            ci2.push_back(ci[k]);
            va2.push_back(va[k]);
          }
        }
        rp2[i + 1] = (int)ci2.size();
      }
    rp.swap(rp2);
    ci.swap(ci2);
    va.swap(va2);
  }
  const long nl = (long)ci.size();
  std::vector<int> trp(B->n + 1, 0), tci(nl);
  std::vector<double> tva(nl);
  for (long k = 0; k < nl; k++) trp[ci[k] + 1]++;
  for (long i = 0; i < B->n; i++) trp[i + 1] += trp[i];
  std::vector<int> fill(trp.begin(), trp.end() - 1);
  for (long i = 0; i < B->n; i++)
    for (int k = rp[i]; k < rp[i + 1]; k++) {
      const int q = fill[ci[k]]++;
      tci[q] = (int)i;
      tva[q] = va[k];
    }
  // ELL form of L and of L^T when every row has at most 8 entries, every
  // column lies within 32767 of its row and the padding stays under half
  // the entries (stencil-pattern factors: 4 entries per row)
  std::vector<short> ld, td;
  std::vector<double> lv, tv;
  auto ell = [&](const std::vector<int>& r, const std::vector<int>& c, const std::vector<double>& v, int* slots,
                 std::vector<short>& d, std::vector<double>& e) {
    const long n = B->n;
    int K = 0;
    for (long i = 0; i < n; i++) K = std::max(K, r[i + 1] - r[i]);
    if (K == 0 || K > 8 || (long)K * n > nl + nl / 2) return false;
    d.assign((size_t)K * n, 0);
    e.assign((size_t)K * n, 0.0);
    for (long i = 0; i < n; i++)
      for (int j = r[i]; j < r[i + 1]; j++) {
        const long delta = (long)c[j] - i;
        if (delta < -32767 || delta > 32767) return false;
        const size_t o = (size_t)(j - r[i]) * n + i;
        d[o] = (short)delta;
        e[o] = v[j];
      }
    *slots = K;
    return true;
  };
  int lk = 0, tk = 0;
  const bool use_ell = nl > 0 && ell(rp, ci, va, &lk, ld, lv) && ell(trp, tci, tva, &tk, td, tv);
  cudaSetDevice(B->device);
  cudaStream_t st = B->stream;
  for (void* p : {(void*)B->lrowptr, (void*)B->lcolidx, (void*)B->trowptr, (void*)B->tcolidx, B->lvals, B->tvals,
                  (void*)B->rf, (void*)B->tf, (void*)B->zf, (void*)B->ldelta, (void*)B->tdelta})
    if (p) cudaFree(p);
  B->lrowptr = B->lcolidx = B->trowptr = B->tcolidx = nullptr;
  B->lvals = B->tvals = nullptr;
  B->rf = B->tf = B->zf = nullptr;
  B->ldelta = B->tdelta = nullptr;
  B->lslots = B->tslots = 0;
  double* tmp = nullptr;
  const size_t es = precision == TBSLA_F64 ? 8 : precision == TBSLA_F32 ? 4 : 2;
  B->lprec = precision;
  CK(alloc(&B->rf, B->n));
  CK(alloc(&B->tf, B->n));
  CK(alloc(&B->zf, B->n));
  if (use_ell) {
    const size_t nle = lv.size(), nte = tv.size();
    CK(alloc(&B->ldelta, nle));
    CK(alloc(&B->tdelta, nte));
    CK(cudaMalloc(&B->lvals, nle * es));
    CK(cudaMalloc(&B->tvals, nte * es));
    CK(alloc(&tmp, nle + nte));
    CK(cudaMemcpyAsync(B->ldelta, ld.data(), nle * 2, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B->tdelta, td.data(), nte * 2, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tmp, lv.data(), nle * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tmp + nle, tv.data(), nte * 8, cudaMemcpyHostToDevice, st));
    CK(convert_values(tmp, B->lvals, precision, (long)nle, st));
    CK(convert_values(tmp + nle, B->tvals, precision, (long)nte, st));
    B->lslots = lk;
    B->tslots = tk;
  } else {
    CK(alloc(&B->lrowptr, rp.size()));
    CK(alloc(&B->lcolidx, std::max<size_t>(ci.size(), 1)));
    CK(alloc(&B->trowptr, trp.size()));
    CK(alloc(&B->tcolidx, std::max<size_t>(tci.size(), 1)));
    CK(cudaMalloc(&B->lvals, std::max<size_t>(nl, 1) * es));
    CK(cudaMalloc(&B->tvals, std::max<size_t>(nl, 1) * es));
    CK(alloc(&tmp, std::max<size_t>(nl, 1) * 2));
    CK(cudaMemcpyAsync(B->lrowptr, rp.data(), rp.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B->lcolidx, ci.data(), ci.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B->trowptr, trp.data(), trp.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B->tcolidx, tci.data(), tci.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tmp, va.data(), nl * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tmp + nl, tva.data(), nl * 8, cudaMemcpyHostToDevice, st));
    CK(convert_values(tmp, B->lvals, precision, nl, st));
    CK(convert_values(tmp + nl, B->tvals, precision, nl, st));
  }
  CK(cudaStreamSynchronize(st));
  cudaFree(tmp);
  if (B->graph_pre == 2) B->graph_pre = -1;  // recapture with the new arrays
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_rows(const tbsla_batch* b, int* nsys, long* offsets) try {
  if (!b) return TBSLA_ERR_INVALID_ARG;
  if (nsys) *nsys = b->nsys;
  if (offsets) std::copy(b->off.begin(), b->off.end(), offsets);
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_cg(tbsla_batch* B, const double* rhs, double* x, int max_iterations, double rel_tol,
                   int precond, int refresh, int graph_iters, int* iterations, double* rel_residual) try {
  if (!B || !rhs || !x || max_iterations < 0 || rel_tol < 0 || precond < 0 || precond > 2 || refresh < 0 ||
      (precond == 2 && !B->rf && !B->dia_factor))
    return TBSLA_ERR_INVALID_ARG;
  cudaSetDevice(B->device);
  if (B->dia && (precond != 2 || B->dia_factor))
    return dia_solve(B, rhs, x, max_iterations, rel_tol, precond, refresh, iterations, rel_residual);
  B->last_engine = 0;
  B->last_graph = 1;
  B->last_st7 = 0;
  B->fallback_h.assign(B->nsys, 0);
  B->mode_h.assign(B->nsys, precond);
  if (precond == 2)
    for (int k = 0; k < B->nsys && k < (int)B->factor_fb.size(); k++)
      if (B->factor_fb[k]) {
        B->fallback_h[k] = B->factor_fb[k];
        B->mode_h[k] = 1;
      }
  const int K = graph_iters > 0 ? graph_iters : 10;
  const double tol2 = rel_tol * rel_tol;
  const CgBatch c = B->view(precond, tol2, max_iterations);
  cudaStream_t s = B->stream;
  const int ns = B->nsys;
  CK(cudaMemcpyAsync(B->b, rhs, B->n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->x, x, B->n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(B->status, 0, ns * sizeof(int), s));
  CK(cudaMemsetAsync(B->iters, 0, ns * sizeof(int), s));
  CK(cudaMemsetAsync(B->scal, 0, (size_t)kNScal * ns * 8, s));
  CK(cg_norms(c, s));
  // r = b - A x (FP64), z, rz; p = z
  CK(cg_true_residual(c, 1 << kActive, true, s));
  CK(cg_restart(c, true, s));
  if (!B->graph || B->graph_k != K || B->graph_pre != precond || B->graph_tol2 != tol2 ||
      B->graph_max != max_iterations) {
    // one eager iteration first: kernel attributes are set outside capture
    CK(cg_spmv_dot(c, s));
    CK(cg_update(c, s));
    CK(cg_factor_apply(c, 1 << kActive, c.rz_new, s));
    CK(cg_scalars(c, s));
    CK(cg_direction(c, s));
    int st = capture(B, c, K);
    if (st) return st;
    B->graph_k = K;
    B->graph_pre = precond;
    B->graph_tol2 = tol2;
    B->graph_max = max_iterations;
  }
  std::vector<int> hs(ns);
  long it = 0, last_refresh = 0;
  const bool narrow = B->prec != TBSLA_F64;
  for (;;) {
    CK(cudaGraphLaunch(B->graph, s));
    it += K;
    CK(cudaMemcpyAsync(hs.data(), B->status, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    bool active = false, verify = false;
    for (int v : hs) {
      active |= v == kActive;
      verify |= v == kVerify;
    }
    const bool refresh_due = narrow && refresh > 0 && active && it - last_refresh >= refresh;
    if (verify || refresh_due) {
      const int mask = (1 << kVerify) | (refresh_due ? 1 << kActive : 0);
      CK(cg_true_residual(c, mask, false, s));
      CK(cg_restart(c, false, s));
      if (refresh_due) last_refresh = it;
      CK(cudaMemcpyAsync(hs.data(), B->status, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      active = false;
      for (int v : hs) active |= v == kActive;
    }
    if (!active) break;
    if (it > (long)max_iterations + 4L * K + 8) break;  // every system has stopped by now
  }
  // true residual of systems that hit the limit, for the report
  CK(cg_true_residual(c, 1 << kStopped, false, s));
  std::vector<double> sc((size_t)kNScal * ns);
  CK(cudaMemcpyAsync(x, B->x, B->n * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(sc.data(), B->scal, sc.size() * 8, cudaMemcpyDeviceToHost, s));
  std::vector<int> hi(ns);
  CK(cudaMemcpyAsync(hi.data(), B->iters, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hs.data(), B->status, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  bool all = true;
  for (int k = 0; k < ns; k++) {
    const double bb = sc[4 * ns + k], rrt = sc[6 * ns + k];
    if (iterations) iterations[k] = hi[k];
    if (rel_residual) rel_residual[k] = bb > 0 ? std::sqrt(rrt / bb) : std::sqrt(rrt);
    all &= hs[k] == kDone;
  }
  return all ? TBSLA_OK : TBSLA_ERR_NOT_CONVERGED;
} TBSLA_API_CATCH

int tbsla_batch_factor_mpnn(tbsla_batch* B, tbsla_mpnn* net, int precision) try {
  if (!B || !net || precision < TBSLA_F64 || precision > TBSLA_BF16) return TBSLA_ERR_INVALID_ARG;
  if (!B->dia) return TBSLA_ERR_UNSUPPORTED;
  const int nsys = B->nsys;
  // L's slots: the diagonal, then A's negative deltas in descending order
  // (the pattern of tril(A))
  std::vector<int> ld((size_t)nsys * kDiaMaxDiag, 0);
  int KL = 1;
  for (int s = 0; s < nsys; s++) {
    int* q = ld.data() + (size_t)s * kDiaMaxDiag;
    int c = 1;
    for (int k = 0; k < B->K; k++) {
      const int d = B->adelta_h[(size_t)s * kDiaMaxDiag + k];
      if (d < 0) q[c++] = d;
    }
    std::sort(q + 1, q + c, [](int a, int b) { return a > b; });
    KL = std::max(KL, c);
  }
  cudaSetDevice(B->device);
  cudaStream_t st = B->stream;
  const int lprec = precision == TBSLA_BF16 ? TBSLA_BF16 : TBSLA_F32;
  B->dia_factor = false;
  if (!B->fdelta) CK(alloc(&B->fdelta, ld.size()));
  CK(lvals_reserve(B, (size_t)KL * B->n * (lprec == TBSLA_BF16 ? 2 : 4)));
  CK(cudaMemcpyAsync(B->fdelta, ld.data(), ld.size() * 4, cudaMemcpyHostToDevice, st));
  const int r = tbsla_impl::mpnn_factor_dia(net, B->n, B->K, B->a64_dia, B->adelta, B->row_sys, KL, B->fdelta,
                                            B->lvals_dia, lprec, st);
  if (r) return r;
  B->fdelta_h = ld;
  B->KL = KL;
  B->lprec_dia = lprec;
  B->dia_factor = true;
  B->factor_fb.assign(nsys, 0);
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_factor_dia(const tbsla_batch* B, int* slots, int* deltas, double* values) try {
  if (!B) return TBSLA_ERR_INVALID_ARG;
  if (!B->dia_factor) return TBSLA_ERR_UNSUPPORTED;
  if (slots) *slots = B->KL;
  if (deltas) std::copy(B->fdelta_h.begin(), B->fdelta_h.end(), deltas);
  if (values) {
    const size_t len = (size_t)B->KL * B->n;
    cudaSetDevice(B->device);
    if (B->lprec_dia == TBSLA_BF16) {
      std::vector<unsigned short> h(len);
      CK(cudaMemcpy(h.data(), B->lvals_dia, len * 2, cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < len; k++) {
        const unsigned u = (unsigned)h[k] << 16;
        float f;
        std::memcpy(&f, &u, 4);
        values[k] = f;
      }
    } else {
      std::vector<float> h(len);
      CK(cudaMemcpy(h.data(), B->lvals_dia, len * 4, cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < len; k++) values[k] = h[k];
    }
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_fallbacks(const tbsla_batch* B, int* fallback, int* precond_used) try {
  if (!B) return TBSLA_ERR_INVALID_ARG;
  for (int k = 0; k < B->nsys; k++) {
    if (fallback) fallback[k] = k < (int)B->fallback_h.size() ? B->fallback_h[k] : 0;
    if (precond_used) precond_used[k] = k < (int)B->mode_h.size() ? B->mode_h[k] : 0;
  }
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_set_ctas_per_sm(tbsla_batch* B, int ctas) try {
  if (!B || ctas < 0 || ctas > 32) return TBSLA_ERR_INVALID_ARG;
  B->ctas_per_sm = ctas;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_tuning(const tbsla_batch* B, int* rows_per_thread, int* ctas_per_sm) try {
  if (!B) return TBSLA_ERR_INVALID_ARG;
  if (rows_per_thread) *rows_per_thread = B->vec4 && !B->vec4_off ? 4 : 1;
  if (ctas_per_sm) *ctas_per_sm = B->ctas_per_sm;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_set_rows_per_thread(tbsla_batch* B, int rows) try {
  if (!B || (rows != 1 && rows != 4)) return TBSLA_ERR_INVALID_ARG;
  B->vec4_off = rows == 1;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_set_wait_limit(tbsla_batch* B, long long ns) try {
  if (!B || ns < 0) return TBSLA_ERR_INVALID_ARG;
  B->wait_ns = ns;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_engine(const tbsla_batch* B, int* persistent, int* graph, int* seven_point) try {
  if (!B) return TBSLA_ERR_INVALID_ARG;
  if (persistent) *persistent = B->last_engine;
  if (graph) *graph = B->last_graph;
  if (seven_point) *seven_point = B->last_st7;
  return TBSLA_OK;
} TBSLA_API_CATCH

int tbsla_batch_set_seven_point(tbsla_batch* B, int on) try {
  if (!B || (on != 0 && on != 1)) return TBSLA_ERR_INVALID_ARG;
  B->st7_off = on == 0;
  return TBSLA_OK;
} TBSLA_API_CATCH

}  // extern "C"

namespace tbsla_impl {

int dev_cg(tbsla_matrix* m, const double* b, double* x, int max_it, double rel_tol, int precond,
           int refresh, int* iterations, double* rel_residual) {
  tbsla_batch* B = nullptr;
  tbsla_matrix* one[1] = {m};
  int st = tbsla_batch_create(&B, one, 1, m->precision);
  if (st) return st;
  int it = 0;
  double rr = 0;
  st = tbsla_batch_cg(B, b, x, max_it, rel_tol, precond, refresh, 0, &it, &rr);
  tbsla_batch_destroy(B);
  if (iterations) *iterations = it;
  if (rel_residual) *rel_residual = rr;
  return st;
}

}  // namespace tbsla_impl
