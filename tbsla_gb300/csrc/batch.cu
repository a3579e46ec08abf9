// Batched CG: block-diagonal device copy of many SPD systems and the solve
// loop around the kernels of kernels/cg.cu.
//
// HBM layout of a batch: the systems' CSR arrays concatenated (rowptr
// int32[n+1], colidx int32[nnz] shifted to global columns, values in the
// storage precision and in FP64), the row-block partition of the SpMV and
// the row chunks of the vector kernels (neither crosses a system boundary,
// each carries its system id), the Jacobi diagonal, six FP64 vectors (b, x,
// r, z, p, q) and per-system scalars.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "device.hpp"
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

  ~tbsla_batch() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    if (graph) cudaGraphExecDestroy(graph);
    void* ps[] = {rowptr, colidx, vals64, blocks, block_sys, chunks, chunk_sys, dinv, b, x, r, z, p, q,
                  scal, status, iters, lrowptr, lcolidx, trowptr, tcolidx, lvals, tvals, rf, tf,
                  ldelta, tdelta, zf};
    for (void* v : ps)
      if (v) cudaFree(v);
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

}  // namespace

extern "C" {

int tbsla_batch_create(tbsla_batch** out, tbsla_matrix* const* systems, int nsys, int precision) {
  if (!out || !systems || nsys <= 0 || precision < TBSLA_F64 || precision > TBSLA_BF16)
    return TBSLA_ERR_INVALID_ARG;
  for (int s = 0; s < nsys; s++)
    if (!systems[s]) return TBSLA_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return TBSLA_ERR_NO_DEVICE;
  }
  auto* B = new tbsla_batch();
  cudaGetDevice(&B->device);
  int st = st_of(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  if (!st) st = build_batch(B, systems, nsys, precision);
  if (st) {
    delete B;
    return st;
  }
  *out = B;
  return TBSLA_OK;
}

int tbsla_batch_destroy(tbsla_batch* b) {
  delete b;
  return TBSLA_OK;
}

int tbsla_batch_set_factors(tbsla_batch* B, tbsla_matrix* const* factors, int nsys, int precision) {
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
}

int tbsla_batch_rows(const tbsla_batch* b, int* nsys, long* offsets) {
  if (!b) return TBSLA_ERR_INVALID_ARG;
  if (nsys) *nsys = b->nsys;
  if (offsets) std::copy(b->off.begin(), b->off.end(), offsets);
  return TBSLA_OK;
}

int tbsla_batch_cg(tbsla_batch* B, const double* rhs, double* x, int max_iterations, double rel_tol,
                   int precond, int refresh, int graph_iters, int* iterations, double* rel_residual) {
  if (!B || !rhs || !x || max_iterations < 0 || rel_tol < 0 || precond < 0 || precond > 2 || refresh < 0 ||
      (precond == 2 && !B->rf))
    return TBSLA_ERR_INVALID_ARG;
  cudaSetDevice(B->device);
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
}

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
