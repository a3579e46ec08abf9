// Host-side format logic: array lengths, validation, and the converting
// constructors from COO.
#include <algorithm>
#include <numeric>
#include <vector>

#include "device.hpp"
#include "matrix.hpp"

namespace tbsla_impl {

size_t value_len(const tbsla_matrix* m) {
  const tbsla_info& I = m->info;
  switch (m->format) {
    case TBSLA_COO:
    case TBSLA_SCOO:
    case TBSLA_CSR:
      return m->values.size();
    case TBSLA_ELL:
      return (size_t)I.ln_row * (size_t)I.max_col;
    case TBSLA_DENSE:
      return (size_t)I.ln_row * (size_t)I.ln_col;
  }
  return 0;
}

namespace {
// true when every index in [b, e) of idx, shifted by -off, lies in [0, len)
bool all_in(const int* idx, long b, long e, long off, long len) {
  bool ok = true;
  parallel_for(e - b, [&](long lb, long le) {
    bool loc = true;
    for (long k = b + lb; k < b + le; k++) {
      long v = (long)idx[k] - off;
      if (v < 0 || v >= len) { loc = false; break; }
    }
    if (!loc) ok = false;  // benign race: any writer stores false
  });
  return ok;
}
}  // namespace

int validate(const tbsla_matrix* m) {
  const tbsla_info& I = m->info;
  if (I.ln_row < 0 || I.ln_col < 0 || I.n_row < 0 || I.n_col < 0 || I.nnz < 0)
    return TBSLA_ERR_BAD_MATRIX;
  switch (m->format) {
    case TBSLA_CSR: {
      if (I.nnz == 0) return TBSLA_OK;  // Ax never reads the arrays
      if (m->idx0.size() != (size_t)I.ln_row + 1) return TBSLA_ERR_BAD_MATRIX;
      const int* rp = m->idx0.data();
      if (rp[0] < 0) return TBSLA_ERR_BAD_MATRIX;
      for (long i = 0; i < I.ln_row; i++)
        if (rp[i + 1] < rp[i]) return TBSLA_ERR_BAD_MATRIX;
      long end = rp[I.ln_row];
      if ((size_t)end > m->idx1.size() || (size_t)end > m->values.size()) return TBSLA_ERR_BAD_MATRIX;
      if (!all_in(m->idx1.data(), rp[0], end, I.f_col, I.ln_col)) return TBSLA_ERR_BAD_MATRIX;
      return TBSLA_OK;
    }
    case TBSLA_COO:
    case TBSLA_SCOO: {
      size_t n = (size_t)I.nnz;
      if (m->values.size() < n || m->idx0.size() < n || m->idx1.size() < n) return TBSLA_ERR_BAD_MATRIX;
      bool scoo = m->format == TBSLA_SCOO;
      long rows = scoo ? I.ln_row : I.n_row, cols = scoo ? I.ln_col : I.n_col;
      long roff = scoo ? I.f_row : 0, coff = scoo ? I.f_col : 0;
      // Rows are checked per call against vect_incr; here only the columns.
      if (!all_in(m->idx1.data(), 0, (long)n, coff, cols)) return TBSLA_ERR_BAD_MATRIX;
      (void)rows;
      (void)roff;
      return TBSLA_OK;
    }
    case TBSLA_ELL: {
      if (I.nnz == 0 || I.max_col == 0) return TBSLA_OK;
      size_t n = value_len(m);
      if (m->values.size() < n || m->idx0.size() < n) return TBSLA_ERR_BAD_MATRIX;
      const int* c = m->idx0.data();
      bool ok = true;
      parallel_for((long)n, [&](long b, long e) {
        for (long k = b; k < e; k++) {
          long v = (long)c[k] - I.f_col;
          if (I.f_col != 0 && v < 0) v = 0;  // MatrixELL.cpp:199
          if (v < 0 || v >= I.ln_col) { ok = false; break; }
        }
      });
      return ok ? TBSLA_OK : TBSLA_ERR_BAD_MATRIX;
    }
    case TBSLA_DENSE: {
      if (I.nnz == 0) return TBSLA_OK;
      return m->values.size() >= value_len(m) ? TBSLA_OK : TBSLA_ERR_BAD_MATRIX;
    }
  }
  return TBSLA_ERR_INVALID_ARG;
}

// Converting constructors MatrixCSR/ELL/SCOO/DENSE(const MatrixCOO&).
int convert_from_coo(tbsla_matrix* out, const tbsla_matrix* coo, int format, bool device) {
  if (coo->format != TBSLA_COO) return TBSLA_ERR_INVALID_ARG;
  const tbsla_info& C = coo->info;
  long nnz = C.nnz;
  const int* row = coo->idx0.data();
  const int* col = coo->idx1.data();
  const double* val = coo->values.data();
  if (nnz > 0) {
    if (coo->values.size() < (size_t)nnz || coo->idx0.size() < (size_t)nnz ||
        coo->idx1.size() < (size_t)nnz)
      return TBSLA_ERR_BAD_MATRIX;
    if (!all_in(row, 0, nnz, 0, C.n_row) || !all_in(col, 0, nnz, 0, C.n_col))
      return TBSLA_ERR_BAD_MATRIX;
  }
  out->invalidate();
  out->format = format;
  out->info = tbsla_info{};
  tbsla_info& I = out->info;
  // MatrixCSR.cpp:50-60 (same in the other converting constructors)
  I.n_row = I.ln_row = C.n_row;
  I.n_col = I.ln_col = C.n_col;
  I.f_row = C.f_row;
  I.f_col = C.f_col;
  I.pr = C.pr; I.pc = C.pc; I.NR = C.NR; I.NC = C.NC;
  I.nnz = nnz;
  out->values.clear(); out->idx0.clear(); out->idx1.clear();

  if (format == TBSLA_SCOO) {  // MatrixSCOO.cpp:75-101: plain copy
    out->values.assign(val, nnz);
    out->idx0.assign(row, nnz);
    out->idx1.assign(col, nnz);
    return TBSLA_OK;
  }
  if (format == TBSLA_DENSE) {  // MatrixDENSE.cpp:15-37: scatter-add in storage order
    if (device) {  // the same sums on the GPU, duplicates added in storage order
      out->values.resize((size_t)I.ln_row * I.ln_col);
      return dev_coo_to_dense(row, col, val, nnz, I.ln_row, I.ln_col, out->values.data());
    }
    out->values.zeros((size_t)I.ln_row * I.ln_col);
    for (long k = 0; k < nnz; k++) out->values[(size_t)row[k] * I.ln_col + col[k]] += val[k];
    return TBSLA_OK;
  }
  if (format != TBSLA_CSR && format != TBSLA_ELL) return TBSLA_ERR_INVALID_ARG;

  // Entries ordered by (row, col), ties in storage order (compare_row,
  // src/cpp/utils/csr.cpp:3-8): a stable counting sort by row, then a
  // stable sort by column inside each row.
  int n_row = C.n_row;
  std::vector<long> start(n_row + 1, 0);
  std::vector<long> perm(nnz);
  if (device) {  // the same order from a radix sort on the GPU (kernels/sort.cu)
    int st = dev_coo_order(row, col, nnz, n_row, C.n_col, start.data(), perm.data());
    if (st) return st;
  } else {
    for (long k = 0; k < nnz; k++) start[row[k] + 1]++;
    for (int i = 0; i < n_row; i++) start[i + 1] += start[i];
    {
      std::vector<long> pos(start.begin(), start.end() - 1);
      for (long k = 0; k < nnz; k++) perm[pos[row[k]]++] = k;
    }
    parallel_for(n_row, [&](long b, long e) {
      for (long i = b; i < e; i++)
        std::stable_sort(perm.begin() + start[i], perm.begin() + start[i + 1],
                         [&](long a, long c) { return col[a] < col[c]; });
    });
  }

  if (format == TBSLA_CSR) {  // MatrixCSR.cpp:62-95
    out->idx0.resize(n_row + 1);
    for (int i = 0; i <= n_row; i++) out->idx0[i] = (int)start[i];
    out->idx1.resize(nnz);
    out->values.resize(nnz);
    parallel_for(nnz, [&](long b, long e) {
      for (long k = b; k < e; k++) {
        out->idx1[k] = col[perm[k]];
        out->values[k] = val[perm[k]];
      }
    });
    return TBSLA_OK;
  }
  // ELL, MatrixELL.cpp:38-78: max_col = longest row; rows packed left,
  // pads are column 0 / value 0.
  if (nnz == 0) {
    I.max_col = 0;
    return TBSLA_OK;
  }
  long mc = 0;
  for (int i = 0; i < n_row; i++) mc = std::max(mc, start[i + 1] - start[i]);
  I.max_col = (int)mc;
  out->values.zeros((size_t)n_row * mc);
  out->idx0.zeros((size_t)n_row * mc);
  parallel_for(n_row, [&](long b, long e) {
    for (long i = b; i < e; i++)
      for (long k = start[i]; k < start[i + 1]; k++) {
        size_t slot = (size_t)i * mc + (k - start[i]);
        out->idx0[slot] = col[perm[k]];
        out->values[slot] = val[perm[k]];
      }
  });
  return TBSLA_OK;
}

}  // namespace tbsla_impl
