// Binary matrix files in the reference's wire format, byte for byte
// (MatrixCOO.cpp:144-204, MatrixSCOO.cpp:166-226, MatrixCSR.cpp:236-295,
// MatrixELL.cpp:208-259, MatrixDENSE.cpp:88-127): a header of
//   int n_row, n_col, ln_row, ln_col, f_row, f_col; long nnz; int pr, pc, NR, NC;
// (ELL appends int max_col), then each array as a size_t element count
// followed by the raw elements, in host byte order.  Unlike the reference,
// reading checks every count against the header and reports a short or
// inconsistent file instead of reading past it.
#include <cstdio>
#include <cstdint>

#include "matrix.hpp"

namespace tbsla_impl {

namespace {

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

template <class T>
bool put(FILE* f, const T& v) {
  return fwrite(&v, sizeof(T), 1, f) == 1;
}

template <class T>
bool put_array(FILE* f, const T* p, size_t n) {
  size_t sz = n;
  if (!put(f, sz)) return false;
  return n == 0 || fwrite(p, sizeof(T), n, f) == n;
}

template <class T>
bool get(FILE* f, T& v) {
  return fread(&v, sizeof(T), 1, f) == 1;
}

// Reads one counted array; the count must equal `expect` unless expect < 0.
template <class T>
bool get_array(FILE* f, Buf<T>& b, long expect) {
  size_t sz;
  if (!get(f, sz)) return false;
  if (expect >= 0 && sz != (size_t)expect) return false;
  if (sz > ((size_t)1 << 40)) return false;
  b.resize(sz);
  return sz == 0 || fread(b.data(), sizeof(T), sz, f) == sz;
}

}  // namespace

int write_file(const tbsla_matrix* m, const char* path, bool append) {
  File F;
  F.f = fopen(path, append ? "ab" : "wb");
  if (!F.f) return TBSLA_ERR_IO;
  const tbsla_info& I = m->info;
  FILE* f = F.f;
  bool ok = put(f, I.n_row) && put(f, I.n_col) && put(f, I.ln_row) && put(f, I.ln_col) &&
            put(f, I.f_row) && put(f, I.f_col) && put(f, I.nnz) && put(f, I.pr) &&
            put(f, I.pc) && put(f, I.NR) && put(f, I.NC);
  size_t nnz = (size_t)I.nnz;
  switch (m->format) {
    case TBSLA_COO:
    case TBSLA_SCOO:
      if (m->values.size() < nnz || m->idx0.size() < nnz || m->idx1.size() < nnz) return TBSLA_ERR_BAD_MATRIX;
      ok = ok && put_array(f, m->values.data(), nnz) && put_array(f, m->idx0.data(), nnz) &&
           put_array(f, m->idx1.data(), nnz);
      break;
    case TBSLA_CSR:
      if (m->values.size() < nnz || m->idx1.size() < nnz || m->idx0.size() < (size_t)I.ln_row + 1)
        return TBSLA_ERR_BAD_MATRIX;
      ok = ok && put_array(f, m->values.data(), nnz) &&
           put_array(f, m->idx0.data(), (size_t)I.ln_row + 1) && put_array(f, m->idx1.data(), nnz);
      break;
    case TBSLA_ELL: {
      size_t n = value_len(m);
      if (m->values.size() < n || m->idx0.size() < n) return TBSLA_ERR_BAD_MATRIX;
      ok = ok && put(f, I.max_col) && put_array(f, m->values.data(), n) &&
           put_array(f, m->idx0.data(), n);
      break;
    }
    case TBSLA_DENSE: {
      size_t n = value_len(m);
      if (m->values.size() < n) return TBSLA_ERR_BAD_MATRIX;
      ok = ok && put_array(f, m->values.data(), n);
      break;
    }
    default:
      return TBSLA_ERR_INVALID_ARG;
  }
  return ok ? TBSLA_OK : TBSLA_ERR_IO;
}

int read_file(tbsla_matrix* m, const char* path, long offset) {
  File F;
  F.f = fopen(path, "rb");
  if (!F.f) return TBSLA_ERR_IO;
  FILE* f = F.f;
  if (offset > 0 && fseek(f, offset, SEEK_SET) != 0) return TBSLA_ERR_IO;
  tbsla_info I{};
  bool ok = get(f, I.n_row) && get(f, I.n_col) && get(f, I.ln_row) && get(f, I.ln_col) &&
            get(f, I.f_row) && get(f, I.f_col) && get(f, I.nnz) && get(f, I.pr) &&
            get(f, I.pc) && get(f, I.NR) && get(f, I.NC);
  if (!ok || I.nnz < 0 || I.ln_row < 0 || I.ln_col < 0) return TBSLA_ERR_IO;
  m->invalidate();
  Buf<double> v;
  Buf<int> a, b;
  switch (m->format) {
    case TBSLA_COO:
    case TBSLA_SCOO:
      ok = get_array(f, v, I.nnz) && get_array(f, a, I.nnz) && get_array(f, b, I.nnz);
      break;
    case TBSLA_CSR:
      ok = get_array(f, v, I.nnz) && get_array(f, a, (long)I.ln_row + 1) && get_array(f, b, I.nnz);
      break;
    case TBSLA_ELL:
      ok = get(f, I.max_col) && I.max_col >= 0 &&
           get_array(f, v, (long)I.ln_row * I.max_col) && get_array(f, a, (long)I.ln_row * I.max_col);
      break;
    case TBSLA_DENSE:
      ok = get_array(f, v, (long)I.ln_row * I.ln_col);
      break;
    default:
      return TBSLA_ERR_INVALID_ARG;
  }
  if (!ok) return TBSLA_ERR_IO;
  m->info = I;
  m->values = std::move(v);
  m->idx0 = std::move(a);
  m->idx1 = std::move(b);
  return TBSLA_OK;
}

}  // namespace tbsla_impl
