// ORACLE — test infrastructure only.
//
// extern "C" shim over the reference TBSLA C++ classes.  It is compiled
// together with the reference's own src/cpp/matrix/*.cpp and
// src/cpp/utils/*.cpp (where they lie in the reference tree, never copied)
// into oracle/_ref/libtbsla_ref.so by oracle/build.py.  Only
// tests/golden/make_golden.py (to record golden vectors) and bench.py's
// CPU-baseline leg load it.
//
// The reference classes keep their arrays protected; each handle here is a
// small subclass that re-exposes them, so arrays can be read back and set
// without going through a serialised stream.
#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>

namespace {

enum { F_COO = 0, F_SCOO = 1, F_CSR = 2, F_ELL = 3, F_DENSE = 4 };

struct Meta : public virtual tbsla::cpp::Matrix {
  void get_meta(int* m, long* nnz_out) const {
    m[0] = n_row; m[1] = n_col; m[2] = ln_row; m[3] = ln_col; m[4] = f_row;
    m[5] = f_col; m[6] = pr; m[7] = pc; m[8] = NR; m[9] = NC;
    *nnz_out = nnz;
  }
  void set_meta(const int* m, long nnz_in) {
    n_row = m[0]; n_col = m[1]; ln_row = m[2]; ln_col = m[3]; f_row = m[4];
    f_col = m[5]; pr = m[6]; pc = m[7]; NR = m[8]; NC = m[9];
    nnz = nnz_in;
  }
};

struct RCOO : tbsla::cpp::MatrixCOO, Meta {
  using tbsla::cpp::MatrixCOO::values; using tbsla::cpp::MatrixCOO::row; using tbsla::cpp::MatrixCOO::col;
};
struct RSCOO : tbsla::cpp::MatrixSCOO, Meta {
  RSCOO() {}
  explicit RSCOO(const tbsla::cpp::MatrixCOO& m) : tbsla::cpp::MatrixSCOO(m) {}
  using tbsla::cpp::MatrixSCOO::values; using tbsla::cpp::MatrixSCOO::row; using tbsla::cpp::MatrixSCOO::col;
};
struct RCSR : tbsla::cpp::MatrixCSR, Meta {
  RCSR() {}
  explicit RCSR(const tbsla::cpp::MatrixCOO& m) : tbsla::cpp::MatrixCSR(m) {}
  using tbsla::cpp::MatrixCSR::values; using tbsla::cpp::MatrixCSR::rowptr; using tbsla::cpp::MatrixCSR::colidx;
};
struct RELL : tbsla::cpp::MatrixELL, Meta {
  RELL() {}
  explicit RELL(const tbsla::cpp::MatrixCOO& m) : tbsla::cpp::MatrixELL(m) {}
  using tbsla::cpp::MatrixELL::values; using tbsla::cpp::MatrixELL::columns; using tbsla::cpp::MatrixELL::max_col;
};
struct RDENSE : tbsla::cpp::MatrixDENSE, Meta {
  RDENSE() {}
  explicit RDENSE(const tbsla::cpp::MatrixCOO& m) : tbsla::cpp::MatrixDENSE(m) {}
  using tbsla::cpp::MatrixDENSE::values;
};

struct Handle {
  int fmt;
  tbsla::cpp::Matrix* m;
  Meta* meta;
  void* obj;  // the concrete R* object (a virtual base cannot be downcast statically)
};

template <class T>
Handle* wrap(int fmt, T* p) { return new Handle{fmt, p, p, p}; }

template <class T>
T* as(Handle* h) { return static_cast<T*>(h->obj); }

// Silences the reference's progress prints while a call runs.
struct Quiet {
  std::streambuf* old;
  std::ostringstream sink;
  Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~Quiet() { std::cout.rdbuf(old); }
};

}  // namespace

extern "C" {

void* ref_new(int fmt) {
  switch (fmt) {
    case F_COO: { auto* p = new RCOO(); return wrap(fmt, p); }
    case F_SCOO: { auto* p = new RSCOO(); return wrap(fmt, p); }
    case F_CSR: { auto* p = new RCSR(); return wrap(fmt, p); }
    case F_ELL: { auto* p = new RELL(); return wrap(fmt, p); }
    case F_DENSE: { auto* p = new RDENSE(); return wrap(fmt, p); }
  }
  return nullptr;
}

void* ref_convert(void* coo, int fmt) {
  auto* h = static_cast<Handle*>(coo);
  const tbsla::cpp::MatrixCOO& c = *as<RCOO>(h);
  switch (fmt) {
    case F_SCOO: { auto* p = new RSCOO(c); return wrap(fmt, p); }
    case F_CSR: { auto* p = new RCSR(c); return wrap(fmt, p); }
    case F_ELL: { auto* p = new RELL(c); return wrap(fmt, p); }
    case F_DENSE: { auto* p = new RDENSE(c); return wrap(fmt, p); }
  }
  return nullptr;
}

void ref_delete(void* hp) {
  auto* h = static_cast<Handle*>(hp);
  switch (h->fmt) {
    case F_COO: delete as<RCOO>(h); break;
    case F_SCOO: delete as<RSCOO>(h); break;
    case F_CSR: delete as<RCSR>(h); break;
    case F_ELL: delete as<RELL>(h); break;
    case F_DENSE: delete as<RDENSE>(h); break;
  }
  delete h;
}

void ref_fill_cdiag(void* hp, int nr, int nc, int c, int pr, int pc, int NR, int NC) {
  Quiet q;
  static_cast<Handle*>(hp)->m->fill_cdiag(nr, nc, c, pr, pc, NR, NC);
}

void ref_fill_cqmat(void* hp, int nr, int nc, int c, double qv, unsigned s, int pr, int pc, int NR, int NC) {
  Quiet q;
  static_cast<Handle*>(hp)->m->fill_cqmat(nr, nc, c, qv, s, pr, pc, NR, NC);
}

void ref_fill_random(void* hp, int nr, int nc, double ratio, unsigned s, int pr, int pc, int NR, int NC) {
  Quiet q;
  static_cast<Handle*>(hp)->m->fill_random(nr, nc, ratio, s, pr, pc, NR, NC);
}

// meta[0..9] = n_row n_col ln_row ln_col f_row f_col pr pc NR NC, meta[10] = max_col (ELL)
void ref_info(void* hp, int* meta, long* nnz) {
  auto* h = static_cast<Handle*>(hp);
  h->meta->get_meta(meta, nnz);
  meta[10] = h->fmt == F_ELL ? as<RELL>(h)->max_col : 0;
}

// Pointers to the object's arrays (owned by the object).
void ref_arrays(void* hp, double** values, int** a, int** b) {
  auto* h = static_cast<Handle*>(hp);
  *a = *b = nullptr;
  switch (h->fmt) {
    case F_COO: { auto* p = as<RCOO>(h); *values = p->values; *a = p->row; *b = p->col; break; }
    case F_SCOO: { auto* p = as<RSCOO>(h); *values = p->values; *a = p->row; *b = p->col; break; }
    case F_CSR: { auto* p = as<RCSR>(h); *values = p->values; *a = p->rowptr; *b = p->colidx; break; }
    case F_ELL: { auto* p = as<RELL>(h); *values = p->values; *a = p->columns; break; }
    case F_DENSE: { auto* p = as<RDENSE>(h); *values = p->values; break; }
  }
}

// Replaces the object's arrays by copies of caller arrays (lengths follow
// the format: COO/SCOO nnz, CSR nnz + ln_row+1, ELL ln_row*max_col, DENSE
// ln_row*ln_col).
void ref_adopt(void* hp, const int* meta, long nnz, const double* values, const int* a, const int* b) {
  auto* h = static_cast<Handle*>(hp);
  h->meta->set_meta(meta, nnz);
  int ln_row = meta[2], ln_col = meta[3];
  switch (h->fmt) {
    case F_COO: case F_SCOO: {
      double*& v = h->fmt == F_COO ? as<RCOO>(h)->values : as<RSCOO>(h)->values;
      int*& r = h->fmt == F_COO ? as<RCOO>(h)->row : as<RSCOO>(h)->row;
      int*& c = h->fmt == F_COO ? as<RCOO>(h)->col : as<RSCOO>(h)->col;
      delete[] v; delete[] r; delete[] c;
      v = new double[nnz]; r = new int[nnz]; c = new int[nnz];
      std::memcpy(v, values, sizeof(double) * nnz);
      std::memcpy(r, a, sizeof(int) * nnz);
      std::memcpy(c, b, sizeof(int) * nnz);
      break;
    }
    case F_CSR: {
      auto* p = as<RCSR>(h);
      delete[] p->values; delete[] p->rowptr; delete[] p->colidx;
      p->values = new double[nnz]; p->rowptr = new int[ln_row + 1]; p->colidx = new int[nnz];
      std::memcpy(p->values, values, sizeof(double) * nnz);
      std::memcpy(p->rowptr, a, sizeof(int) * (ln_row + 1));
      std::memcpy(p->colidx, b, sizeof(int) * nnz);
      break;
    }
    case F_ELL: {
      auto* p = as<RELL>(h);
      p->max_col = meta[10];
      long n = (long)ln_row * p->max_col;
      delete[] p->values; delete[] p->columns;
      p->values = new double[n]; p->columns = new int[n];
      std::memcpy(p->values, values, sizeof(double) * n);
      std::memcpy(p->columns, a, sizeof(int) * n);
      break;
    }
    case F_DENSE: {
      auto* p = as<RDENSE>(h);
      long n = (long)ln_row * ln_col;
      delete[] p->values;
      p->values = new double[n];
      std::memcpy(p->values, values, sizeof(double) * n);
      break;
    }
  }
}

int ref_write(void* hp, const char* path) {
  std::ofstream os(path, std::ofstream::binary);
  if (!os.is_open()) return -1;
  static_cast<Handle*>(hp)->m->write(os);
  return 0;
}

int ref_read(void* hp, const char* path) {
  std::ifstream is(path, std::ifstream::binary);
  if (!is.is_open()) return -1;
  static_cast<Handle*>(hp)->m->read(is);
  return 0;
}

void ref_Ax(void* hp, double* r, const double* v, int vect_incr) {
  static_cast<Handle*>(hp)->m->Ax(r, v, vect_incr);
}

void ref_spmv(void* hp, const double* v, int vect_incr, double* out, int n_out) {
  double* r = static_cast<Handle*>(hp)->m->spmv(v, vect_incr);
  std::memcpy(out, r, sizeof(double) * n_out);
  delete[] r;
}

void ref_a_axpx_(void* hp, const double* v, int vect_incr, double* out, int n_out) {
  double* r = static_cast<Handle*>(hp)->m->a_axpx_(v, vect_incr);
  std::memcpy(out, r, sizeof(double) * n_out);
  delete[] r;
}

void ref_AAxpAx(void* hp, double* r, double* v, double* buffer, int vect_incr) {
  static_cast<Handle*>(hp)->m->AAxpAx(r, v, buffer, vect_incr);
}

void ref_AAxpAxpx(void* hp, double* r, double* v, double* buffer, int vect_incr) {
  static_cast<Handle*>(hp)->m->AAxpAxpx(r, v, buffer, vect_incr);
}

void ref_get_col_sums(void* hp, double* s) {
  Quiet q;
  static_cast<Handle*>(hp)->m->get_col_sums(s);
}

void ref_normalize_cols(void* hp, double* s) {
  Quiet q;
  static_cast<Handle*>(hp)->m->normalize_cols(s);
}

// CSR only (MatrixCSR.cpp:1269-1334).
void ref_dense_multiply(void* hp, const double* B, double* Cm, int cols) {
  as<RCSR>(static_cast<Handle*>(hp))->dense_multiply(B, Cm, cols);
}

void ref_row_max_abs(void* hp, double* out) {
  Quiet q;
  as<RCSR>(static_cast<Handle*>(hp))->get_row_max_abs(out);
}

void ref_row_sums(void* hp, double* out) {
  Quiet q;
  as<RCSR>(static_cast<Handle*>(hp))->get_row_sums(out);
}

void ref_normalize_rows(void* hp, double* s) {
  Quiet q;
  as<RCSR>(static_cast<Handle*>(hp))->normalize_rows(s);
}

void ref_apply_exponential(void* hp, double* max_abs, int base) {
  Quiet q;
  as<RCSR>(static_cast<Handle*>(hp))->apply_exponential(max_abs, base);
}

}  // extern "C"
