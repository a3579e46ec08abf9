// Source-compatible C++ drop-in for tbsla::cpp::Matrix
// (src/cpp/include/tbsla/cpp/Matrix.hpp:11-57 of the reference), backed by
// the GB300 C ABI (include/tbsla_gb300.h).  An object owns one tbsla_matrix
// handle: the reference's host arrays plus a lazily built device copy; Ax /
// spmv / a_axpx_ / AAxpAx / AAxpAxpx run on the GPU with host pointers, as
// the reference's run on the host.
//
// Differences from the reference, all deliberate:
//  - errors raise tbsla::cpp::GpuError (status code inside) instead of
//    undefined behaviour (the reference has no error convention);
//  - NUMAinit() builds the device copy (the GPU analogue of first-touch
//    placement);
//  - get_vectorization() names the CUDA target;
//  - fill_brain (the brain-model generator, not on the SpMV / PageRank / CG
//    path) raises GpuError(TBSLA_ERR_UNSUPPORTED); the sparse-softmax
//    helpers get_row_sums / normalize_rows / get_row_max_abs /
//    apply_exponential and MatrixCSR::dense_multiply run on the GPU for CSR
//    (other formats raise TBSLA_ERR_UNSUPPORTED);
//  - get_row_sums / normalize_rows do not print the reference's progress
//    lines.
#ifndef TBSLA_GB300_CPP_MATRIX
#define TBSLA_GB300_CPP_MATRIX

#include <cstddef>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "tbsla_gb300.h"

namespace tbsla { namespace cpp {

struct GpuError : public std::runtime_error {
  int status;
  GpuError(int s, const std::string& what)
      : std::runtime_error(what + ": " + tbsla_status_string(s)), status(s) {}
};

struct MatrixFormatReadException : public std::exception {
  const char* what() const throw() { return "This Matrix format import is not implemented!"; }
};

class Matrix {
 public:
  virtual ~Matrix();
  Matrix(const Matrix&) = delete;
  Matrix& operator=(const Matrix&) = delete;
  friend std::ostream& operator<<(std::ostream& os, const Matrix& m) { return m.print(os); }

  // Matrix.hpp:14-15: spmv returns a new[] array the caller delete[]s.
  virtual double* spmv(const double* v, int vect_incr = 0) const;
  virtual void Ax(double* r, const double* v, int vect_incr = 0) const;
  void make_stochastic(double* s);
  void AAxpAx(double* r, double* v, double* buffer, int vect_incr = 0) const;
  void AAxpAxpx(double* r, double* v, double* buffer, int vect_incr = 0) const;
  double* a_axpx_(const double* v, int vect_incr = 0) const;
  // Declared as in Matrix.hpp:20 of the reference, which defines it nowhere:
  // a program that calls it links against neither library.
  double*& saxpy(const double* x, double* y);

  int get_n_row() const { return info().n_row; }
  int get_n_col() const { return info().n_col; }
  int get_f_row() const { return info().f_row; }
  int get_f_col() const { return info().f_col; }
  int get_ln_row() const { return info().ln_row; }
  int get_ln_col() const { return info().ln_col; }
  int get_pr() const { return info().pr; }
  int get_pc() const { return info().pc; }
  int get_NR() const { return info().NR; }
  int get_NC() const { return info().NC; }
  long int get_nnz() const { return info().nnz; }
  std::string get_vectorization() const { return "CUDA sm_103a"; }

  virtual std::ostream& write(std::ostream& os);
  virtual std::istream& read(std::istream& is, std::size_t pos = 0, std::size_t n = 1);
  virtual std::ostream& print(std::ostream& os) const;
  virtual std::ostream& print_as_dense(std::ostream& os);
  virtual void NUMAinit();

  virtual void fill_cdiag(int n_row, int n_col, int cdiag, int pr = 0, int pc = 0, int NR = 1, int NC = 1);
  virtual void fill_cqmat(int n_row, int n_col, int c, double q, unsigned int seed_mult = 1, int pr = 0,
                          int pc = 0, int NR = 1, int NC = 1);
  virtual void fill_random(int n_row, int n_col, double nnz_ratio, unsigned int seed_mult = 1, int pr = 0,
                           int pc = 0, int NR = 1, int NC = 1);
  virtual void fill_brain(int n_row, int n_col, int* neuron_type,
                          std::vector<std::vector<double> > proba_conn,
                          std::vector<std::unordered_map<int, std::vector<int> > > brain_struct,
                          unsigned int seed_mult, int pr = 0, int pc = 0, int NR = 1, int NC = 1);

  virtual void get_row_sums(double* buffer);
  virtual void normalize_rows(double* s);
  virtual void get_col_sums(double* buffer);
  virtual void normalize_cols(double* s);
  virtual void get_row_max_abs(double* max_abs);
  virtual void apply_exponential(double* max_abs, int base);

  // GB300 additions
  void set_precision(int precision);  // TBSLA_F64 / TBSLA_F32 / TBSLA_BF16 device values
  tbsla_matrix* handle() const { return h_; }
  tbsla_info info() const;

 protected:
  explicit Matrix(int format);
  Matrix(int format, tbsla_matrix* adopt);
  static void check(int status, const char* what);
  long out_len() const;
  tbsla_matrix* h_;
  int format_;
};

}}  // namespace tbsla::cpp

#endif
