// Implementation of the C++ drop-in classes over the C ABI.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sstream>

#include <unistd.h>

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

namespace tbsla { namespace cpp {

void Matrix::check(int status, const char* what) {
  if (status != TBSLA_OK) throw GpuError(status, what);
}

Matrix::Matrix(int format) : h_(nullptr), format_(format) {
  check(tbsla_matrix_create(&h_, format), "create");
}

Matrix::Matrix(int format, tbsla_matrix* adopt) : h_(adopt), format_(format) {}

Matrix::~Matrix() { tbsla_matrix_destroy(h_); }

tbsla_info Matrix::info() const {
  tbsla_info i;
  check(tbsla_matrix_info(h_, &i), "info");
  return i;
}

long Matrix::out_len() const {
  tbsla_info i = info();
  return format_ == TBSLA_COO ? i.n_row : i.ln_row;
}

double* Matrix::spmv(const double* v, int vect_incr) const {
  long n = out_len();
  double* r = new double[n > 0 ? n : 1]();
  int st = tbsla_spmv(h_, r, v, vect_incr);
  if (st != TBSLA_OK) {
    delete[] r;
    check(st, "spmv");
  }
  return r;
}

void Matrix::Ax(double* r, const double* v, int vect_incr) const { check(tbsla_Ax(h_, r, v, vect_incr), "Ax"); }

void Matrix::make_stochastic(double* s) { check(tbsla_make_stochastic(h_, s), "make_stochastic"); }

void Matrix::AAxpAx(double* r, double* v, double* buffer, int vect_incr) const {
  check(tbsla_AAxpAx(h_, r, v, buffer, vect_incr), "AAxpAx");
}

void Matrix::AAxpAxpx(double* r, double* v, double* buffer, int vect_incr) const {
  check(tbsla_AAxpAxpx(h_, r, v, buffer, vect_incr), "AAxpAxpx");
}

double* Matrix::a_axpx_(const double* v, int vect_incr) const {
  long n = out_len();
  double* r = new double[n > 0 ? n : 1]();
  int st = tbsla_a_axpx_(h_, r, v, vect_incr);
  if (st != TBSLA_OK) {
    delete[] r;
    check(st, "a_axpx_");
  }
  return r;
}

// Stream I/O goes through a temporary file so that the byte layout is the
// single implementation behind tbsla_matrix_write / tbsla_matrix_read.
namespace {
struct TmpFile {
  std::string path;
  TmpFile() {
    char buf[] = "/tmp/tbsla_gb300_XXXXXX";
    int fd = mkstemp(buf);
    if (fd >= 0) close(fd);
    path = buf;
  }
  ~TmpFile() { std::remove(path.c_str()); }
};
}  // namespace

std::ostream& Matrix::write(std::ostream& os) {
  TmpFile t;
  check(tbsla_matrix_write(h_, t.path.c_str(), 0), "write");
  std::ifstream in(t.path, std::ios::binary);
  os << in.rdbuf();
  return os;
}

std::istream& Matrix::read(std::istream& is, std::size_t, std::size_t) {
  // Copy exactly one matrix record: header first, then the counted arrays.
  TmpFile t;
  std::ofstream out(t.path, std::ios::binary);
  auto copy = [&](size_t bytes) {
    std::vector<char> b(bytes);
    is.read(b.data(), (std::streamsize)bytes);
    if ((size_t)is.gcount() != bytes) throw GpuError(TBSLA_ERR_IO, "read");
    out.write(b.data(), (std::streamsize)bytes);
    return b;
  };
  copy(6 * sizeof(int) + sizeof(long) + 4 * sizeof(int));
  int arrays = format_ == TBSLA_DENSE ? 1 : format_ == TBSLA_ELL ? 2 : 3;
  if (format_ == TBSLA_ELL) copy(sizeof(int));
  int elem[3];
  switch (format_) {
    case TBSLA_COO: case TBSLA_SCOO: case TBSLA_CSR: elem[0] = 8; elem[1] = 4; elem[2] = 4; break;
    case TBSLA_ELL: elem[0] = 8; elem[1] = 4; break;
    default: elem[0] = 8;
  }
  for (int a = 0; a < arrays; a++) {
    std::vector<char> s = copy(sizeof(size_t));
    size_t count;
    std::memcpy(&count, s.data(), sizeof(size_t));
    copy(count * (size_t)elem[a]);
  }
  out.close();
  check(tbsla_matrix_read(h_, t.path.c_str(), 0), "read");
  return is;
}

std::ostream& Matrix::print(std::ostream& os) const {
  static const char* names[] = {"COO", "SCOO", "CSR", "ELL", "DENSE"};
  tbsla_info i = info();
  os << "-----------------\n------ " << names[format_] << " ------\n-----------------\n";
  os << "number of rows             -  n_row   : " << i.n_row << "\n";
  os << "number of columns          -  n_col   : " << i.n_col << "\n";
  os << "local number of rows       -  ln_row  : " << i.ln_row << "\n";
  os << "local number of columns    -  ln_col  : " << i.ln_col << "\n";
  os << "first row                  -  f_row   : " << i.f_row << "\n";
  os << "first column               -  f_col   : " << i.f_col << "\n";
  os << "number of non-zero elts    -  nnz     : " << i.nnz << "\n";
  os << "block position (row)       -  pr      : " << i.pr << "\n";
  os << "block position (column)    -  pc      : " << i.pc << "\n";
  os << "number of blocks (row)     -  NR      : " << i.NR << "\n";
  os << "number of blocks (column)  -  NC      : " << i.NC << "\n";
  if (format_ == TBSLA_ELL) os << "maximum number of columns  -  max_col : " << i.max_col << "\n";
  os << "-----------------" << std::endl;
  return os;
}

std::ostream& Matrix::print_as_dense(std::ostream& os) {
  tbsla_info i = info();
  std::vector<double> d((size_t)i.ln_row * i.ln_col, 0.0);
  const double* v;
  const int *a, *b;
  check(tbsla_matrix_arrays(h_, &v, &a, &b), "arrays");
  switch (format_) {
    case TBSLA_COO: case TBSLA_SCOO:
      for (long k = 0; k < i.nnz; k++) d[(size_t)(a[k] - i.f_row) * i.ln_col + (b[k] - i.f_col)] += v[k];
      break;
    case TBSLA_CSR:
      if (i.nnz) for (int r = 0; r < i.ln_row; r++)
        for (int k = a[r]; k < a[r + 1]; k++) d[(size_t)r * i.ln_col + (b[k] - i.f_col)] += v[k];
      break;
    case TBSLA_ELL:
      for (int r = 0; r < i.ln_row; r++)
        for (int k = 0; k < i.max_col; k++)
          d[(size_t)r * i.ln_col + (a[(size_t)r * i.max_col + k] - i.f_col)] += v[(size_t)r * i.max_col + k];
      break;
    default:
      if (v) std::memcpy(d.data(), v, d.size() * sizeof(double));
  }
  os << std::fixed << std::setprecision(1);
  for (int r = 0; r < i.ln_row; r++) {
    for (int c = 0; c < i.ln_col; c++) os << std::setw(6) << d[(size_t)r * i.ln_col + c] << "  ";
    os << "\n";
  }
  return os;
}

void Matrix::NUMAinit() { check(tbsla_matrix_upload(h_), "upload"); }

void Matrix::fill_cdiag(int n_row, int n_col, int cdiag, int pr, int pc, int NR, int NC) {
  check(tbsla_matrix_fill_cdiag(h_, n_row, n_col, cdiag, pr, pc, NR, NC), "fill_cdiag");
}

void Matrix::fill_cqmat(int n_row, int n_col, int c, double q, unsigned int seed_mult, int pr, int pc, int NR,
                        int NC) {
  check(tbsla_matrix_fill_cqmat(h_, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC), "fill_cqmat");
}

void Matrix::fill_random(int n_row, int n_col, double nnz_ratio, unsigned int seed_mult, int pr, int pc,
                         int NR, int NC) {
  check(tbsla_matrix_fill_random(h_, n_row, n_col, nnz_ratio, seed_mult, pr, pc, NR, NC), "fill_random");
}

void Matrix::fill_brain(int, int, int*, std::vector<std::vector<double> >,
                        std::vector<std::unordered_map<int, std::vector<int> > >, unsigned int, int, int, int,
                        int) {
  throw GpuError(TBSLA_ERR_UNSUPPORTED, "fill_brain");
}

void Matrix::get_row_sums(double* buffer) { check(tbsla_get_row_sums(h_, buffer), "get_row_sums"); }
void Matrix::normalize_rows(double* s) { check(tbsla_normalize_rows(h_, s), "normalize_rows"); }
void Matrix::get_col_sums(double* buffer) { check(tbsla_get_col_sums(h_, buffer), "get_col_sums"); }
void Matrix::normalize_cols(double* s) { check(tbsla_normalize_cols(h_, s), "normalize_cols"); }
void Matrix::get_row_max_abs(double* max_abs) { check(tbsla_get_row_max_abs(h_, max_abs), "get_row_max_abs"); }
void Matrix::apply_exponential(double* max_abs, int base) {
  check(tbsla_apply_exponential(h_, max_abs, base), "apply_exponential");
}

void Matrix::set_precision(int precision) { check(tbsla_matrix_set_precision(h_, precision), "set_precision"); }

// ---- formats ------------------------------------------------------------------

namespace {
tbsla_matrix* convert(const Matrix& coo, int format) {
  tbsla_matrix* out = nullptr;
  int st = tbsla_matrix_convert(&out, coo.handle(), format);
  if (st != TBSLA_OK) throw GpuError(st, "convert");
  return out;
}
tbsla_info square_info(int n_row, int n_col, long nnz) {
  tbsla_info i{};
  i.n_row = i.ln_row = n_row;
  i.n_col = i.ln_col = n_col;
  i.nnz = nnz;
  i.NR = i.NC = 1;
  return i;
}
}  // namespace

MatrixCOO::MatrixCOO() : Matrix(TBSLA_COO) {}
MatrixCOO::MatrixCOO(int n_row, int n_col, long nnz, const double* values, const int* row, const int* col)
    : Matrix(TBSLA_COO) {
  tbsla_info i = square_info(n_row, n_col, nnz);
  check(tbsla_matrix_set_coo(h_, &i, values, row, col), "set_coo");
}
MatrixCOO::MatrixCOO(int n_row, int n_col, double*, int*, int*) : Matrix(TBSLA_COO) {
  tbsla_info i = square_info(n_row, n_col, 0);
  check(tbsla_matrix_set_coo(h_, &i, nullptr, nullptr, nullptr), "set_coo");
}
MatrixCOO::MatrixCOO(int n_row, int n_col, long n_values) : Matrix(TBSLA_COO) {
  if (n_values < 0) throw GpuError(TBSLA_ERR_INVALID_ARG, "MatrixCOO");
  std::vector<double> v((size_t)n_values, 0.0);
  std::vector<int> z((size_t)n_values, 0);
  tbsla_info i = square_info(n_row, n_col, n_values);
  check(tbsla_matrix_set_coo(h_, &i, v.data(), z.data(), z.data()), "set_coo");
}
MatrixCOO::MatrixCOO(int n_row, int n_col) : Matrix(TBSLA_COO) {
  tbsla_info i = square_info(n_row, n_col, 0);
  check(tbsla_matrix_set_coo(h_, &i, nullptr, nullptr, nullptr), "set_coo");
}
const double* MatrixCOO::get_values() const {
  const double* v;
  check(tbsla_matrix_arrays(h_, &v, nullptr, nullptr), "arrays");
  return v;
}
const int* MatrixCOO::get_row() const {
  const int* a;
  check(tbsla_matrix_arrays(h_, nullptr, &a, nullptr), "arrays");
  return a;
}
const int* MatrixCOO::get_col() const {
  const int* b;
  check(tbsla_matrix_arrays(h_, nullptr, nullptr, &b), "arrays");
  return b;
}

void MatrixCOO::readMM(std::string name) {
  std::ifstream is(name);
  std::string line;
  if (!std::getline(is, line) || line.rfind("%%MatrixMarket matrix coordinate", 0) != 0)
    throw MatrixFormatReadException();
  bool symmetric = line.find("symmetric") != std::string::npos;
  bool pattern = line.find("pattern") != std::string::npos;
  while (std::getline(is, line) && !line.empty() && line[0] == '%') {
  }
  std::istringstream hdr(line);
  long nr, nc, ne;
  if (!(hdr >> nr >> nc >> ne)) throw MatrixFormatReadException();
  std::vector<int> r, c;
  std::vector<double> v;
  for (long k = 0; k < ne; k++) {
    long i, j;
    double x = 1.0;
    if (!(is >> i >> j)) throw MatrixFormatReadException();
    if (!pattern && !(is >> x)) throw MatrixFormatReadException();
    r.push_back((int)i - 1);
    c.push_back((int)j - 1);
    v.push_back(x);
    if (symmetric && i != j) {
      r.push_back((int)j - 1);
      c.push_back((int)i - 1);
      v.push_back(x);
    }
  }
  tbsla_info inf = square_info((int)nr, (int)nc, (long)v.size());
  check(tbsla_matrix_set_coo(h_, &inf, v.data(), r.data(), c.data()), "set_coo");
}

MatrixSCOO::MatrixSCOO() : Matrix(TBSLA_SCOO) {}
MatrixSCOO::MatrixSCOO(const MatrixCOO& m) : Matrix(TBSLA_SCOO, convert(m, TBSLA_SCOO)) {}
MatrixSCOO::MatrixSCOO(int n_row, int n_col, long nnz, const double* values, const int* row, const int* col)
    : Matrix(TBSLA_SCOO) {
  tbsla_info i = square_info(n_row, n_col, nnz);
  check(tbsla_matrix_set_coo(h_, &i, values, row, col), "set_coo");
}

MatrixSCOO::MatrixSCOO(int n_row, int n_col, int) : MatrixSCOO(n_row, n_col) {}
MatrixSCOO::MatrixSCOO(int n_row, int n_col) : Matrix(TBSLA_SCOO) {
  tbsla_info i = square_info(n_row, n_col, 0);
  check(tbsla_matrix_set_coo(h_, &i, nullptr, nullptr, nullptr), "set_coo");
}
void MatrixSCOO::push_back(int r, int c, double v) { check(tbsla_matrix_push_back(h_, r, c, v), "push_back"); }

MatrixCSR::MatrixCSR() : Matrix(TBSLA_CSR) {}
void MatrixCSR::apply_exponential(double* max_abs, int base) { Matrix::apply_exponential(max_abs, base); }
MatrixCSR::MatrixCSR(const MatrixCOO& m) : Matrix(TBSLA_CSR, convert(m, TBSLA_CSR)) {}
MatrixCSR::MatrixCSR(int n_row, int n_col, double* values, int* rowptr, int* colidx) : Matrix(TBSLA_CSR) {
  tbsla_info i = square_info(n_row, n_col, rowptr ? rowptr[n_row] : 0);
  check(tbsla_matrix_set_csr(h_, &i, values, rowptr, colidx), "set_csr");
}

double* MatrixCSR::page_rank(double beta, double epsilon, int max_iterations, int& nb_iterations_done) {
  long n = get_n_row();
  double* r = new double[n > 0 ? n : 1]();
  double err = 0;
  int st = tbsla_page_rank(h_, beta, epsilon, max_iterations, r, &nb_iterations_done, &err);
  if (st != TBSLA_OK && st != TBSLA_ERR_NOT_CONVERGED) {
    delete[] r;
    check(st, "page_rank");
  }
  return r;
}

void MatrixCSR::CG(const double* b, double* x, int max_iterations, int& nb_iterations_done, double rel_tol,
                   int precond) {
  double rr = 0;
  int st = tbsla_cg(h_, b, x, max_iterations, rel_tol, precond, 50, &nb_iterations_done, &rr);
  if (st != TBSLA_OK && st != TBSLA_ERR_NOT_CONVERGED) check(st, "cg");
}

void MatrixCSR::dense_multiply(const double* B, double* C, int cols_B) {
  check(tbsla_dense_multiply(h_, B, C, cols_B), "dense_multiply");
}

MatrixELL::MatrixELL() : Matrix(TBSLA_ELL) {}
MatrixELL::MatrixELL(const MatrixCOO& m) : Matrix(TBSLA_ELL, convert(m, TBSLA_ELL)) {}

MatrixDENSE::MatrixDENSE() : Matrix(TBSLA_DENSE) {}
MatrixDENSE::MatrixDENSE(const MatrixCOO& m) : Matrix(TBSLA_DENSE, convert(m, TBSLA_DENSE)) {}

}}  // namespace tbsla::cpp
