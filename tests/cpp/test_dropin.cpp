// Known-answer test of the C++ drop-in classes (tbsla::cpp::Matrix*), written
// as a reference user would: the cdiag sweep of the reference's
// src/cpp/tests/test_Ax_cdiag.cpp (every format, filled directly and
// converted from COO, shapes (10,10) (5,10) (10,5) c = 0..12 and (30,30)
// (20,30) (30,20) c = 0..24 step 2), checked exactly against the closed form
// of src/cpp/utils/array.cpp:17-30; plus spmv (new[] result), a_axpx_, a
// stream write/read round trip and SCOO blocks built by push_back.  Exits
// non-zero on the first mismatch.
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <vector>

using namespace tbsla::cpp;

static std::vector<double> closed_form(int nr, int nc, int c, const std::vector<double>& v) {
  std::vector<double> r(nr, 0.0);
  for (int i = 0; i < nr; i++) {
    if (c == 0) {
      if (i < nc) r[i] = v[i];
      continue;
    }
    if (i - c >= 0 && i - c < nc) r[i] += v[i - c];
    if (i + c < nc) r[i] += v[i + c];
  }
  return r;
}

static int failures = 0;

static void check(Matrix& m, int nr, int nc, int c, const char* what) {
  std::vector<double> v(nc), r(nr, 0.0);
  for (int i = 0; i < nc; i++) v[i] = i;
  m.Ax(r.data(), v.data());
  std::vector<double> e = closed_form(nr, nc, c, v);
  for (int i = 0; i < nr; i++)
    if (r[i] != e[i]) {
      std::printf("error %s nr=%d nc=%d c=%d i=%d r=%g exp=%g\n", what, nr, nc, c, i, r[i], e[i]);
      failures++;
      return;
    }
  double* s = m.spmv(v.data());
  for (int i = 0; i < nr; i++)
    if (s[i] != e[i]) {
      std::printf("spmv error %s nr=%d nc=%d c=%d i=%d\n", what, nr, nc, c, i);
      failures++;
      break;
    }
  delete[] s;
}

static void test_cdiag(int nr, int nc, int c) {
  MatrixCOO coo;
  coo.fill_cdiag(nr, nc, c);
  check(coo, nr, nc, c, "COO");
  MatrixSCOO scoo(coo);
  check(scoo, nr, nc, c, "SCOO(COO)");
  MatrixSCOO scoo2;
  scoo2.fill_cdiag(nr, nc, c);
  check(scoo2, nr, nc, c, "SCOO");
  MatrixCSR csr(coo);
  check(csr, nr, nc, c, "CSR(COO)");
  MatrixCSR csr2;
  csr2.fill_cdiag(nr, nc, c);
  check(csr2, nr, nc, c, "CSR");
  MatrixELL ell(coo);
  check(ell, nr, nc, c, "ELL(COO)");
  MatrixELL ell2;
  ell2.fill_cdiag(nr, nc, c);
  check(ell2, nr, nc, c, "ELL");
  MatrixDENSE dense(coo);
  check(dense, nr, nc, c, "DENSE(COO)");
  MatrixDENSE dense2;
  dense2.fill_cdiag(nr, nc, c);
  check(dense2, nr, nc, c, "DENSE");
  // the same entries appended one by one (MatrixSCOO::push_back)
  MatrixSCOO scoo3(nr, nc, (int)coo.get_nnz());
  const double* cv = coo.get_values();
  const int* cr = coo.get_row();
  const int* cc = coo.get_col();
  for (long k = 0; k < coo.get_nnz(); k++) scoo3.push_back(cr[k], cc[k], cv[k]);
  check(scoo3, nr, nc, c, "SCOO(push_back)");
}

int main() {
  for (int i = 0; i <= 12; i++) test_cdiag(10, 10, i);
  for (int i = 0; i <= 12; i++) test_cdiag(5, 10, i);
  for (int i = 0; i <= 12; i++) test_cdiag(10, 5, i);
  for (int i = 0; i <= 12; i++) test_cdiag(30, 30, 2 * i);
  for (int i = 0; i <= 12; i++) test_cdiag(20, 30, 2 * i);
  for (int i = 0; i <= 12; i++) test_cdiag(30, 20, 2 * i);

  // a_axpx_ on a square cdiag matrix: A(Av + v), v = 2i + 1
  {
    int n = 30, c = 3;
    MatrixCSR m;
    m.fill_cdiag(n, n, c);
    std::vector<double> v(n);
    for (int i = 0; i < n; i++) v[i] = 2 * i + 1;
    std::vector<double> t = closed_form(n, n, c, v);
    for (int i = 0; i < n; i++) t[i] += v[i];
    std::vector<double> e = closed_form(n, n, c, t);
    double* r = m.a_axpx_(v.data());
    for (int i = 0; i < n; i++)
      if (r[i] != e[i]) {
        std::printf("a_axpx_ error i=%d\n", i);
        failures++;
        break;
      }
    delete[] r;
  }
  // stream round trip in the reference wire format
  {
    MatrixCSR m;
    m.fill_cqmat(40, 40, 5, 0.5, 2);
    std::stringstream ss;
    m.write(ss);
    MatrixCSR m2;
    m2.read(ss);
    if (m2.get_nnz() != m.get_nnz() || m2.get_n_row() != 40) {
      std::printf("stream round trip error\n");
      failures++;
    }
    std::vector<double> v(40, 1.0), a(40), b(40);
    m.Ax(a.data(), v.data());
    m2.Ax(b.data(), v.data());
    if (a != b) {
      std::printf("stream round trip Ax error\n");
      failures++;
    }
  }
  if (failures) return 1;
  std::printf("=== finished without error ===\n");
  return 0;
}
