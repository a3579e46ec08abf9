// Drop-in for tbsla::cpp::MatrixSCOO (src/cpp/include/tbsla/cpp/MatrixSCOO.hpp of
// the reference) on the GB300 C ABI; see Matrix.hpp.
#ifndef TBSLA_GB300_CPP_MATRIXSCOO
#define TBSLA_GB300_CPP_MATRIXSCOO

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>

namespace tbsla { namespace cpp {

class MatrixSCOO : public Matrix {
  public:
    MatrixSCOO();
    explicit MatrixSCOO(const MatrixCOO& m);
    MatrixSCOO(int n_row, int n_col, long nnz, const double* values, const int* row, const int* col);
    // MatrixSCOO.hpp:15-16: an n_row x n_col block with no entries yet (the
    // reference allocates n_values uninitialised slots for push_back).
    MatrixSCOO(int n_row, int n_col, int n_values);
    MatrixSCOO(int n_row, int n_col);
    // MatrixSCOO.hpp:25: appends the entry (r, c, v); declared but never
    // defined by the reference.
    void push_back(int r, int c, double v);
};

}}  // namespace tbsla::cpp

#endif
