// Drop-in for tbsla::cpp::MatrixCOO (src/cpp/include/tbsla/cpp/MatrixCOO.hpp of
// the reference) on the GB300 C ABI; see Matrix.hpp.
#ifndef TBSLA_GB300_CPP_MATRIXCOO
#define TBSLA_GB300_CPP_MATRIXCOO

#include <tbsla/cpp/Matrix.hpp>

namespace tbsla { namespace cpp {

class MatrixCOO : public Matrix {
  public:
    MatrixCOO();

    MatrixCOO(int n_row, int n_col, long nnz, const double* values, const int* row, const int* col);
    const double* get_values() const;
    const int* get_row() const;
    const int* get_col() const;
    // Matrix Market coordinate reader (MatrixCOO.cpp:206-278): 1-based
    // "row col value" lines after the "%%MatrixMarket matrix coordinate real"
    // banner and the size line; throws MatrixFormatReadException otherwise.
    void readMM(std::string name);
};

}}  // namespace tbsla::cpp

#endif
