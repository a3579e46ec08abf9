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
    // MatrixCOO.hpp:13: the reference adopts the three pointers but leaves
    // nnz uninitialised (MatrixCOO.cpp:45-65), so their length is unknown.
    // Here the matrix is n_row x n_col with no entries and the arrays are
    // neither read nor adopted: pass the length with the overload above.
    MatrixCOO(int n_row, int n_col, double* values, int* row, int* col);
    // MatrixCOO.hpp:14: n_values zero entries at (0, 0) (the reference's
    // zero-filled arrays of that length).
    MatrixCOO(int n_row, int n_col, long n_values);
    // MatrixCOO.hpp:15: an n_row x n_col matrix with no entries.
    MatrixCOO(int n_row, int n_col);
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
