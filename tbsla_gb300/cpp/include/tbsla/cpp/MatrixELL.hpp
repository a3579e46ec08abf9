// Drop-in for tbsla::cpp::MatrixELL (src/cpp/include/tbsla/cpp/MatrixELL.hpp of
// the reference) on the GB300 C ABI; see Matrix.hpp.
#ifndef TBSLA_GB300_CPP_MATRIXELL
#define TBSLA_GB300_CPP_MATRIXELL

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>

namespace tbsla { namespace cpp {

class MatrixELL : public Matrix {
  public:
    MatrixELL();
    explicit MatrixELL(const MatrixCOO& m);
    int get_max_col() const { return info().max_col; }
};

}}  // namespace tbsla::cpp

#endif
