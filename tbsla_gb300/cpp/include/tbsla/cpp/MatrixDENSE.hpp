// Drop-in for tbsla::cpp::MatrixDENSE (src/cpp/include/tbsla/cpp/MatrixDENSE.hpp of
// the reference) on the GB300 C ABI; see Matrix.hpp.
#ifndef TBSLA_GB300_CPP_MATRIXDENSE
#define TBSLA_GB300_CPP_MATRIXDENSE

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>

namespace tbsla { namespace cpp {

class MatrixDENSE : public Matrix {
  public:
    MatrixDENSE();
    explicit MatrixDENSE(const MatrixCOO& m);

};

}}  // namespace tbsla::cpp

#endif
