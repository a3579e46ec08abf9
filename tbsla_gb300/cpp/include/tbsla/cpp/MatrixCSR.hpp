// Drop-in for tbsla::cpp::MatrixCSR (src/cpp/include/tbsla/cpp/MatrixCSR.hpp of
// the reference) on the GB300 C ABI; see Matrix.hpp.
#ifndef TBSLA_GB300_CPP_MATRIXCSR
#define TBSLA_GB300_CPP_MATRIXCSR

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>

namespace tbsla { namespace cpp {

class MatrixCSR : public Matrix {
  public:
    MatrixCSR();
    explicit MatrixCSR(const MatrixCOO& m);
    // Adopts copies of the arrays (the reference constructor of this
    // signature ignores them, MatrixCSR.cpp:21-38).
    MatrixCSR(int n_row, int n_col, double* values, int* rowptr, int* colidx);
    // PageRank (result: new[] array, caller delete[]s) and CG of the GPU path
    double* page_rank(double beta, double epsilon, int max_iterations, int& nb_iterations_done);
    void CG(const double* b, double* x, int max_iterations, int& nb_iterations_done,
            double rel_tol = 1e-8, int precond = 0);
    // C = A B (MatrixCSR.cpp:1269-1281), on the GPU
    void dense_multiply(const double* B, double* C, int cols_B);
    // MatrixCSR.hpp:33: base -1 (the default) is e^x
    void apply_exponential(double* max_abs, int base = -1) override;
};

}}  // namespace tbsla::cpp

#endif
