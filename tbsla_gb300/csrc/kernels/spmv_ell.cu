// ELL SpMV on a column-major device copy.
//
// Replaces tbsla::cpp::MatrixELL::Ax (src/cpp/matrix/MatrixELL.cpp:181-205):
// y_i = sum over all max_col slots of values[i][j] * v[columns[i][j] - f_col],
// pads included, overwriting y; with f_col != 0 a negative shifted index is
// clamped to 0 as the reference does.
//
// The reference stores ELL row-major (values[i*max_col + j]); the device
// copy is transposed once at upload to slot-major (values[j*ln_row + i]) so
// that a warp's 32 threads -- 32 consecutive rows -- read 32 consecutive
// elements of every slot.  One thread sums one row in slot order with each
// product rounded before the add: the reference's rounding, bit for bit.
#include <algorithm>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;

template <class V, bool SHIFT>
__global__ void __launch_bounds__(NT) k_ell(const V* __restrict__ vals, const int* __restrict__ cols,
                                           int ln_row, int max_col, int f_col,
                                           const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * NT + threadIdx.x;
  if (i >= ln_row) return;
  const uint64_t pol = policy_evict_first();
  double acc = 0;
  int j = 0;
  for (; j + 4 <= max_col; j += 4) {
    const size_t k = (size_t)j * ln_row + i;
    int c[4];
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      c[u] = ld_stream(cols + k + (size_t)u * ln_row, pol) - f_col;
      v[u] = widen(ld_stream(vals + k + (size_t)u * ln_row, pol));
      if (SHIFT && c[u] < 0) c[u] = 0;
    }
    double xv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) xv[u] = ld_gather(x + c[u]);
#pragma unroll
    for (int u = 0; u < 4; u++) acc = add_rn(acc, mul_rn(v[u], xv[u]));
  }
  for (; j < max_col; j++) {
    const size_t k = (size_t)j * ln_row + i;
    int c = ld_stream(cols + k, pol) - f_col;
    if (SHIFT && c < 0) c = 0;
    acc = add_rn(acc, mul_rn(widen(ld_stream(vals + k, pol)), ld_gather(x + c)));
  }
  y[i] = acc;
}

template <class V>
__global__ void k_ell_transpose(const double* __restrict__ vrm, const int* __restrict__ crm,
                                V* __restrict__ vcm, int* __restrict__ ccm, int ln_row, int max_col) {
  const size_t n = (size_t)ln_row * max_col;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / max_col, j = k % max_col;
    vcm[j * ln_row + i] = narrow<V>(vrm[k]);
    ccm[j * ln_row + i] = crm[k];
  }
}

template <class V>
cudaError_t launch(const void* vals, const int* cols, int ln_row, int max_col, int f_col,
                   const double* x, double* y, cudaStream_t s) {
  const int grid = (ln_row + NT - 1) / NT;
  if (f_col != 0)
    k_ell<V, true><<<grid, NT, 0, s>>>(static_cast<const V*>(vals), cols, ln_row, max_col, f_col, x, y);
  else
    k_ell<V, false><<<grid, NT, 0, s>>>(static_cast<const V*>(vals), cols, ln_row, max_col, 0, x, y);
  return cudaGetLastError();
}

}  // namespace

cudaError_t ell_spmv(const void* vals, int prec, const int* cols, int ln_row, int max_col,
                     int f_col, const double* x, double* y, cudaStream_t s) {
  if (ln_row == 0) return cudaSuccess;
  switch (prec) {
    case kF64: return launch<double>(vals, cols, ln_row, max_col, f_col, x, y, s);
    case kF32: return launch<float>(vals, cols, ln_row, max_col, f_col, x, y, s);
    case kBF16: return launch<__nv_bfloat16>(vals, cols, ln_row, max_col, f_col, x, y, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t ell_transpose(const double* vals_rm, const int* cols_rm, void* vals_cm, int prec,
                          int* cols_cm, int ln_row, int max_col, cudaStream_t s) {
  const size_t n = (size_t)ln_row * max_col;
  if (n == 0) return cudaSuccess;
  const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 32);
  switch (prec) {
    case kF64: k_ell_transpose<double><<<grid, 256, 0, s>>>(vals_rm, cols_rm, (double*)vals_cm, cols_cm, ln_row, max_col); break;
    case kF32: k_ell_transpose<float><<<grid, 256, 0, s>>>(vals_rm, cols_rm, (float*)vals_cm, cols_cm, ln_row, max_col); break;
    case kBF16: k_ell_transpose<__nv_bfloat16><<<grid, 256, 0, s>>>(vals_rm, cols_rm, (__nv_bfloat16*)vals_cm, cols_cm, ln_row, max_col); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
