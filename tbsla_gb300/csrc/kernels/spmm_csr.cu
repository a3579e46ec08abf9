// CSR times a dense block, and the sparse-softmax helpers of MatrixCSR.
//
// csr_dense_multiply replaces tbsla::cpp::MatrixCSR::dense_multiply
// (src/cpp/matrix/MatrixCSR.cpp:1269-1281): C = A B with B (n_col x k) and
// C (n_row x k) row-major, B indexed by the column as stored.  One warp per
// row; lanes take 32 columns of C at a time, so each entry of the row costs
// one coalesced load of a B row segment and one FMA per lane, in entry
// order.  csr_row_max_abs / csr_apply_exponential replace get_row_max_abs
// (:1283-1312) and apply_exponential (:1315-1334): one warp per row.
// csr_row_sums / csr_normalize_rows replace get_row_sums (:1147-1164: each
// row summed in entry order, so one thread per row) and normalize_rows
// (:1177-1190: a_ij / s_i, or 0 where s_i = 0; one warp per row).
#include <algorithm>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;

__device__ __forceinline__ long warp_id() { return ((long)blockIdx.x * NT + threadIdx.x) / kWarp; }
__device__ __forceinline__ long warp_count() { return (long)gridDim.x * NT / kWarp; }

template <class V>
__global__ void __launch_bounds__(NT) k_spmm(const V* __restrict__ vals, const int* __restrict__ rowptr,
                                            const int* __restrict__ colidx, int n_row, const double* __restrict__ B,
                                            int k, double* __restrict__ Cm) {
  const int lane = threadIdx.x & 31;
  for (long i = warp_id(); i < n_row; i += warp_count()) {
    const int s = rowptr[i], e = rowptr[i + 1];
    for (int c0 = 0; c0 < k; c0 += kWarp) {
      const int c = c0 + lane;
      double acc = 0;
      for (int j = s; j < e; j++) {
        const double v = widen(vals[j]);
        const long col = colidx[j];
        if (c < k) acc = fma_rn(v, B[col * k + c], acc);
      }
      if (c < k) Cm[i * k + c] = acc;
    }
  }
}

__global__ void __launch_bounds__(NT) k_row_max_abs(const double* __restrict__ vals, const int* __restrict__ rowptr,
                                                   int n_row, double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (long i = warp_id(); i < n_row; i += warp_count()) {
    double m = 0;
    for (int j = rowptr[i] + lane; j < rowptr[i + 1]; j += kWarp) m = fmax(m, fabs(vals[j]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) out[i] = m;
  }
}

__global__ void __launch_bounds__(NT) k_apply_exp(double* __restrict__ vals, const int* __restrict__ rowptr,
                                                 int n_row, const double* __restrict__ max_abs, int base) {
  const int lane = threadIdx.x & 31;
  for (long i = warp_id(); i < n_row; i += warp_count()) {
    const double sh = max_abs ? max_abs[i] : 0.0;
    for (int j = rowptr[i] + lane; j < rowptr[i + 1]; j += kWarp) {
      const double z = vals[j];
      if (z == 0) continue;
      const double a = max_abs ? z - sh : z;
      vals[j] = base <= 0 ? exp(a) : pow((double)base, a);
    }
  }
}

__global__ void __launch_bounds__(NT) k_row_sums(const double* __restrict__ vals, const int* __restrict__ rowptr,
                                                int n_row, double* __restrict__ out) {
  for (long i = (long)blockIdx.x * NT + threadIdx.x; i < n_row; i += (long)gridDim.x * NT) {
    double sum = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) sum = add_rn(sum, vals[j]);
    out[i] = sum;
  }
}

__global__ void __launch_bounds__(NT) k_normalize_rows(double* __restrict__ vals, const int* __restrict__ rowptr,
                                                      int n_row, const double* __restrict__ s) {
  const int lane = threadIdx.x & 31;
  for (long i = warp_id(); i < n_row; i += warp_count()) {
    const double si = s[i];
    for (int j = rowptr[i] + lane; j < rowptr[i + 1]; j += kWarp) vals[j] = si != 0 ? vals[j] / si : 0.0;
  }
}

int warp_grid(long rows) { return (int)std::max<long>(1, std::min<long>((rows + 7) / 8, 152L * 16)); }

}  // namespace

cudaError_t csr_dense_multiply(const void* vals, int prec, const int* rowptr, const int* colidx, int n_row,
                               const double* B, int k, double* Cm, cudaStream_t s) {
  if (n_row <= 0 || k <= 0) return cudaSuccess;
  const int g = warp_grid(n_row);
  switch (prec) {
    case kF64: k_spmm<double><<<g, NT, 0, s>>>(static_cast<const double*>(vals), rowptr, colidx, n_row, B, k, Cm); break;
    case kF32: k_spmm<float><<<g, NT, 0, s>>>(static_cast<const float*>(vals), rowptr, colidx, n_row, B, k, Cm); break;
    case kBF16:
      k_spmm<__nv_bfloat16><<<g, NT, 0, s>>>(static_cast<const __nv_bfloat16*>(vals), rowptr, colidx, n_row, B, k,
                                             Cm);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t csr_row_max_abs(const double* vals, const int* rowptr, int n_row, double* out, cudaStream_t s) {
  if (n_row <= 0) return cudaSuccess;
  k_row_max_abs<<<warp_grid(n_row), NT, 0, s>>>(vals, rowptr, n_row, out);
  return cudaGetLastError();
}

cudaError_t csr_apply_exponential(double* vals, const int* rowptr, int n_row, const double* max_abs, int base,
                                  cudaStream_t s) {
  if (n_row <= 0) return cudaSuccess;
  k_apply_exp<<<warp_grid(n_row), NT, 0, s>>>(vals, rowptr, n_row, max_abs, base);
  return cudaGetLastError();
}

cudaError_t csr_row_sums(const double* vals, const int* rowptr, int n_row, double* out, cudaStream_t s) {
  if (n_row <= 0) return cudaSuccess;
  const int g = (int)std::max<long>(1, std::min<long>((n_row + NT - 1) / NT, 152L * 16));
  k_row_sums<<<g, NT, 0, s>>>(vals, rowptr, n_row, out);
  return cudaGetLastError();
}

cudaError_t csr_normalize_rows(double* vals, const int* rowptr, int n_row, const double* sums, cudaStream_t s) {
  if (n_row <= 0) return cudaSuccess;
  k_normalize_rows<<<warp_grid(n_row), NT, 0, s>>>(vals, rowptr, n_row, sums);
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
