// DENSE GEMV and the small vector / preparation kernels of the path.
//
// dense_gemv and dense_gemv_df replace tbsla::cpp::MatrixDENSE::Ax
// (src/cpp/matrix/MatrixDENSE.cpp:77-86): r_i += sum_j A_ij v_j on a
// row-major ln_row x ln_col matrix.  FP64 values: a CTA per row for rows of
// at least 2048 columns, a warp per row below; 16-byte loads (pairs of
// doubles) where the row start is 16-byte aligned, x through L1 (every row
// reuses it), one FP64 multiply-add per entry (GB300's FP64 pipe, not HBM,
// bounds an FP64 GEMV), partial sums combined in a fixed order and added to
// r_i.  Values of every precision whose magnitudes lie in [2^-40, 2^40]
// (checked once at upload): double-float arithmetic on the FP32 pipes
// (dense_gemv_df, below); an FP64 value is split on load, on the integer
// pipe, into two floats that hold it to 2^-48.
#include <algorithm>

#include "common.cuh"
#include "df.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;
constexpr int kDenseU = 4;  // 16-byte loads in flight per thread, CTA-per-row kernel
// rows per CTA pass, double-float kernel; 2 (each xh / xl load serving two
// rows) measured 0.366 / 0.329 ms against 0.362 / 0.321 ms with 1 (FP32 /
// BF16 values, 32768 x 16384)
constexpr int kDenseDfRows = 1;

__device__ __forceinline__ double2 ld_stream2(const double* p, uint64_t pol) {
  double2 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(pol));
  return v;
}

template <class V>
__global__ void __launch_bounds__(NT) k_dense(const V* __restrict__ A, int ln_row, int ln_col,
                                             const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x % kWarp;
  const int gw = (blockIdx.x * NT + threadIdx.x) / kWarp;
  const int nw = gridDim.x * NT / kWarp;
  const uint64_t pol = policy_evict_first();
  for (int row = gw; row < ln_row; row += nw) {
    const V* a = A + (size_t)row * ln_col;
    double acc = 0;
    int j = lane;
    for (; j + 3 * kWarp < ln_col; j += 4 * kWarp) {
      double v0 = widen(ld_stream(a + j, pol)), v1 = widen(ld_stream(a + j + kWarp, pol));
      double v2 = widen(ld_stream(a + j + 2 * kWarp, pol)), v3 = widen(ld_stream(a + j + 3 * kWarp, pol));
      acc = fma_rn(v0, __ldg(x + j), acc);
      acc = fma_rn(v1, __ldg(x + j + kWarp), acc);
      acc = fma_rn(v2, __ldg(x + j + 2 * kWarp), acc);
      acc = fma_rn(v3, __ldg(x + j + 3 * kWarp), acc);
    }
    for (; j < ln_col; j += kWarp) acc = fma_rn(widen(ld_stream(a + j, pol)), __ldg(x + j), acc);
    acc = warp_sum(acc);
    if (lane == 0) y[row] = add_rn(y[row], acc);
  }
}

// FP64 rows of at least 2*NT*U columns with 16-byte aligned starts: one CTA
// per row (launched with a CTA per row; the loop also accepts fewer CTAs),
// every thread with U 16-byte loads in flight.
// A warp per row leaves the last round of rows to a fraction of the warps
// (32768 rows over 9728 warps: 4 rounds for some, 3 for the rest); a CTA per
// row spreads each row over the whole CTA and the rows over 8x fewer
// workers, so the last round is a small share of the launch.  Partial sums:
// warp butterfly, then the NT/32 warp sums in a fixed order (a double-
// buffered slot per row parity, one barrier per row).
template <int U>
__global__ void __launch_bounds__(NT) k_dense_rows_f64x2(const double* __restrict__ A, int ln_row,
                                                        int ln_col, const double* __restrict__ x,
                                                        double* __restrict__ y) {
  __shared__ double s_part[2][NT / kWarp];
  const int lane = threadIdx.x % kWarp, warp = threadIdx.x / kWarp;
  const uint64_t pol = policy_evict_first();
  const int half = ln_col / 2;
  const double2* x2 = reinterpret_cast<const double2*>(x);
  int parity = 0;
  for (int row = blockIdx.x; row < ln_row; row += gridDim.x, parity ^= 1) {
    const double* a = A + (size_t)row * ln_col;
    double acc0 = 0, acc1 = 0;
    int j = threadIdx.x;
    for (; j + (U - 1) * NT < half; j += U * NT) {
      double2 av[U], bv[U];
#pragma unroll
      for (int u = 0; u < U; u++) av[u] = ld_stream2(a + 2 * (j + u * NT), pol);
#pragma unroll
      for (int u = 0; u < U; u++) bv[u] = __ldg(x2 + j + u * NT);
#pragma unroll
      for (int u = 0; u < U; u++) {
        acc0 = fma_rn(av[u].x, bv[u].x, acc0);
        acc1 = fma_rn(av[u].y, bv[u].y, acc1);
      }
    }
    for (; j < half; j += NT) {
      const double2 a0 = ld_stream2(a + 2 * j, pol);
      const double2 b0 = __ldg(x2 + j);
      acc0 = fma_rn(a0.x, b0.x, acc0);
      acc1 = fma_rn(a0.y, b0.y, acc1);
    }
    const double w = warp_sum(add_rn(acc0, acc1));
    if (lane == 0) s_part[parity][warp] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
#pragma unroll
      for (int i = 0; i < NT / kWarp; i++) t = add_rn(t, s_part[parity][i]);
      y[row] = add_rn(y[row], t);
    }
  }
}

// FP32 / BF16 values in double-float arithmetic.  Widening every value to
// FP64 for one FP64 multiply-add kept the FP64 pipe as busy as the FP64
// matrix does (0.99 ms for 537 M entries) although the bytes halve.  Here:
//  * x is split once per call into floats xh = fl32(x), xl = fl32(x - xh),
//    which hold x to 2^-48 relative, kept as two arrays;
//  * each thread accumulates its columns with compensated Dot2 steps (the
//    product's and the sum's rounding errors carried exactly into a second
//    float), 4 columns per step: one load of values (16 bytes FP32, 8 bytes
//    BF16) and one 16-byte load each of xh and xl, consecutive across the
//    warp;
//  * the thread pairs are summed across the warp in double-float (TwoSum-
//    based additions), and the NT/32 warp values in FP64, in a fixed order
//    (keeping the warp values in double-float up to one conversion per row,
//    so that fewer FP64 instructions occupy the pipe, measured 2-6% slower).
// The float arithmetic is exact only inside the float exponent range, so the
// path needs every nonzero |x| and |a| in [2^-40, 2^40] (products within
// [2^-80, 2^80], sums of up to 2^31 of them finite, error terms normal): the
// values are checked once at upload, x by the split kernel on every call,
// which sets *bad; a launch that reads *bad set runs every row in FP64, in the
// same kernel (no host round trip).
constexpr float kDfLo = 9.094947017729282e-13f;  // 2^-40
constexpr float kDfHi = 1.099511627776e12f;      // 2^40

__device__ __forceinline__ bool df_in_range(double v) {
  const double a = fabs(v);
  return a == 0.0 || (a >= (double)kDfLo && a <= (double)kDfHi);  // false for NaN
}

// xs[0, n) = xh, xs[n, 2n) = xl: separate arrays, so that the GEMV's lanes
// read consecutive words of each.
__global__ void k_df_split_x(const double* __restrict__ x, int n, float* __restrict__ xs,
                             int* __restrict__ bad) {
  int any = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = __double2float_rn(v);
    xs[i] = h;
    xs[n + i] = __double2float_rn(v - (double)h);
    any |= !df_in_range(v);
  }
  if (__any_sync(0xffffffffu, any) && threadIdx.x % kWarp == 0) atomicOr(bad, 1);
}

template <class V>
__global__ void k_df_range_vals(const V* __restrict__ a, size_t n, int* __restrict__ bad) {
  int any = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    any |= !df_in_range(widen(a[i]));
  if (__any_sync(0xffffffffu, any) && threadIdx.x % kWarp == 0) atomicOr(bad, 1);
}

// An FP64 value a = h + l split into two floats on the integer pipe: h is a
// truncated to its 24 leading significand bits (exact), l the float nearest
// to the rest a - h (29 bits, exact in FP64, rounded to 24: a is held to
// about 2^-48 relative).  For a == 0 or |a| in [2^-74, 2^128); the values
// reaching it passed the [2^-40, 2^40] check.  No FP64 instruction.
__device__ __forceinline__ void split_f64(double a, float& h, float& l) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  if (e == 0) {
    h = l = 0.f;
    return;
  }
  h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
  const float scale = __uint_as_float((unsigned)(e - 948) << 23);  // 2^(e - 1075)
  const float r = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), scale);
  l = sign ? -r : r;
}

// Values of one lane: out[k] (+ outl[k], the low parts of FP64 values).
template <class V, int VEC>
__device__ __forceinline__ void ld_vals_dd(float (&out)[VEC], float (&outl)[VEC], const V* p, uint64_t pol) {
  static_assert(sizeof(V) == 8, "FP64 values");
  if constexpr (VEC == 1) {
    split_f64(ld_stream(reinterpret_cast<const double*>(p), pol), out[0], outl[0]);
  } else {
    static_assert(VEC == 4, "four values per lane");
    double v[4];
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                 : "=d"(v[0]), "=d"(v[1]) : "l"(p), "l"(pol));
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                 : "=d"(v[2]), "=d"(v[3]) : "l"(reinterpret_cast<const double*>(p) + 2), "l"(pol));
#pragma unroll
    for (int k = 0; k < 4; k++) split_f64(v[k], out[k], outl[k]);
  }
}

template <class V, int VEC>
__device__ __forceinline__ void ld_vals(float (&out)[VEC], const V* p, uint64_t pol) {
  if constexpr (VEC == 1) {
    if constexpr (sizeof(V) == 4) {
      out[0] = ld_stream(reinterpret_cast<const float*>(p), pol);
    } else {  // bfloat16: the high 16 bits of a float
      const __nv_bfloat16 b = ld_stream(reinterpret_cast<const __nv_bfloat16*>(p), pol);
      out[0] = __uint_as_float((unsigned)*reinterpret_cast<const unsigned short*>(&b) << 16);
    }
  } else if constexpr (sizeof(V) == 4) {  // 4 floats: one 16-byte load
    static_assert(VEC == 4, "four values per lane");
    uint4 w;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(w.x), "=r"(w.y), "=r"(w.z), "=r"(w.w) : "l"(p), "l"(pol));
    out[0] = __uint_as_float(w.x); out[1] = __uint_as_float(w.y);
    out[2] = __uint_as_float(w.z); out[3] = __uint_as_float(w.w);
  } else {  // 4 bfloat16 (the high 16 bits of a float): one 8-byte load
    static_assert(VEC == 4, "four values per lane");
    unsigned u0, u1;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(u0), "=r"(u1) : "l"(p), "l"(pol));
    out[0] = __uint_as_float(u0 << 16); out[1] = __uint_as_float(u0 & 0xffff0000u);
    out[2] = __uint_as_float(u1 << 16); out[3] = __uint_as_float(u1 & 0xffff0000u);
  }
}

template <class V, int VEC, int R>
__global__ void __launch_bounds__(NT) k_dense_rows_df(const V* __restrict__ A, int ln_row, int ln_col,
                                                     const float* __restrict__ xs,
                                                     const double* __restrict__ x,
                                                     const int* __restrict__ bad, double* __restrict__ y) {
  __shared__ double s_part[2][R][NT / kWarp];
  const int lane = threadIdx.x % kWarp, warp = threadIdx.x / kWarp;
  const uint64_t pol = policy_evict_first();
  const bool fp64 = *bad != 0;
  const int groups = ln_col / VEC;  // VEC divides ln_col
  int parity = 0;
  // R rows per pass share every load of xh / xl
  for (int row0 = blockIdx.x * R; row0 < ln_row; row0 += gridDim.x * R, parity ^= 1) {
    const int nr = min(R, ln_row - row0);
    double w[R];
    if (fp64) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        double acc = 0;
        if (r < nr) {
          const V* a = A + (size_t)(row0 + r) * ln_col;
          for (int j = threadIdx.x; j < ln_col; j += NT) acc = fma_rn(widen(ld_stream(a + j, pol)), __ldg(x + j), acc);
        }
        w[r] = warp_sum(acc);
      }
    } else {
      float sh[R], sc[R];
#pragma unroll
      for (int r = 0; r < R; r++) sh[r] = sc[r] = 0.f;
      for (int g = threadIdx.x; g < groups; g += NT) {
        float xh[VEC], xl[VEC];
        if constexpr (VEC == 4) {
          const float4 h4 = __ldg(reinterpret_cast<const float4*>(xs) + g);
          const float4 l4 = __ldg(reinterpret_cast<const float4*>(xs + ln_col) + g);
          xh[0] = h4.x; xh[1] = h4.y; xh[2] = h4.z; xh[3] = h4.w;
          xl[0] = l4.x; xl[1] = l4.y; xl[2] = l4.z; xl[3] = l4.w;
        } else {
          xh[0] = __ldg(xs + g);
          xl[0] = __ldg(xs + ln_col + g);
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r < nr) {
            float av[VEC];
            if constexpr (sizeof(V) == 8) {
              // a = ah + al: Dot2 on ah (x as xh + xl), then al * xh into the
              // error term (al * xl is below 2^-48 of the product)
              float al[VEC];
              ld_vals_dd<V, VEC>(av, al, A + (size_t)(row0 + r) * ln_col + (size_t)g * VEC, pol);
#pragma unroll
              for (int k = 0; k < VEC; k++) {
                dot2_step(sh[r], sc[r], av[k], DF{xh[k], xl[k]});
                sc[r] = __fmaf_rn(al[k], xh[k], sc[r]);
              }
            } else {
              ld_vals<V, VEC>(av, A + (size_t)(row0 + r) * ln_col + (size_t)g * VEC, pol);
#pragma unroll
              for (int k = 0; k < VEC; k++) dot2_step(sh[r], sc[r], av[k], DF{xh[k], xl[k]});
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; r++) {
        DF t = two_sum(sh[r], sc[r]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
          t = df_add(t, DF{__shfl_xor_sync(0xffffffffu, t.h, o), __shfl_xor_sync(0xffffffffu, t.l, o)});
        w[r] = lane == 0 ? df_val(t) : 0.0;
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) s_part[parity][r][warp] = w[r];
    }
    __syncthreads();
    if (threadIdx.x < nr) {
      double t = 0;
#pragma unroll
      for (int i = 0; i < NT / kWarp; i++) t = add_rn(t, s_part[parity][threadIdx.x][i]);
      y[row0 + threadIdx.x] = add_rn(y[row0 + threadIdx.x], t);
    }
  }
}

// FP64 rows with 16-byte aligned starts (ln_col even): 16-byte loads.
__global__ void __launch_bounds__(NT) k_dense_f64x2(const double* __restrict__ A, int ln_row,
                                                   int ln_col, const double* __restrict__ x,
                                                   double* __restrict__ y) {
  const int lane = threadIdx.x % kWarp;
  const int gw = (blockIdx.x * NT + threadIdx.x) / kWarp;
  const int nw = gridDim.x * NT / kWarp;
  const uint64_t pol = policy_evict_first();
  const int half = ln_col / 2;
  const double2* x2 = reinterpret_cast<const double2*>(x);
  for (int row = gw; row < ln_row; row += nw) {
    const double* a = A + (size_t)row * ln_col;
    double acc0 = 0, acc1 = 0;
    int j = lane;
    for (; j + 3 * kWarp < half; j += 4 * kWarp) {
      double2 a0 = ld_stream2(a + 2 * j, pol), a1 = ld_stream2(a + 2 * (j + kWarp), pol);
      double2 a2 = ld_stream2(a + 2 * (j + 2 * kWarp), pol), a3 = ld_stream2(a + 2 * (j + 3 * kWarp), pol);
      double2 b0 = __ldg(x2 + j), b1 = __ldg(x2 + j + kWarp);
      double2 b2 = __ldg(x2 + j + 2 * kWarp), b3 = __ldg(x2 + j + 3 * kWarp);
      acc0 = fma_rn(a0.x, b0.x, acc0); acc1 = fma_rn(a0.y, b0.y, acc1);
      acc0 = fma_rn(a1.x, b1.x, acc0); acc1 = fma_rn(a1.y, b1.y, acc1);
      acc0 = fma_rn(a2.x, b2.x, acc0); acc1 = fma_rn(a2.y, b2.y, acc1);
      acc0 = fma_rn(a3.x, b3.x, acc0); acc1 = fma_rn(a3.y, b3.y, acc1);
    }
    for (; j < half; j += kWarp) {
      double2 a0 = ld_stream2(a + 2 * j, pol);
      double2 b0 = __ldg(x2 + j);
      acc0 = fma_rn(a0.x, b0.x, acc0);
      acc1 = fma_rn(a0.y, b0.y, acc1);
    }
    double acc = warp_sum(add_rn(acc0, acc1));
    if (lane == 0) y[row] = add_rn(y[row], acc);
  }
}

__global__ void k_vec_add(double* __restrict__ y, const double* __restrict__ x, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = add_rn(y[i], x[i]);
}

__global__ void k_vec_fill(double* __restrict__ y, double v, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = v;
}

// Warp per row; each entry's value added to its column's sum.
__global__ void k_col_sums(const double* __restrict__ vals, const int* __restrict__ rowptr,
                           const int* __restrict__ colidx, int n_row, int f_col, double* s) {
  const int lane = threadIdx.x % kWarp;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int nw = gridDim.x * blockDim.x / kWarp;
  for (int row = gw; row < n_row; row += nw)
    for (int j = rowptr[row] + lane; j < rowptr[row + 1]; j += kWarp)
      atomicAdd(s + (colidx[j] - f_col), vals[j]);
}

__global__ void k_normalize_cols(double* __restrict__ vals, const int* __restrict__ rowptr,
                                 const int* __restrict__ colidx, int n_row, int f_col,
                                 const double* __restrict__ s) {
  const int lane = threadIdx.x % kWarp;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int nw = gridDim.x * blockDim.x / kWarp;
  for (int row = gw; row < n_row; row += nw)
    for (int j = rowptr[row] + lane; j < rowptr[row + 1]; j += kWarp) {
      const double sv = s[colidx[j] - f_col];
      if (sv > 0) vals[j] = __ddiv_rn(vals[j], sv);
    }
}

// Pass 1: CTA b sums rows b, b + grid, ... per column into partials[b][k].
// With ncol == 1 all 256 threads stride over the vector.
__global__ void __launch_bounds__(256) k_colsum_pass1(const double* __restrict__ x, long n, int ncol,
                                                     double* __restrict__ partials) {
  __shared__ double s[256];
  double acc = 0;
  if (ncol == 1) {
    for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256) acc = add_rn(acc, x[i]);
    s[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int i = 0; i < 256; i++) t = add_rn(t, s[i]);
      partials[(size_t)blockIdx.x * 32] = t;
    }
    return;
  }
  const int lane = threadIdx.x % kWarp, warp = threadIdx.x / kWarp;
  if (lane < ncol)
    for (long i = (long)blockIdx.x * 8 + warp; i < n; i += (long)gridDim.x * 8) acc = add_rn(acc, x[i * ncol + lane]);
  s[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < ncol) {
    double t = 0;
    for (int w = 0; w < 8; w++) t = add_rn(t, s[w * kWarp + threadIdx.x]);
    partials[(size_t)blockIdx.x * 32 + threadIdx.x] = t;
  }
}

__global__ void k_colsum_pass2(const double* __restrict__ partials, int nblk, int ncol, double* out) {
  if ((int)threadIdx.x >= ncol) return;
  double t = 0;
  for (int b = 0; b < nblk; b++) t = add_rn(t, partials[(size_t)b * 32 + threadIdx.x]);
  out[threadIdx.x] = t;
}

__global__ void k_scale_cols(double* __restrict__ x, long n, int ncol, const double* __restrict__ d) {
  const long total = n * ncol;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    x[i] = __ddiv_rn(x[i], d[i % ncol]);
}

template <class V>
__global__ void k_convert(const double* __restrict__ src, V* __restrict__ dst, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = narrow<V>(src[i]);
}

inline int grid_for(long n, int per = 256) {
  return (int)std::max<long>(1, std::min<long>((n + per - 1) / per, 152L * 16));
}

}  // namespace

cudaError_t dense_gemv(const void* vals, int prec, int ln_row, int ln_col, const double* x,
                       double* y, cudaStream_t s) {
  if (ln_row == 0 || ln_col == 0) return cudaSuccess;
  const int grid = (int)std::min<long>(((long)ln_row + NT / kWarp - 1) / (NT / kWarp), 152L * 8);
  switch (prec) {
    case kF64:
      if (ln_col % 2 == 0 && ln_col >= 2 * NT * kDenseU && ((uintptr_t)vals % 16) == 0 && ((uintptr_t)x % 16) == 0)
        k_dense_rows_f64x2<kDenseU><<<ln_row, NT, 0, s>>>(  // a CTA per row, scheduled as CTAs retire
            static_cast<const double*>(vals), ln_row, ln_col, x, y);
      else if (ln_col % 2 == 0 && ((uintptr_t)vals % 16) == 0 && ((uintptr_t)x % 16) == 0)
        k_dense_f64x2<<<grid, NT, 0, s>>>(static_cast<const double*>(vals), ln_row, ln_col, x, y);
      else
        k_dense<double><<<grid, NT, 0, s>>>(static_cast<const double*>(vals), ln_row, ln_col, x, y);
      break;
    case kF32: k_dense<float><<<grid, NT, 0, s>>>(static_cast<const float*>(vals), ln_row, ln_col, x, y); break;
    case kBF16: k_dense<__nv_bfloat16><<<grid, NT, 0, s>>>(static_cast<const __nv_bfloat16*>(vals), ln_row, ln_col, x, y); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t dense_values_df_range(const void* vals, int prec, size_t n, int* flag, bool* ok, cudaStream_t s) {
  *ok = false;
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
  if (e) return e;
  const int grid = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16));
  if (prec == kF64) k_df_range_vals<double><<<grid, 256, 0, s>>>(static_cast<const double*>(vals), n, flag);
  else if (prec == kF32) k_df_range_vals<float><<<grid, 256, 0, s>>>(static_cast<const float*>(vals), n, flag);
  else k_df_range_vals<__nv_bfloat16><<<grid, 256, 0, s>>>(static_cast<const __nv_bfloat16*>(vals), n, flag);
  int h = 1;
  if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return e;
  *ok = h == 0;
  return cudaSuccess;
}

cudaError_t dense_gemv_df(const void* vals, int prec, int ln_row, int ln_col, const double* x, float* xs,
                          int* bad, double* y, cudaStream_t s) {
  if (ln_row == 0 || ln_col == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (e) return e;
  k_df_split_x<<<std::min((ln_col + 255) / 256, 152 * 4), 256, 0, s>>>(x, ln_col, xs, bad);
  // four values per lane when every row starts on a 16-byte boundary (xs from cudaMalloc)
  const bool vec = (uintptr_t)vals % 16 == 0 && (uintptr_t)xs % 16 == 0 && ln_col % 4 == 0;
  constexpr int R = kDenseDfRows;
  const int grid = (ln_row + R - 1) / R;
  if (prec == kF64) {
    const double* a = static_cast<const double*>(vals);
    if (vec) k_dense_rows_df<double, 4, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
    else k_dense_rows_df<double, 1, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
  } else if (prec == kF32) {
    const float* a = static_cast<const float*>(vals);
    if (vec) k_dense_rows_df<float, 4, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
    else k_dense_rows_df<float, 1, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
  } else {
    const __nv_bfloat16* a = static_cast<const __nv_bfloat16*>(vals);
    if (vec) k_dense_rows_df<__nv_bfloat16, 4, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
    else k_dense_rows_df<__nv_bfloat16, 1, R><<<grid, NT, 0, s>>>(a, ln_row, ln_col, xs, x, bad, y);
  }
  return cudaGetLastError();
}

cudaError_t vec_add(double* y, const double* x, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_vec_add<<<grid_for(n), 256, 0, s>>>(y, x, n);
  return cudaGetLastError();
}

cudaError_t vec_fill(double* y, double v, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_vec_fill<<<grid_for(n), 256, 0, s>>>(y, v, n);
  return cudaGetLastError();
}

cudaError_t mat_colsum(const double* x, long n, int ncol, double* partials, double* out,
                       cudaStream_t s) {
  if (ncol < 1 || ncol > kWarp) return cudaErrorInvalidValue;
  k_colsum_pass1<<<kSumBlocks, 256, 0, s>>>(x, n, ncol, partials);
  k_colsum_pass2<<<1, 32, 0, s>>>(partials, kSumBlocks, ncol, out);
  return cudaGetLastError();
}

cudaError_t mat_scale_cols(double* x, long n, int ncol, const double* denom, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_scale_cols<<<grid_for(n * ncol), 256, 0, s>>>(x, n, ncol, denom);
  return cudaGetLastError();
}

cudaError_t csr_col_sums(const double* vals, const int* rowptr, const int* colidx, int n_row,
                         int f_col, double* s, cudaStream_t st) {
  if (n_row <= 0) return cudaSuccess;
  k_col_sums<<<grid_for((long)n_row * kWarp), 256, 0, st>>>(vals, rowptr, colidx, n_row, f_col, s);
  return cudaGetLastError();
}

cudaError_t csr_normalize_cols(double* vals, const int* rowptr, const int* colidx, int n_row,
                               int f_col, const double* s, cudaStream_t st) {
  if (n_row <= 0) return cudaSuccess;
  k_normalize_cols<<<grid_for((long)n_row * kWarp), 256, 0, st>>>(vals, rowptr, colidx, n_row, f_col, s);
  return cudaGetLastError();
}

cudaError_t convert_values(const double* src, void* dst, int prec, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  switch (prec) {
    case kF64: return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    case kF32: k_convert<float><<<grid_for(n), 256, 0, s>>>(src, (float*)dst, n); break;
    case kBF16: k_convert<__nv_bfloat16><<<grid_for(n), 256, 0, s>>>(src, (__nv_bfloat16*)dst, n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
