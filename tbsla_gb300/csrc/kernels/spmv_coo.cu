// COO / SCOO SpMV as a segmented reduction over a row-sorted device copy.
//
// Replaces tbsla::cpp::MatrixCOO::Ax (src/cpp/matrix/MatrixCOO.cpp:135-142)
// and tbsla::cpp::MatrixSCOO::Ax (src/cpp/matrix/MatrixSCOO.cpp:154-164):
// r[row + row_off] += values * v[col + col_off] for every triplet, where the
// reference uses an OpenMP array reduction (one private copy of r per
// thread).  Here the triplets are stably sorted by row once at upload, and
// every warp reduces chunks of 32*U consecutive triplets by key on its own
// (no shared memory, no block barrier):
//  1. lane l owns triplets base + l*U .. base + l*U + U-1 and reads them
//     with 16-byte vector loads (rows, columns, values), which across the
//     warp cover consecutive addresses; all x gathers are issued before any
//     arithmetic;
//  2. each lane sums its own U products in order, closing a segment at each
//     row change (a segment that starts and ends inside the lane is final
//     there); one segmented scan across the 32 lanes (shuffles) then gives
//     each lane the sum of the segment running into it;
//  3. each finished segment is added to r with one FP64 reduction (no
//     returned value, so the warp never waits on it), except the segments
//     of a row that continues into a neighbouring chunk: those go to the
//     chunk's head / tail carry, and a second pass (one thread per chunk)
//     adds each such row's carries in chunk order and then adds the row's
//     total to r once.
// So every row of r receives exactly one addition per launch, and the
// result is the same from run to run (FP64 atomics from several warps
// would sum in arrival order).
// Each product is added with one fused multiply-add (GB300 retires one
// warp-wide FP64 instruction per 16 cycles per SM, and a separate multiply
// and add per triplet kept that pipe 77% busy); the reference rounds the
// product first, so sums differ from its loop by that rounding only.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;

__device__ __forceinline__ uint4 ld_stream_v4(const void* p, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p), "l"(pol));
  return v;
}

// U consecutive elements of type T from a 16-byte aligned address.
template <class T, int U>
__device__ __forceinline__ void ld_run(T (&out)[U], const T* p, uint64_t pol) {
  static_assert(U * sizeof(T) % 16 == 0, "runs are whole 16-byte vectors");
  constexpr int NV = U * (int)sizeof(T) / 16;
  uint4 w[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) w[i] = ld_stream_v4(reinterpret_cast<const uint4*>(p) + i, pol);
  memcpy(out, w, sizeof(out));
}

// Chunk flags of the carry pass.
enum : int { kHeadCont = 1, kTailCont = 2, kOneRow = 4 };

template <class V, int U, bool VEC>
__global__ void __launch_bounds__(NT, 4) k_coo(const int* __restrict__ rows, const int* __restrict__ cols,
                                           const V* __restrict__ vals, long nnz, int row_off,
                                           int col_off, const double* __restrict__ x,
                                           double* __restrict__ y, CooCarry cc) {
  constexpr long CH = (long)kWarp * U;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x % kWarp;
  const long gw = ((long)blockIdx.x * NT + threadIdx.x) / kWarp;
  const long nw = (long)gridDim.x * NT / kWarp;
  const uint64_t pol = policy_evict_first();
  for (long base = gw * CH; base < nnz; base += nw * CH) {
    const long e0 = base + (long)lane * U;
    const long chunk = base / CH, end = min(base + CH, nnz);
    // the chunk's first and last rows, and whether they continue from the
    // previous chunk / into the next (same address on every lane: one load)
    const int fr = __ldg(rows + base), lr = __ldg(rows + end - 1);
    const bool hc = base > 0 && __ldg(rows + base - 1) == fr;
    const bool tc = end < nnz && __ldg(rows + end) == lr;
    if (lane == 0) cc.flags[chunk] = (hc ? kHeadCont : 0) | (tc ? kTailCont : 0) | (fr == lr ? kOneRow : 0);
    // rows whose segments go to the carries (-2: none; rows are >= 0)
    const int hrow = hc ? fr : -2, trow = tc ? lr : -2;
    // one segment sum of row `row`: to the carries if the row crosses a
    // chunk boundary, else straight to r (its only addition)
    auto emit = [&](int row, double v) {
      if (row == hrow)
        cc.head[chunk] = v;
      else if (row == trow)
        cc.tail[chunk] = v;
      else
        atomicAdd(y + row + row_off, v);
    };
    int r[U], c[U];
    V v[U];
    if (VEC && e0 + U <= nnz) {
      ld_run<int, U>(r, rows + e0, pol);
      ld_run<int, U>(c, cols + e0, pol);
      ld_run<V, U>(v, vals + e0, pol);
    } else {
#pragma unroll
      for (int k = 0; k < U; k++) {
        r[k] = -1;  // past the end: a row of its own, never written
        c[k] = 0;
        v[k] = V(0);
        if (e0 + k < nnz) {
          r[k] = ld_stream(rows + e0 + k, pol);
          c[k] = ld_stream(cols + e0 + k, pol);
          v[k] = ld_stream(vals + e0 + k, pol);
        }
      }
    }
    double xg[U];
#pragma unroll
    for (int k = 0; k < U; k++) xg[k] = r[k] >= 0 ? ld_gather(x + c[k] + col_off) : 0.0;

    // Row before this lane's first triplet (-2 at the chunk start: a new
    // segment, which may continue a row of the previous chunk).
    int prev = __shfl_up_sync(full, r[U - 1], 1);
    if (lane == 0) prev = -2;
    const int h0 = r[0] != prev;
    // In-lane pass: first = sum up to the first row change after k = 0
    // (the part of the lane's first segment), acc = the open tail.
    double acc = mul_rn(widen(v[0]), xg[0]), first = 0;
    int closed = 0;  // a row change after k = 0 was seen
#pragma unroll
    for (int k = 1; k < U; k++) {
      if (r[k] != r[k - 1]) {
        if (!closed) first = acc;
        else if (r[k - 1] >= 0) emit(r[k - 1], acc);
        closed = 1;
        acc = 0;
      }
      acc = fma_rn(widen(v[k]), xg[k], acc);
    }
    // Segmented scan of (starts a segment, open tail sum) across lanes:
    // (fa, ta) then (fb, tb) -> (fa | fb, fb ? tb : ta + tb).
    int f = h0 | closed;
    double t = acc;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
      const double tu = __shfl_up_sync(full, t, o);
      const int fu = __shfl_up_sync(full, f, o);
      if (lane >= o) {
        if (!f) t = add_rn(tu, t);
        f |= fu;
      }
    }
    // Sum of the segment running into this lane: the inclusive value of lane - 1.
    double in = __shfl_up_sync(full, t, 1);
    if (lane == 0) in = 0;
    if (h0) {
      // the incoming segment ended at the previous lane's last triplet
      if (lane > 0 && prev >= 0) emit(prev, in);
      if (closed && r[0] >= 0) emit(r[0], first);
    } else if (closed && r[0] >= 0) {
      emit(r[0], add_rn(in, first));
    }
    // the chunk's last segment (it may continue in the next chunk)
    if (lane == kWarp - 1 && r[U - 1] >= 0) emit(r[U - 1], t);
  }
}

// Rows that cross chunk boundaries: the chunk where such a row ends (its
// head continues the row, and the row does not go on past it) walks back to
// the chunk where the row starts, then adds that chunk's tail carry and the
// head carries of the chunks after it, in chunk order, and adds the total
// to r.  No other thread writes those rows in this launch.
__global__ void __launch_bounds__(NT) k_coo_carry(const int* __restrict__ rows, long nchunks, long chunk_len,
                                                 int row_off, double* __restrict__ y, CooCarry cc) {
  for (long c = blockIdx.x * (long)NT + threadIdx.x; c < nchunks; c += (long)gridDim.x * NT) {
    const int f = cc.flags[c];
    if (!(f & kHeadCont) || ((f & kOneRow) && (f & kTailCont))) continue;
    // the nearest chunk before c that is not wholly inside the row (chunk 0
    // never continues a row), 8 flags per round of loads
    long a = c - 1;
    for (;;) {
      int f8[8];
#pragma unroll
      for (int k = 0; k < 8; k++) f8[k] = a - k >= 0 ? cc.flags[a - k] : 0;
      int stop = -1;
#pragma unroll
      for (int k = 7; k >= 0; k--)
        if (!((f8[k] & kOneRow) && (f8[k] & kHeadCont))) stop = k;
      if (stop >= 0) {
        a -= stop;
        break;
      }
      a -= 8;
    }
    double v = cc.tail[a];
#pragma unroll 8
    for (long k = a + 1; k <= c; k++) v = add_rn(v, cc.head[k]);
    double* yr = y + rows[c * chunk_len] + row_off;
    *yr = add_rn(*yr, v);
  }
}

template <class V>
cudaError_t launch(const void* vals, const int* rows, const int* cols, long nnz, int row_off,
                   int col_off, const double* x, double* y, const CooCarry& cc, cudaStream_t s) {
  constexpr int U = kCooChunk / kWarp;  // 41.9 M triplets: 0.216 ms; 16 per lane (93 registers, 2 CTAs / SM): 0.283 ms
  constexpr long per_cta = (long)NT / kWarp * kWarp * U;
  const long grid = (nnz + per_cta - 1) / per_cta;  // one chunk per warp: the block scheduler balances
  const bool vec = ((uintptr_t)rows % 16 == 0) && ((uintptr_t)cols % 16 == 0) && ((uintptr_t)vals % 16 == 0);
  if (vec)
    k_coo<V, U, true><<<(unsigned)grid, NT, 0, s>>>(rows, cols, static_cast<const V*>(vals), nnz, row_off,
                                                    col_off, x, y, cc);
  else
    k_coo<V, U, false><<<(unsigned)grid, NT, 0, s>>>(rows, cols, static_cast<const V*>(vals), nnz, row_off,
                                                     col_off, x, y, cc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long nchunks = coo_chunks(nnz);
  if (nchunks > 1) {
    const long g2 = std::min<long>((nchunks + NT - 1) / NT, 152L * 8);
    k_coo_carry<<<(unsigned)g2, NT, 0, s>>>(rows, nchunks, kCooChunk, row_off, y, cc);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace

cudaError_t coo_spmv(const void* vals, int prec, const int* rows, const int* cols, long nnz,
                     int row_off, int col_off, const double* x, double* y, const CooCarry& cc, cudaStream_t s) {
  if (nnz <= 0) return cudaSuccess;
  switch (prec) {
    case kF64: return launch<double>(vals, rows, cols, nnz, row_off, col_off, x, y, cc, s);
    case kF32: return launch<float>(vals, rows, cols, nnz, row_off, col_off, x, y, cc, s);
    case kBF16: return launch<__nv_bfloat16>(vals, rows, cols, nnz, row_off, col_off, x, y, cc, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tbsla_gpu
