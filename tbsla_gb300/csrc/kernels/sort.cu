// Stable LSD radix sort of (64-bit key, int32 value) pairs, and the COO ->
// CSR ordering built on it.
//
// Replaces the ordering step of tbsla::cpp::MatrixCSR(const MatrixCOO&)
// (src/cpp/matrix/MatrixCSR.cpp:49-96 with compare_row,
// src/cpp/utils/csr.cpp:3-8): entries ordered by (row, column), ties kept
// in storage order.  The reference sorts a permutation with std::sort on
// the host; here the key (row << column bits | column) is sorted on the
// GPU with 8-bit digits, stable pass by pass, so equal keys keep their
// storage order and the permutation equals the host's stable sort exactly.
//
// One pass = per-tile digit histograms (tiles of 4096 keys), an exclusive
// scan of the histograms in digit-major order (global output offsets), and
// a stable scatter: each tile walks its keys in index order 256 at a time;
// lanes with the same digit find each other with __match_any_sync, and the
// per-warp counts in shared memory give every key its place after the
// earlier warps and rounds of its tile.
#include <algorithm>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int RT = 256;
constexpr int TILE = 4096;
constexpr int RADIX = 256;
constexpr int SCAN_CHUNK = 2048;  // elements per CTA in the scan (8 per thread)
constexpr unsigned FULL = 0xffffffffu;

__global__ void __launch_bounds__(RT) k_hist(const uint64_t* __restrict__ keys, long n, int shift, int ntiles,
                                            unsigned* __restrict__ hist) {
  __shared__ unsigned h[RADIX];
  for (int d = threadIdx.x; d < RADIX; d += RT) h[d] = 0;
  __syncthreads();
  const long base = (long)blockIdx.x * TILE;
  for (int k = threadIdx.x; k < TILE; k += RT) {
    const long i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += RT) hist[(long)d * ntiles + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(RT) k_scatter(const uint64_t* __restrict__ keys, const int* __restrict__ vals,
                                               uint64_t* __restrict__ okeys, int* __restrict__ ovals, long n,
                                               int shift, int ntiles, const unsigned* __restrict__ offs) {
  __shared__ unsigned base[RADIX];
  __shared__ unsigned wcnt[RT / kWarp][RADIX];
  const int lane = threadIdx.x & 31, warp = threadIdx.x / kWarp;
  for (int d = threadIdx.x; d < RADIX; d += RT) base[d] = offs[(long)d * ntiles + blockIdx.x];
  const long t0 = (long)blockIdx.x * TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < TILE / RT; r++) {
    for (int d = lane; d < RADIX; d += kWarp) wcnt[warp][d] = 0;
    __syncthreads();
    const long i = t0 + (long)r * RT + threadIdx.x;
    const bool valid = i < n;
    const uint64_t key = valid ? keys[i] : 0;
    const int dg = valid ? (int)((key >> shift) & (RADIX - 1)) : RADIX;  // RADIX: no key
    const unsigned peers = __match_any_sync(FULL, dg);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) wcnt[warp][dg] = __popc(peers);
    __syncthreads();
    if (valid) {
      unsigned p = base[dg] + rank;
      for (int w = 0; w < warp; w++) p += wcnt[w][dg];
      okeys[p] = key;
      ovals[p] = vals[i];
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += RT) {
      unsigned s = 0;
      for (int w = 0; w < RT / kWarp; w++) s += wcnt[w][d];
      base[d] += s;
    }
    __syncthreads();
  }
}

// In-place exclusive scan of each SCAN_CHUNK-element chunk; chunk totals to
// sums[blockIdx.x].
__global__ void __launch_bounds__(RT) k_scan_chunks(unsigned* __restrict__ a, long n, unsigned* __restrict__ sums) {
  __shared__ unsigned ws[RT / kWarp];
  const long c0 = (long)blockIdx.x * SCAN_CHUNK;
  constexpr int PER = SCAN_CHUNK / RT;
  unsigned v[PER];
  unsigned t = 0;
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const long i = c0 + (long)threadIdx.x * PER + k;
    v[k] = i < n ? a[i] : 0u;
    t += v[k];
  }
  // exclusive scan of the per-thread totals over the CTA
  const int lane = threadIdx.x & 31, warp = threadIdx.x / kWarp;
  unsigned incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  unsigned wpre = 0;
  for (int w = 0; w < warp; w++) wpre += ws[w];
  unsigned run = wpre + incl - t;
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const long i = c0 + (long)threadIdx.x * PER + k;
    if (i < n) a[i] = run;
    run += v[k];
  }
  if (threadIdx.x == RT - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(unsigned* __restrict__ a, long n, const unsigned* __restrict__ sums) {
  const long i = (long)blockIdx.x * SCAN_CHUNK + threadIdx.x;
  const unsigned add = sums[blockIdx.x];
  for (long k = i; k < std::min(n, (long)(blockIdx.x + 1) * SCAN_CHUNK); k += RT) a[k] += add;
}

__global__ void k_keys(const int* __restrict__ row, const int* __restrict__ col, long n, int cbits,
                       uint64_t* __restrict__ keys, int* __restrict__ idx) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    keys[i] = ((uint64_t)(unsigned)row[i] << cbits) | (unsigned)col[i];
    idx[i] = (int)i;
  }
}

__global__ void k_count_rows(const int* __restrict__ row, long n, unsigned* __restrict__ cnt) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    atomicAdd(cnt + row[i], 1u);
}

int grid_for(long n) { return (int)std::max<long>(1, std::min<long>((n + RT - 1) / RT, 152L * 32)); }

}  // namespace

// Exclusive scan of a[0..n) in place; scratch: at least scan_scratch(n) words.
long scan_scratch(long n) {
  long s = 0;
  while (n > 1) {
    n = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    s += n;
  }
  return s + 1;
}

cudaError_t exclusive_scan(unsigned* a, long n, unsigned* scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const long nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  k_scan_chunks<<<(unsigned)nb, RT, 0, s>>>(a, n, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nb == 1) return e;
  e = exclusive_scan(scratch, nb, scratch + nb, s);
  if (e != cudaSuccess) return e;
  k_scan_add<<<(unsigned)nb, RT, 0, s>>>(a, n, scratch);
  return cudaGetLastError();
}

long radix_scratch(long n) {
  const long ntiles = (n + TILE - 1) / TILE;
  return (long)RADIX * ntiles + scan_scratch((long)RADIX * ntiles);
}

cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* keys_alt, int* vals, int* vals_alt, long n, int bits,
                             unsigned* scratch, int* result_in_alt, cudaStream_t s) {
  *result_in_alt = 0;
  if (n <= 1) return cudaSuccess;
  const long ntiles = (n + TILE - 1) / TILE;
  unsigned* hist = scratch;
  unsigned* sc = scratch + RADIX * ntiles;
  int flip = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    const uint64_t* ki = flip ? keys_alt : keys;
    uint64_t* ko = flip ? keys : keys_alt;
    const int* vi = flip ? vals_alt : vals;
    int* vo = flip ? vals : vals_alt;
    k_hist<<<(unsigned)ntiles, RT, 0, s>>>(ki, n, shift, (int)ntiles, hist);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = exclusive_scan(hist, (long)RADIX * ntiles, sc, s);
    if (e != cudaSuccess) return e;
    k_scatter<<<(unsigned)ntiles, RT, 0, s>>>(ki, vi, ko, vo, n, shift, (int)ntiles, hist);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    flip ^= 1;
  }
  *result_in_alt = flip;
  return cudaSuccess;
}

// COO -> DENSE (MatrixDENSE.cpp:15-37): the entries in (row, column) order,
// ties in storage order, so each run of one position sums its values in the
// reference's order (starting from 0), written once; a thread per sorted
// entry, the first of a run does the run.
__global__ void k_dense_scatter(const int* __restrict__ perm, const int* __restrict__ row,
                                const int* __restrict__ col, const double* __restrict__ val, long n, long ln_col,
                                double* __restrict__ dense) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const int p = perm[k];
    const int r = row[p], c = col[p];
    if (k > 0) {
      const int q = perm[k - 1];
      if (row[q] == r && col[q] == c) continue;  // inside a run
    }
    double sum = 0.0;
    for (long t = k; t < n; t++) {
      const int u = perm[t];
      if (row[u] != r || col[u] != c) break;
      sum = __dadd_rn(sum, val[u]);
    }
    dense[(size_t)r * ln_col + c] = sum;
  }
}

cudaError_t coo_dense_scatter(const int* perm, const int* row, const int* col, const double* val, long n,
                              long ln_col, double* dense, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_dense_scatter<<<grid_for(n), RT, 0, s>>>(perm, row, col, val, n, ln_col, dense);
  return cudaGetLastError();
}

cudaError_t coo_order(const int* row, const int* col, long n, int n_row, int n_col, uint64_t* keys,
                      uint64_t* keys_alt, int* perm, int* perm_alt, unsigned* rowcount, unsigned* scratch,
                      int* perm_in_alt, cudaStream_t s) {
  int rbits = 0, cbits = 0;
  while (rbits < 31 && (1L << rbits) < (long)n_row) rbits++;
  while (cbits < 31 && (1L << cbits) < (long)n_col) cbits++;
  cudaError_t e = cudaMemsetAsync(rowcount, 0, ((size_t)n_row + 1) * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    k_keys<<<grid_for(n), RT, 0, s>>>(row, col, n, cbits, keys, perm);
    k_count_rows<<<grid_for(n), RT, 0, s>>>(row, n, rowcount);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  e = exclusive_scan(rowcount, (long)n_row + 1, scratch, s);  // row starts
  if (e != cudaSuccess) return e;
  return radix_sort_pairs(keys, keys_alt, perm, perm_alt, n, rbits + cbits, scratch, perm_in_alt, s);
}

}  // namespace tbsla_gpu
