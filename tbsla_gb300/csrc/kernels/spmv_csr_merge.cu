// CSR SpMV with a merge-path split of the work (after Merrill & Garland,
// "Merge-based parallel sparse matrix-vector multiplication", SC'16), built
// for GB300's narrow FP64 pipe.
//
// Replaces tbsla::cpp::MatrixCSR::Ax (src/cpp/matrix/MatrixCSR.cpp:209-233):
// y_i = sum_j values_j * v[colidx_j - f_col], overwriting y.
//
// The n row ends and the nnz entries form one merged sequence of n + nnz
// items (a row end is placed after the row's last entry).  A CTA takes a
// tile of 256 * ITEMS consecutive items and each thread ITEMS of them, so
// every thread issues exactly ITEMS fused multiply-adds (predicated off only
// where the item is a row end): the FP64 pipe sees full warps whatever the
// row-length distribution.  Per tile:
//   1. coalesced loads of the tile's row ends and of its entries' values and
//      column indices; x gathered for every entry; (value, x) staged in
//      shared memory;
//   2. each thread finds its start on the merge path (binary search in
//      shared memory), multiplies-and-adds its entries in order and writes
//      the sum of every row that both starts and ends in its range;
//   3. a row that starts in an earlier thread is completed by the thread
//      holding its end, which adds the tails of the preceding threads in
//      order (a short walk in shared memory);
//   4. a row still open at the tile's end leaves its partial sum (the
//      tile's carry) in a per-tile scratch slot; a second small kernel adds
//      the carries, in tile order, to the rows they belong to.
// Results are deterministic (no atomics).
#include <algorithm>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;

// Staged entries are stored at e + e/32 (one pad slot per 32): the striped
// writes stay conflict-free and the per-thread sequential reads, whose lanes
// sit about ITEMS entries apart, spread over more banks.
__device__ __forceinline__ int padded(int e) { return e + (e >> 5); }

// Padded staging slots, rounded up to a multiple of 8 so that every region
// of the dynamic shared memory (doubles, then values of 8, 4 or 2 bytes,
// then ints) starts 16-byte aligned.
template <int ITEMS>
constexpr int merge_slots() {
  return ((NT * ITEMS + (NT * ITEMS) / 32 + 1) + 7) / 8 * 8;
}

template <class V, int ITEMS>
constexpr size_t merge_smem() {
  // x (padded TILE doubles), values (padded TILE V), row ends (TILE + 1 ints)
  return (size_t)merge_slots<ITEMS>() * (sizeof(double) + sizeof(V)) + (size_t)(NT * ITEMS + 1) * sizeof(int);
}

struct ThreadState {
  int tail_row;
  double tail_val;
  int has_end;
};

// Merge-path start of tile t (row index i; the entry index is t*TILE - i):
// the largest i in [max(0, d - nnz), min(d, n)] whose preceding row end lies
// at or before entry d - i.
__global__ void k_merge_coords(const int* __restrict__ rowptr, int n, long nnz, long tile,
                               long ntiles, int* __restrict__ coord) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t <= ntiles; t += (long)gridDim.x * blockDim.x) {
    const long d = std::min(t * tile, (long)n + nnz);
    long lo = std::max(0L, d - nnz), hi = std::min(d, (long)n);
    const int base = rowptr[0];
    while (lo < hi) {
      const long mid = (lo + hi) >> 1;
      if ((long)(rowptr[mid + 1] - base) <= d - mid - 1) lo = mid + 1;
      else hi = mid;
    }
    coord[t] = (int)lo;
  }
}

template <class V, int ITEMS>
__global__ void __launch_bounds__(NT) k_csr_merge(const V* __restrict__ vals, const int* __restrict__ rowptr,
                                                 const int* __restrict__ colidx, int n, long nnz, int f_col,
                                                 const int* __restrict__ coord, const double* __restrict__ x,
                                                 double* __restrict__ y, int* __restrict__ carry_row,
                                                 double* __restrict__ carry_val) {
  constexpr int TILE = NT * ITEMS;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int SLOTS = merge_slots<ITEMS>();
  static_assert(SLOTS % 8 == 0, "staging regions must stay 16-byte aligned");
  double* s_x = reinterpret_cast<double*>(smem);
  V* s_v = reinterpret_cast<V*>(smem + (size_t)SLOTS * sizeof(double));
  int* s_end = reinterpret_cast<int*>(smem + (size_t)SLOTS * (sizeof(double) + sizeof(V)));
  __shared__ ThreadState s_ts[NT];
  __shared__ int s_start[NT + 1];

  const int tid = threadIdx.x;
  const long t = blockIdx.x;
  const int base = rowptr[0];
  const long d0 = t * (long)TILE;
  const long d1 = std::min(d0 + TILE, (long)n + nnz);
  const int i0 = coord[t], i1 = coord[t + 1];
  const long j0 = d0 - i0, j1 = d1 - i1;  // entry range [j0, j1) relative to base
  const int ni = i1 - i0;
  const int nj = (int)(j1 - j0);
  const uint64_t pol = policy_evict_first();

  // 1. row ends of the tile, entries' values and x
  for (int k = tid; k < ni; k += NT) s_end[k] = ld_stream(rowptr + i0 + 1 + k, pol) - base;
  {
    int c[ITEMS];
    V v[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      const int e = k * NT + tid;
      if (e < nj) {
        c[k] = ld_stream(colidx + base + j0 + e, pol);
        v[k] = ld_stream(vals + base + j0 + e, pol);
      }
    }
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      const int e = k * NT + tid;
      if (e < nj) {
        s_x[padded(e)] = ld_gather(x + c[k] - f_col);
        s_v[padded(e)] = v[k];
      }
    }
  }
  __syncthreads();

  // 2. this thread's start on the merge path inside the tile
  {
    const int dt = std::min(tid * ITEMS, ni + nj);
    int lo = std::max(0, dt - nj), hi = std::min(dt, ni);
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((long)s_end[mid] <= j0 + (dt - mid) - 1) lo = mid + 1;
      else hi = mid;
    }
    s_start[tid] = lo;
    if (tid == 0) s_start[NT] = ni;
  }
  __syncthreads();
  int it = s_start[tid];
  const int it_end = s_start[tid + 1];
  const int dt = std::min(tid * ITEMS, ni + nj);
  const int jt = dt - it;
  const int jt_end = std::min((tid + 1) * ITEMS, ni + nj) - it_end;
  const int m = jt_end - jt;

  double acc = 0;
  int first_row = -1;
  double first_val = 0;
  bool ended = false;
#pragma unroll
  for (int k = 0; k < ITEMS; k++) {
    if (k < m) {
      while (it < it_end && (long)s_end[it] <= j0 + jt + k) {  // rows ending before entry k
        if (!ended) {
          first_row = it;
          first_val = acc;
          ended = true;
        } else {
          y[i0 + it] = acc;
        }
        acc = 0;
        it++;
      }
    }
    // Reconverge before the multiply-add so that it issues once for the
    // whole warp (lanes past their last entry add 0 * 0).
    __syncwarp();
    const int e = padded(min(jt + k, TILE - 1));
    const bool live = k < m;
    const double av = live ? widen(s_v[e]) : 0.0;
    const double xv = live ? s_x[e] : 0.0;
    acc = fma_rn(av, xv, acc);
  }
  while (it < it_end) {  // row ends after the last entry of the range
    if (!ended) {
      first_row = it;
      first_val = acc;
      ended = true;
    } else {
      y[i0 + it] = acc;
    }
    acc = 0;
    it++;
  }
  s_ts[tid].tail_row = it;  // row still open after this thread's range
  s_ts[tid].tail_val = acc;
  s_ts[tid].has_end = ended;
  __syncthreads();

  // 3. the first row ending in this thread: add the preceding threads' tails
  //    (a row open at the tile's start also gets the earlier tiles' carries,
  //    added by k_merge_carries after this kernel)
  if (ended) {
    double total = first_val;
    for (int k = tid - 1; k >= 0; k--) {
      if (s_ts[k].tail_row != first_row) break;
      total = add_rn(s_ts[k].tail_val, total);
      if (s_ts[k].has_end) break;
    }
    y[i0 + first_row] = total;
  }
  // 4. the tile's carry: partial sum of the row open at its end (row i1)
  if (tid == NT - 1) {
    double total = 0;
    for (int k = NT - 1; k >= 0; k--) {
      if (s_ts[k].tail_row != ni) break;
      total = add_rn(s_ts[k].tail_val, total);
      if (s_ts[k].has_end) break;
    }
    carry_row[t] = i1 < n ? i1 : -1;
    carry_val[t] = total;
  }
}

// Adds each run of equal carry rows, in tile order, to its row.
__global__ void k_merge_carries(const int* __restrict__ carry_row, const double* __restrict__ carry_val,
                                long ntiles, double* __restrict__ y) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ntiles; t += (long)gridDim.x * blockDim.x) {
    const int r = carry_row[t];
    if (r < 0 || (t > 0 && carry_row[t - 1] == r)) continue;
    double s = 0;
    for (long u = t; u < ntiles && carry_row[u] == r; u++) s = add_rn(s, carry_val[u]);
    y[r] = add_rn(y[r], s);
  }
}

template <class V, int ITEMS>
cudaError_t launch(const MergeArgs& a, const double* x, double* y, cudaStream_t s) {
  constexpr size_t smem = merge_smem<V, ITEMS>();
  cudaError_t ready = smem_opt_in<k_csr_merge<V, ITEMS>>(smem);
  if (ready != cudaSuccess) return ready;
  k_csr_merge<V, ITEMS><<<(unsigned)a.ntiles, NT, smem, s>>>(
      static_cast<const V*>(a.vals), a.rowptr, a.colidx, a.n, a.nnz, a.f_col, a.coord, x, y, a.carry_row,
      a.carry_val);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<long>((a.ntiles + 255) / 256, 152L * 8);
  k_merge_carries<<<grid, 256, 0, s>>>(a.carry_row, a.carry_val, a.ntiles, y);
  return cudaGetLastError();
}

template <class V>
cudaError_t by_items(const MergeArgs& a, const double* x, double* y, cudaStream_t s) {
  switch (a.items) {
    case 4: return launch<V, 4>(a, x, y, s);
    case 8: return launch<V, 8>(a, x, y, s);
    case 16: return launch<V, 16>(a, x, y, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

long merge_tiles(int n, long nnz, int items) {
  const long tile = (long)NT * items;
  return ((long)n + nnz + tile - 1) / tile;
}

cudaError_t csr_merge_setup(const int* rowptr, int n, long nnz, int items, int* coord, cudaStream_t s) {
  const long tile = (long)NT * items;
  const long ntiles = merge_tiles(n, nnz, items);
  const int grid = (int)std::min<long>((ntiles + 256) / 256, 152L * 8);
  k_merge_coords<<<grid, 256, 0, s>>>(rowptr, n, nnz, tile, ntiles, coord);
  return cudaGetLastError();
}

cudaError_t csr_merge_spmv(const MergeArgs& a, const double* x, double* y, cudaStream_t s) {
  if (a.ntiles == 0) return cudaSuccess;
  switch (a.prec) {
    case kF64: return by_items<double>(a, x, y, s);
    case kF32: return by_items<float>(a, x, y, s);
    case kBF16: return by_items<__nv_bfloat16>(a, x, y, s);
  }
  return cudaErrorInvalidValue;
}

// ---- Allocation-free variant ---------------------------------------------------
// The same merge-path SpMV (FP64 values, 8 items per thread) with its
// scratch -- tile starts and per-tile carries -- in a file-scope device
// array instead of per-matrix allocations, for callers that hold a CSR
// matrix in their own device memory and may not allocate on the call path
// (an application whose memory pool owns the whole device, or a loop that
// must not call the CUDA allocator).  The array serves up to
// kNoAllocTiles tiles of 2048 merge items (n_row + nnz <= 134,217,728);
// bigger inputs are rejected.  Its size is 65,536 FP64 carries + 65,536
// int32 carry rows + 65,537 int32 tile starts = 1,048,580 bytes, rounded up
// to 1,048,832 (about 1 MiB), held on every device that loads the library.  Every scratch word is written before it is
// read within a call, so nothing needs clearing between calls.  Calls that
// overlap in time (other streams, other host threads) share the array and
// race: the caller serialises them.
namespace {

constexpr long kNoAllocTiles = 65536;
constexpr size_t kNoAllocBytes =
    (size_t)kNoAllocTiles * sizeof(double) + (size_t)kNoAllocTiles * sizeof(int) + (kNoAllocTiles + 1) * sizeof(int);
static __device__ __align__(256) unsigned char g_noalloc_scratch[(kNoAllocBytes + 255) / 256 * 256];

// Device address of the scratch array on the current device.  It is looked
// up on every call (the lookup allocates nothing), so the address stays right
// when a device was reset and the module reloaded at another address.  The
// first lookup on a device loads the module there, so the first call on a
// device belongs before any stream capture.
cudaError_t noalloc_base(void** base) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *base = p;
  return cudaSuccess;
}

}  // namespace

long csr_merge_noalloc_max_items() { return kNoAllocTiles * NT * 8L; }

cudaError_t csr_merge_spmv_noalloc(const double* vals, const int* rowptr, const int* colidx, int n, long nnz,
                                   int f_col, const double* x, double* y, cudaStream_t s) {
  const long ntiles = merge_tiles(n, nnz, 8);
  if (ntiles > kNoAllocTiles) return cudaErrorInvalidValue;
  if (ntiles == 0) return cudaSuccess;
  void* base = nullptr;
  cudaError_t e = noalloc_base(&base);
  if (e != cudaSuccess) return e;
  double* carry_val = static_cast<double*>(base);
  int* carry_row = reinterpret_cast<int*>(carry_val + kNoAllocTiles);
  int* coord = carry_row + kNoAllocTiles;
  e = csr_merge_setup(rowptr, n, nnz, 8, coord, s);
  if (e != cudaSuccess) return e;
  const MergeArgs a{vals, kF64, rowptr, colidx, n, nnz, f_col, 8, coord, ntiles, carry_row, carry_val};
  return csr_merge_spmv(a, x, y, s);
}

}  // namespace tbsla_gpu
