// CSR SpMV through a sliced-ELL device layout (SELL-C-sigma, Kreutzer et
// al., SIAM J. Sci. Comput. 2014, with C = 32 = the warp) -- the default CSR
// kernel on GB300.
//
// Replaces tbsla::cpp::MatrixCSR::Ax (src/cpp/matrix/MatrixCSR.cpp:209-233):
// y_i = sum_j values_j * v[colidx_j - f_col], overwriting y.
//
// Why this layout on GB300: its FP64 pipe accepts one warp-instruction per
// ~17 cycles per SM whatever the number of active lanes, so the only way to
// reach the HBM roofline is to issue the one DFMA per entry from full warps
// and to spend almost nothing else.  Rows are grouped 32 at a time into
// slices of similar length (one lane per row), so a warp's DFMAs are nearly
// all live, no reduction across lanes is needed, and the entries of a step
// are 32 consecutive words (256-byte coalesced loads).  Sorting is done
// within windows of `sigma` consecutive rows for short rows (x near the
// diagonal and y stay local), over the whole matrix for medium rows (so that
// a slice's rows have nearly equal lengths), and the few rows longer than
// `long_thr` are read straight from the CSR arrays by a whole warp each.
// Work items (long rows, medium slices, short slices, in that order) are
// fetched dynamically per warp, longest first.
//
// Each row is summed in entry order with fused multiply-adds.
#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "host/parallel.hpp"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;
constexpr int UNROLL = 4;

template <class V>
__device__ __forceinline__ double slice_rows(const V* __restrict__ sv, const int* __restrict__ sc, long off,
                                             int len, int width, const double* __restrict__ x, int f_col,
                                             uint64_t pol) {
  double acc = 0;
  for (int j = 0; j < width; j += UNROLL) {
    // dead lanes keep a zero value and a valid column, so nothing they
    // might touch is out of bounds
    V v[UNROLL];
    int c[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      v[u] = V(0.0f);
      c[u] = f_col;
    }
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      if (j + u < len) {
        v[u] = ld_stream(sv + off + (long)(j + u) * 32, pol);
        c[u] = ld_stream(sc + off + (long)(j + u) * 32, pol);
      }
    }
    double xv[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) xv[u] = (j + u < len) ? ld_gather(x + c[u] - f_col) : 0.0;
    __syncwarp();
#pragma unroll
    for (int u = 0; u < UNROLL; u++) acc = fma_rn((j + u < len) ? widen(v[u]) : 0.0, xv[u], acc);
  }
  return acc;
}

template <class V>
__device__ __forceinline__ double warp_row(const V* __restrict__ vals, const int* __restrict__ colidx, int s,
                                           int e, const double* __restrict__ x, int f_col, int lane,
                                           uint64_t pol) {
  double acc = 0;
  for (int base = s; base < e; base += 32 * UNROLL) {
    // dead lanes keep a zero value and a valid column, so nothing they
    // might touch is out of bounds
    V v[UNROLL];
    int c[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      v[u] = V(0.0f);
      c[u] = f_col;
    }
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      const int j = base + u * 32 + lane;
      if (j < e) {
        v[u] = ld_stream(vals + j, pol);
        c[u] = ld_stream(colidx + j, pol);
      }
    }
    double xv[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) xv[u] = (base + u * 32 + lane < e) ? ld_gather(x + c[u] - f_col) : 0.0;
    __syncwarp();
#pragma unroll
    for (int u = 0; u < UNROLL; u++)
      acc = fma_rn((base + u * 32 + lane < e) ? widen(v[u]) : 0.0, xv[u], acc);
  }
  return warp_sum(acc);
}

struct Lane {
  int row;
  int len;
  long off;
};

// Decodes lane `lane` of medium / short item k (k counted from the first
// medium slice).
__device__ __forceinline__ Lane slice_lane(const SellPlan& p, const int* rowptr, int k, int lane) {
  Lane l;
  if (k < p.nmed) {
    l.row = p.med_rows[(long)k * 32 + lane];
    l.len = l.row >= 0 ? rowptr[l.row + 1] - rowptr[l.row] : 0;
    l.off = p.med_off[k] + lane;
  } else {
    k -= p.nmed;
    const int m = p.short_meta[(long)k * 32 + lane];
    l.row = m >= 0 ? p.short_base[k] + (m >> 8) : -1;
    l.len = m >= 0 ? (m & 255) : 0;
    l.off = p.short_off[k] + lane;
  }
  return l;
}

template <class V>
__global__ void __launch_bounds__(NT) k_sell(SellArgs a, const double* __restrict__ x, double* __restrict__ y,
                                            unsigned* __restrict__ counter) {
  const int lane = threadIdx.x & 31;
  const SellPlan& p = a.plan;
  const int nitems = p.nlong + p.nmed + p.nshort;
  const uint64_t pol = policy_evict_first();
  const V* vals = static_cast<const V*>(a.vals);
  const V* sv = static_cast<const V*>(a.svals);
  for (;;) {
    int item = 0;
    if (lane == 0) item = (int)atomicAdd(counter, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= nitems) break;
    if (item < p.nlong) {
      const int row = p.long_rows[item];
      const double acc = warp_row(vals, a.colidx, a.rowptr[row], a.rowptr[row + 1], x, a.f_col, lane, pol);
      if (lane == 0) y[row] = acc;
    } else {
      const Lane l = slice_lane(p, a.rowptr, item - p.nlong, lane);
      const int width = __reduce_max_sync(0xffffffffu, l.len);
      const double acc = slice_rows(sv, a.scols, l.off, l.len, width, x, a.f_col, pol);
      if (l.row >= 0) y[l.row] = acc;
    }
  }
  // The last warp to finish resets the work counter for the next launch.
  if (lane == 0) {
    const unsigned total = gridDim.x * (NT / 32);
    if (atomicAdd(counter + 1, 1u) == total - 1) {
      counter[0] = 0;
      counter[1] = 0;
    }
  }
}

template <class V>
__global__ void __launch_bounds__(NT) k_sell_fill(SellArgs a, V* __restrict__ sv, int* __restrict__ sc) {
  const int lane = threadIdx.x & 31;
  const SellPlan& p = a.plan;
  const V* vals = static_cast<const V*>(a.vals);
  const long nitems = (long)p.nmed + p.nshort;
  const long warps = (long)gridDim.x * (NT / 32);
  for (long k = (blockIdx.x * (long)NT + threadIdx.x) / 32; k < nitems; k += warps) {
    const Lane l = slice_lane(p, a.rowptr, (int)k, lane);
    if (l.row < 0) continue;
    const int s = a.rowptr[l.row];
    for (int j = 0; j < l.len; j++) {
      sv[l.off + (long)j * 32] = vals[s + j];
      sc[l.off + (long)j * 32] = a.colidx[s + j];
    }
  }
}

template <class V>
cudaError_t launch(const SellArgs& a, const double* x, double* y, unsigned* counter, cudaStream_t s) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sell<V>, NT, 0);
  const int grid = std::max(1, sms * std::max(1, per));
  k_sell<V><<<grid, NT, 0, s>>>(a, x, y, counter);
  return cudaGetLastError();
}

template <class V>
cudaError_t launch_fill(const SellArgs& a, void* sv, int* sc, cudaStream_t s) {
  const long items = (long)a.plan.nmed + a.plan.nshort;
  const int grid = (int)std::max<long>(1, std::min<long>((items + 7) / 8, 152L * 32));
  k_sell_fill<V><<<grid, NT, 0, s>>>(a, static_cast<V*>(sv), sc);
  return cudaGetLastError();
}

}  // namespace

void sell_plan_build(const int* rp, int n, int sthr, int lthr, int sigma, SellPlan* p) {
  using tbsla_impl::parallel_for;
  *p = SellPlan{};
  p->n = n;
  p->short_thr = sthr = std::min(sthr, 255);
  p->long_thr = lthr = std::max(lthr, sthr);
  p->sigma = sigma;
  auto len = [&](int i) { return rp[i + 1] - rp[i]; };
  // long rows: longest first
  std::vector<int> lng, med;
  for (int i = 0; i < n; i++) {
    const int l = len(i);
    if (l > lthr) lng.push_back(i);
    else if (l > sthr) med.push_back(i);
  }
  auto by_len = [&](int a, int b) { return len(a) > len(b); };
  std::stable_sort(lng.begin(), lng.end(), by_len);
  std::stable_sort(med.begin(), med.end(), by_len);
  p->nlong = (int)lng.size();
  p->long_rows = new int[std::max<size_t>(lng.size(), 1)];
  std::copy(lng.begin(), lng.end(), p->long_rows);
  // medium slices over the whole matrix
  p->nmed = (int)((med.size() + 31) / 32);
  p->med_rows = new int[std::max(32L * p->nmed, 1L)];
  p->med_off = new long[p->nmed + 1];
  long off = 0;
  for (int k = 0; k < p->nmed; k++) {
    p->med_off[k] = off;
    int width = 0;
    for (int l = 0; l < 32; l++) {
      const size_t q = (size_t)k * 32 + l;
      const int row = q < med.size() ? med[q] : -1;
      p->med_rows[q] = row;
      if (row >= 0) width = std::max(width, len(row));
    }
    off += 32L * width;
  }
  p->med_off[p->nmed] = off;
  // short slices, sorted within windows
  const int nwin = (n + sigma - 1) / sigma;
  std::vector<std::vector<int>> win(nwin);
  parallel_for(nwin, [&](long b, long e) {
    for (long w = b; w < e; w++) {
      const int r0 = (int)(w * sigma), r1 = (int)std::min<long>((w + 1) * (long)sigma, n);
      auto& v = win[w];
      for (int i = r0; i < r1; i++)
        if (len(i) <= sthr) v.push_back(i);
      std::stable_sort(v.begin(), v.end(), by_len);
    }
  });
  std::vector<long> first(nwin + 1, 0);
  for (int w = 0; w < nwin; w++) first[w + 1] = first[w] + (long)((win[w].size() + 31) / 32);
  p->nshort = (int)first[nwin];
  p->short_meta = new int[std::max(32L * p->nshort, 1L)];
  p->short_base = new int[std::max(p->nshort, 1)];
  p->short_off = new long[p->nshort + 1];
  std::vector<long> width(std::max(p->nshort, 1), 0);
  parallel_for(nwin, [&](long b, long e) {
    for (long w = b; w < e; w++) {
      const auto& v = win[w];
      const int base = (int)(w * sigma);
      for (long k = first[w]; k < first[w + 1]; k++) {
        p->short_base[k] = base;
        int wd = 0;
        for (int l = 0; l < 32; l++) {
          const size_t q = (size_t)(k - first[w]) * 32 + l;
          int m = -1;
          if (q < v.size()) {
            m = ((v[q] - base) << 8) | len(v[q]);
            wd = std::max(wd, len(v[q]));
          }
          p->short_meta[k * 32 + l] = m;
        }
        width[k] = wd;
      }
    }
  });
  for (int k = 0; k < p->nshort; k++) {
    p->short_off[k] = off;
    off += 32L * width[k];
  }
  p->short_off[p->nshort] = off;
  p->sell_len = off;
}

void sell_plan_free(SellPlan* p) {
  delete[] p->long_rows;
  delete[] p->med_rows;
  delete[] p->med_off;
  delete[] p->short_meta;
  delete[] p->short_base;
  delete[] p->short_off;
  *p = SellPlan{};
}

cudaError_t sell_fill(const SellArgs& a, void* svals, int* scols, cudaStream_t s) {
  if ((long)a.plan.nmed + a.plan.nshort == 0) return cudaSuccess;
  switch (a.prec) {
    case kF64: return launch_fill<double>(a, svals, scols, s);
    case kF32: return launch_fill<float>(a, svals, scols, s);
    case kBF16: return launch_fill<__nv_bfloat16>(a, svals, scols, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t sell_spmv(const SellArgs& a, const double* x, double* y, unsigned* counter, cudaStream_t s) {
  if ((long)a.plan.nlong + a.plan.nmed + a.plan.nshort == 0) return cudaSuccess;
  switch (a.prec) {
    case kF64: return launch<double>(a, x, y, counter, s);
    case kF32: return launch<float>(a, x, y, counter, s);
    case kBF16: return launch<__nv_bfloat16>(a, x, y, counter, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tbsla_gpu
