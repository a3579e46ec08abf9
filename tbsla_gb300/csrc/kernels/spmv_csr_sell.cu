// CSR SpMV through a sliced-ELL device layout (SELL-C-sigma, Kreutzer et
// al., SIAM J. Sci. Comput. 2014, with C = 32 = the warp, extended with G
// lanes per row for long rows) -- the default CSR kernel on GB300.
//
// Replaces tbsla::cpp::MatrixCSR::Ax (src/cpp/matrix/MatrixCSR.cpp:209-233):
// y_i = sum_j values_j * v[colidx_j - f_col], overwriting y.
//
// Why this layout on GB300: its FP64 pipe accepts one warp-instruction per
// ~16 cycles per SM whatever the number of active lanes, so the only way to
// reach the memory roofline is to issue the one DFMA per entry from full
// warps and to spend almost nothing else.  A slice is 32 lanes wide; each
// row gets G = 2^g consecutive lanes (entry j of a row on lane j mod G of
// its group, at step j / G), with G the smallest power of two that keeps the
// slice at most `long_thr` steps wide (G = 1 for rows of up to `short_thr`
// entries; those are sorted by length within windows of `sigma` consecutive
// rows, so x near the diagonal and y stay local; longer rows are sorted by
// length over the whole matrix).  A slice's rows thus have nearly equal
// lengths, its DFMAs are nearly all live, the entries of a step are 32
// consecutive words (256-byte coalesced loads) and no work item takes much
// longer than another: one warp per slice, fetched dynamically, widest first.
//
// Each lane sums its entries in entry order with fused multiply-adds; G > 1
// lanes of a row are combined by a fixed butterfly of additions.
#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "csr_block.cuh"
#include "host/parallel.hpp"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int NT = 256;
constexpr unsigned FULL = 0xffffffffu;

// K steps of one lane's row: predicated loads (lanes past their row's end
// issue none, so padding costs no traffic), the K gathers of x in flight
// together, then K full-warp DFMAs (dead lanes add 0 * 0).
template <class V, int K>
__device__ __forceinline__ double steps_k(const V* __restrict__ sv, const int* __restrict__ sc, long off, int j,
                                          int steps, const double* __restrict__ x, int f_col, uint64_t pol,
                                          double acc) {
  V v[K];
  int c[K];
#pragma unroll
  for (int u = 0; u < K; u++) {
    v[u] = V(0.0f);
    c[u] = f_col;
  }
#pragma unroll
  for (int u = 0; u < K; u++) {
    if (j + u < steps) {
      v[u] = ld_stream(sv + off + (long)(j + u) * 32, pol);
      c[u] = ld_stream(sc + off + (long)(j + u) * 32, pol);
    }
  }
  double xv[K];
#pragma unroll
  for (int u = 0; u < K; u++) xv[u] = (j + u < steps) ? ld_gather(x + c[u] - f_col) : 0.0;
  __syncwarp();
#pragma unroll
  for (int u = 0; u < K; u++) acc = fma_rn(widen(v[u]), xv[u], acc);
  return acc;
}

// Sum of one lane's `steps` entries of a slice `width` steps wide (width is
// warp-uniform, so every branch below is too and no DFMA is issued past it).
// With FP64 values, full groups of U steps are software-pipelined on the
// column stream: the next group's column indices are loaded while the
// current group's gathers are in flight, so a group waits for one memory
// latency (the gathers), not for two (the columns, then the gathers).  It
// costs 9 registers (FP64: 71 -> 80, still 3 CTAs per SM; FP32 values would
// drop from 4 CTAs per SM to 3, which loses more than the overlap gains).
template <class V, int U>
__device__ __forceinline__ double slice_rows(const V* __restrict__ sv, const int* __restrict__ sc, long off,
                                             int steps, int width, const double* __restrict__ x, int f_col,
                                             uint64_t pol) {
  double acc = 0;
  int j = 0;
  if (sizeof(V) != 8) {
    for (; j + U <= width; j += U) acc = steps_k<V, U>(sv, sc, off, j, steps, x, f_col, pol, acc);
  } else if (U <= width) {
    int cn[U];
#pragma unroll
    for (int u = 0; u < U; u++) cn[u] = u < steps ? ld_stream(sc + off + (long)u * 32, pol) : f_col;
    for (; j + U <= width; j += U) {
      V v[U];
      double xv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const bool live = j + u < steps;
        xv[u] = live ? ld_gather(x + cn[u] - f_col) : 0.0;
        v[u] = live ? ld_stream(sv + off + (long)(j + u) * 32, pol) : V(0.0f);
      }
      const bool more = j + 2 * U <= width;
#pragma unroll
      for (int u = 0; u < U; u++)
        cn[u] = (more && j + U + u < steps) ? ld_stream(sc + off + (long)(j + U + u) * 32, pol) : f_col;
      __syncwarp();
#pragma unroll
      for (int u = 0; u < U; u++) acc = fma_rn(widen(v[u]), xv[u], acc);
    }
  }
  // remainder (< U steps) in binary pieces
  if (U > 8 && j + 8 <= width) {
    acc = steps_k<V, 8>(sv, sc, off, j, steps, x, f_col, pol, acc);
    j += 8;
  }
  if (U > 4 && j + 4 <= width) {
    acc = steps_k<V, 4>(sv, sc, off, j, steps, x, f_col, pol, acc);
    j += 4;
  }
  if (j + 2 <= width) {
    acc = steps_k<V, 2>(sv, sc, off, j, steps, x, f_col, pol, acc);
    j += 2;
  }
  if (j < width) acc = steps_k<V, 1>(sv, sc, off, j, steps, x, f_col, pol, acc);
  return acc;
}

struct Lane {
  int row;    // -1: unused lane
  int len;    // the row's entries in this column block
  int steps;  // live steps of this lane
};

// Decodes lane `lane` of slice k with descriptor d = {step offset, width, g,
// base}: a window slice (base >= 0) packs (row - base) << 8 | length per
// lane; a slice sorted over the whole block (base = -1) holds the row, with
// its length in lane_len.
__device__ __forceinline__ Lane slice_lane(const SellPlan& p, const int4& d, int meta, long k, int lane) {
  Lane l{-1, 0, 0};
  if (meta < 0) return l;
  if (d.w >= 0) {
    l.row = d.w + (meta >> 8);
    l.len = l.steps = meta & 255;
  } else {
    l.row = meta;
    l.len = __ldg(p.lane_len + k * 32 + lane);
    const int sub = lane & ((1 << d.z) - 1);
    l.steps = l.len > sub ? (l.len - sub + (1 << d.z) - 1) >> d.z : 0;
  }
  return l;
}

// Work claims of k_sell, spread over kQueues counters kQueueStride words
// (256 bytes) apart: one counter drew every warp's atomic to a single L2
// slice, which then ran at its tag-lookup limit and delayed the gathers
// that live in that slice.  Queue q hands out items q, q + kQueues, ...; a
// warp starts on queue (its index mod kQueues) and moves on to the next
// queue when its own runs dry.  Lane 0 holds the state.
constexpr int kQueues = 8, kQueueStride = 64;
static_assert(kQueues * kQueueStride + 1 <= kSellCounterRegion, "counter scratch");
struct Claims {
  unsigned* counter;
  int nitems;
  int q;     // queue the next ticket is drawn from
  int left;  // queues not yet visited
  __device__ __forceinline__ int ticket() { return (int)atomicAdd(counter + q * kQueueStride, 1u); }
  // item of ticket t, drawn from queue q; past the end of q, the next queues
  __device__ __forceinline__ int resolve(int t) {
    int it = q + kQueues * t;
    while (it >= nitems && left > 0) {
      q = (q + 1) % kQueues;
      left--;
      it = q + kQueues * ticket();
    }
    return it;
  }
};

// One column block: y = A_block x (block 0) or y += A_block x (later blocks,
// whose plans leave out the rows without entries in the block).
//
// PR: a one-block plan runs the PageRank step's epilogue (EpiPageRank) on
// each row as it is summed, instead of writing A x for a separate pass: the
// head lane of a row forms the new iterate and adds its terms of the three
// sums in registers.  For a fixed order of those sums the slices are then
// dealt to the warps statically (warp w takes w, w + W, ...: the plan's
// widest-first order interleaves evenly), the CTA partials are summed in
// CTA order by the last CTA to finish (csr::reduce_and_finish), and the
// launch grid is fixed by the plan and the occupancy, so every step of a
// solve adds its terms in the same order.  The FP64 operations of the
// epilogue then overlap the gathers of x instead of running in a pass of
// their own that GB300's FP64 pipe bounds.
template <class V, int U, bool PR>
__global__ void __launch_bounds__(NT) k_sell(SellPlan p, const V* __restrict__ sv, const int* __restrict__ sc,
                                            int f_col, int accumulate, const double* __restrict__ x,
                                            double* __restrict__ y, unsigned* __restrict__ counter,
                                            const int* __restrict__ done, PageRankArgs pr, Ctl ctl) {
  // a set done flag (an iteration that has converged) makes the launch a
  // no-op; no warp has touched the counters then
  if (done && *(volatile const int*)done) return;
  const int lane = threadIdx.x & 31;
  const int nitems = p.nslices;
  const uint64_t pol = policy_evict_first();
  double red[3] = {0, 0, 0};
  csr::EpiPageRank epi{};
  if constexpr (PR) {
    const double s = pr.coef_in[0], t = pr.coef_in[1];
    epi = csr::EpiPageRank{y, x, pr.colw, pr.tele, mul_rn(pr.beta, s), s, t, t / pr.n_nodes};
  }
  // Two items are claimed ahead, and the descriptor of the next one is
  // loaded while the current one runs, so neither the work counters'
  // atomics nor the descriptor loads sit on the critical path.
  const int warp = blockIdx.x * (NT / 32) + (threadIdx.x >> 5), nwarps = gridDim.x * (NT / 32);
  Claims cl{counter, nitems, warp % kQueues, kQueues - 1};
  int cur = 0, nxt = 0;
  if constexpr (PR) {
    cur = warp;
    nxt = warp + nwarps;
  } else {
    if (lane == 0) {
      cur = cl.resolve(cl.ticket());
      nxt = cl.resolve(cl.ticket());
    }
    cur = __shfl_sync(FULL, cur, 0);
    nxt = __shfl_sync(FULL, nxt, 0);
  }
  int4 d = make_int4(0, 0, 0, 0);
  int meta = -1;
  if (cur < nitems) {
    d = __ldg(p.slice + cur);
    meta = __ldg(p.lane + (long)cur * 32 + lane);
  }
  while (cur < nitems) {
    int after = 0;
    if (!PR && lane == 0) after = cl.ticket();
    int4 dn = make_int4(0, 0, 0, 0);
    int mn = -1;
    if (nxt < nitems) {
      dn = __ldg(p.slice + nxt);
      mn = __ldg(p.lane + (long)nxt * 32 + lane);
    }
    const Lane l = slice_lane(p, d, meta, cur, lane);
    const bool head = l.row >= 0 && (lane & ((1 << d.z) - 1)) == 0;
    const double y0 = (!PR && accumulate && head) ? y[l.row] : 0.0;  // issued before the sum
    double acc = slice_rows<V, U>(sv, sc, (long)d.x * 32 + lane, l.steps, d.y, x, f_col, pol);
    for (int o = (1 << d.z) >> 1; o > 0; o >>= 1) acc = add_rn(acc, __shfl_xor_sync(FULL, acc, o));
    if constexpr (PR) {
      if (head) epi.emit(l.row, acc, red);
      cur = nxt;
      nxt += nwarps;
    } else {
      if (head) y[l.row] = accumulate ? add_rn(y0, acc) : acc;
      if (lane == 0) after = cl.resolve(after);
      cur = nxt;
      nxt = __shfl_sync(FULL, after, 0);
    }
    d = dn;
    meta = mn;
  }
  if constexpr (PR) {
    __shared__ csr::Smem sm;
    csr::reduce_and_finish<3>(ctl, red, sm, csr::PageRankFinish::of(pr));
    return;
  }
  // The last warp to finish resets the work counters for the next launch:
  // every warp's claims were answered before it counts itself out here.
  if (lane == 0) {
    const unsigned total = gridDim.x * (NT / 32);
    if (atomicAdd(counter + kQueues * kQueueStride, 1u) == total - 1) {
      for (int q = 0; q < kQueues; q++) counter[q * kQueueStride] = 0;
      counter[kQueues * kQueueStride] = 0;
    }
  }
}

// Fills one column block's slices from the CSR arrays: the G lanes of a row
// walk its entries G at a time and place those of the block, in entry
// order, at position q -> (step q / G, lane q mod G of the group).  Unused
// positions get a zero value on a valid column (never read by k_sell).
template <class V>
__global__ void __launch_bounds__(NT) k_sell_fill(SellPlan p, const V* __restrict__ vals,
                                                 const int* __restrict__ rowptr, const int* __restrict__ colidx,
                                                 int f_col, V* __restrict__ sv, int* __restrict__ sc) {
  const int lane = threadIdx.x & 31;
  const long warps = (long)gridDim.x * (NT / 32);
  for (long k = (blockIdx.x * (long)NT + threadIdx.x) / 32; k < p.nslices; k += warps) {
    const int4 d = p.slice[k];
    const Lane l = slice_lane(p, d, p.lane[k * 32 + lane], k, lane);
    const int G = 1 << d.z, sub = lane & (G - 1), group = lane & ~(G - 1);
    const long off = (long)d.x * 32;
    const int s = l.row >= 0 ? rowptr[l.row] : 0;
    const int e = l.row >= 0 ? rowptr[l.row + 1] : 0;
    const int span = __reduce_max_sync(FULL, e - s);
    int placed = 0;  // entries of this lane's row placed so far
    for (int base = 0; base < span; base += G) {
      const int j = s + base + sub;
      const int col = j < e ? colidx[j] - f_col : -1;
      const bool in = col >= p.col_lo && col < p.col_hi;
      const unsigned m = (__ballot_sync(FULL, in) >> group) & (G == 32 ? FULL : (1u << G) - 1);
      if (in) {
        const int q = placed + __popc(m & ((1u << sub) - 1));
        const long o = off + (long)(q >> d.z) * 32 + group + (q & (G - 1));
        sv[o] = vals[j];
        sc[o] = colidx[j];
      }
      placed += __popc(m);
    }
    for (int t = l.steps; t < d.y; t++) {
      sv[off + (long)t * 32 + lane] = V(0.0f);
      sc[off + (long)t * 32 + lane] = f_col;
    }
  }
}

template <class V, int U>
cudaError_t launch(const SellArgs& a, const double* x, double* y, unsigned* counter, const int* done,
                   cudaStream_t s) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sell<V, U, false>, NT, 0);
  const int grid = std::max(1, sms * std::max(1, per));
  const bool fork = a.side && a.parts > 1 && a.nblocks >= a.parts;
  const int first_part = a.nblocks - a.parts;
  for (int b = 0; b < a.nblocks; b++) {
    const SellPlan& p = a.blocks[b];
    const int k = fork && b >= first_part ? b - first_part : 0;  // row part (0: matrix stream)
    cudaStream_t ls = k > 0 ? a.side[k - 1] : s;
    // a small plan gets about one warp per slice, not the whole resident
    // grid (whose warps would mostly find no work and then all count out on
    // one atomic)
    const int pg = std::min(grid, std::max(1, (p.nslices + NT / 32 - 1) / (NT / 32)));
    cudaError_t e = cudaSuccess;
    if (fork && b == first_part) e = cudaEventRecord(a.fork, s);
    if (e == cudaSuccess && k > 0) e = cudaStreamWaitEvent(ls, a.fork, 0);
    if (e == cudaSuccess && a.ready && b > 0) e = cudaStreamWaitEvent(ls, a.ready[b], 0);
    if (e == cudaSuccess && p.nslices > 0) {
      k_sell<V, U, false><<<pg, NT, 0, ls>>>(p, static_cast<const V*>(a.svals), a.scols, a.f_col, b > 0 ? 1 : 0,
                                             x, y, counter + k * kSellCounterRegion, done, PageRankArgs{}, Ctl{});
      e = cudaGetLastError();
    }
    // recorded for an empty plan too: the event then marks the earlier plans
    if (e == cudaSuccess && a.after && a.after[b]) e = cudaEventRecord(a.after[b], ls);
    if (e == cudaSuccess && k > 0) e = cudaEventRecord(a.join[k - 1], ls);
    if (e != cudaSuccess) return e;
  }
  if (fork)
    for (int k = 1; k < a.parts; k++) {
      cudaError_t e = cudaStreamWaitEvent(s, a.join[k - 1], 0);
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

template <class V>
cudaError_t launch_fill(const SellArgs& a, cudaStream_t s) {
  for (int b = 0; b < a.nblocks; b++) {
    const SellPlan& p = a.blocks[b];
    if (p.nslices == 0) continue;
    const int grid = (int)std::max<long>(1, std::min<long>((p.nslices + 7) / 8, 152L * 32));
    k_sell_fill<V><<<grid, NT, 0, s>>>(p, static_cast<const V*>(a.vals), a.rowptr, a.colidx, a.f_col,
                                       static_cast<V*>(a.svals), a.scols);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The PageRank step over a one-block plan (k_sell with PR): grid = the
// resident CTAs (at most 8 per SM), fewer for a small plan.
template <class V, int U>
cudaError_t launch_pr(const SellArgs& a, const double* x, double* y, const PageRankArgs& pr, Ctl ctl,
                      cudaStream_t s) {
  if (a.nblocks != 1 || a.parts != 1) return cudaErrorInvalidValue;
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sell<V, U, true>, NT, 0);
  const SellPlan& p = a.blocks[0];
  const int grid = std::max(1, std::min(sms * std::max(1, std::min(per, 8)), (p.nslices + NT / 32 - 1) / (NT / 32)));
  k_sell<V, U, true><<<grid, NT, 0, s>>>(p, static_cast<const V*>(a.svals), a.scols, a.f_col, 0, x, y, nullptr,
                                         pr.done, pr, ctl);
  return cudaGetLastError();
}

template <class V>
cudaError_t launch_pr_u(const SellArgs& a, const double* x, double* y, const PageRankArgs& pr, Ctl ctl,
                        cudaStream_t s) {
  switch (a.unroll) {
    case 4: return launch_pr<V, 4>(a, x, y, pr, ctl, s);
    case 16: return launch_pr<V, 16>(a, x, y, pr, ctl, s);
    default: return launch_pr<V, 8>(a, x, y, pr, ctl, s);
  }
}

template <class V>
cudaError_t launch_u(const SellArgs& a, const double* x, double* y, unsigned* counter, const int* done,
                     cudaStream_t s) {
  switch (a.unroll) {
    case 4: return launch<V, 4>(a, x, y, counter, done, s);
    case 16: return launch<V, 16>(a, x, y, counter, done, s);
    default: return launch<V, 8>(a, x, y, counter, done, s);
  }
}

}  // namespace

void sell_plan_build(const int* L, int n, int sthr, int lthr, int sigma, bool skip_empty, long step0,
                     SellPlan* p) {
  using tbsla_impl::parallel_for_items;
  *p = SellPlan{};
  p->n = n;
  sthr = std::max(1, std::min(sthr, 255));
  lthr = std::max(lthr, 1);
  sigma = std::max(32, std::min(sigma, 1 << 23));
  auto len = [&](int i) { return L[i]; };
  // lanes per row (log2) of a row longer than short_thr
  auto lanes_log2 = [&](int l) {
    int g = 0;
    while (g < 5 && (l + (1 << g) - 1) >> g > lthr) g++;
    return g;
  };
  // Rows past short_thr: per lane count, sorted by length over the block.
  std::vector<int> lng[6];
  for (int i = 0; i < n; i++) {
    const int l = len(i);
    if (l > sthr) lng[lanes_log2(l)].push_back(i);
  }
  struct Slice {
    int width, g;
    long first;  // index into wide_rows of its first row
  };
  std::vector<int4> desc;
  std::vector<int> meta, meta_len;
  std::vector<std::pair<int, int>> order;  // (width, slice) of the wide slices
  std::vector<Slice> wide;
  std::vector<int> wide_rows;
  auto by_len = [&](int a, int b) { return len(a) > len(b); };
  for (int g = 0; g <= 5; g++) {
    auto& v = lng[g];
    std::stable_sort(v.begin(), v.end(), by_len);
    const int per = 32 >> g;
    for (size_t q = 0; q < v.size(); q += per) {
      Slice s{(len(v[q]) + (1 << g) - 1) >> g, g, (long)wide_rows.size()};
      for (int r = 0; r < per; r++) wide_rows.push_back(q + r < v.size() ? v[q + r] : -1);
      order.push_back({s.width, (int)wide.size()});
      wide.push_back(s);
    }
  }
  std::stable_sort(order.begin(), order.end(), [](auto& a, auto& b) { return a.first > b.first; });
  long off = step0;  // in steps of 32 entries
  for (auto& o : order) {
    const Slice& s = wide[o.second];
    desc.push_back(make_int4((int)off, s.width, s.g, -1));
    for (int l = 0; l < 32; l++) {
      const int row = wide_rows[s.first + (l >> s.g)];
      meta.push_back(row);
      meta_len.push_back(row >= 0 ? len(row) : 0);
    }
    off += s.width;
  }
  // Short rows: one lane each, sorted by length within windows.
  const int nwin = (n + sigma - 1) / sigma;
  std::vector<std::vector<int>> win(nwin);
  parallel_for_items(nwin, [&](long b, long e) {
    for (long w = b; w < e; w++) {
      const int r0 = (int)(w * sigma), r1 = (int)std::min<long>((w + 1) * (long)sigma, n);
      auto& v = win[w];
      for (int i = r0; i < r1; i++)
        if (len(i) <= sthr && (len(i) > 0 || !skip_empty)) v.push_back(i);
      std::stable_sort(v.begin(), v.end(), by_len);
    }
  });
  std::vector<long> first(nwin + 1, 0);
  for (int w = 0; w < nwin; w++) first[w + 1] = first[w] + (long)((win[w].size() + 31) / 32);
  const long nwide = (long)desc.size();
  const long nshort = first[nwin];
  desc.resize(nwide + nshort);
  meta.resize(32 * (nwide + nshort));
  parallel_for_items(nwin, [&](long b, long e) {
    for (long w = b; w < e; w++) {
      const auto& v = win[w];
      const int base = (int)(w * sigma);
      for (long k = first[w]; k < first[w + 1]; k++) {
        int wd = 0;
        for (int l = 0; l < 32; l++) {
          const size_t q = (size_t)(k - first[w]) * 32 + l;
          int m = -1;
          if (q < v.size()) {
            m = ((v[q] - base) << 8) | len(v[q]);
            wd = std::max(wd, len(v[q]));
          }
          meta[(nwide + k) * 32 + l] = m;
        }
        desc[nwide + k] = make_int4(0, wd, 0, base);
      }
    }
  });
  for (long k = nwide; k < nwide + nshort; k++) {
    desc[k].x = (int)off;
    off += desc[k].y;
  }
  p->nwide = (int)nwide;
  p->nslices = (int)(nwide + nshort);
  p->sell_len = (off - step0) * 32;
  p->slice = new int4[std::max<size_t>(desc.size(), 1)];
  std::copy(desc.begin(), desc.end(), p->slice);
  p->lane = new int[std::max<size_t>(meta.size(), 1)];
  std::copy(meta.begin(), meta.end(), p->lane);
  p->lane_len = new int[std::max<size_t>(meta_len.size(), 1)];
  std::copy(meta_len.begin(), meta_len.end(), p->lane_len);
}

void sell_plan_free(SellPlan* p) {
  delete[] p->slice;
  delete[] p->lane;
  delete[] p->lane_len;
  *p = SellPlan{};
}

cudaError_t sell_fill(const SellArgs& a, cudaStream_t s) {
  switch (a.prec) {
    case kF64: return launch_fill<double>(a, s);
    case kF32: return launch_fill<float>(a, s);
    case kBF16: return launch_fill<__nv_bfloat16>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t sell_spmv(const SellArgs& a, const double* x, double* y, unsigned* counter, cudaStream_t s,
                      const int* done) {
  switch (a.prec) {
    case kF64: return launch_u<double>(a, x, y, counter, done, s);
    case kF32: return launch_u<float>(a, x, y, counter, done, s);
    case kBF16: return launch_u<__nv_bfloat16>(a, x, y, counter, done, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t sell_pagerank(const SellArgs& a, const double* x, double* y, const PageRankArgs& p, Ctl ctl,
                          cudaStream_t s) {
  switch (a.prec) {
    case kF64: return launch_pr_u<double>(a, x, y, p, ctl, s);
    case kF32: return launch_pr_u<float>(a, x, y, p, ctl, s);
    case kBF16: return launch_pr_u<__nv_bfloat16>(a, x, y, p, ctl, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tbsla_gpu
