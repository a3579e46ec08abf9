// Host-side representation of a tbsla_matrix handle.
//
// The handle keeps exactly the arrays a reference tbsla::cpp::Matrix object
// owns (src/cpp/include/tbsla/cpp/Matrix*.hpp), in the reference layouts,
// plus an optional device copy (DeviceMatrix, device.cu) that is rebuilt
// lazily after any host-side mutation.
#pragma once

#include <cstddef>
#include <cstring>
#include <memory>

#include "tbsla_gb300.h"

namespace tbsla_impl {

// Uninitialised host array (std::vector would zero-fill 3 GB for nothing).
template <class T>
struct Buf {
  std::unique_ptr<T[]> p;
  size_t n = 0, cap = 0;
  void resize(size_t k) {
    p.reset(k ? new T[k] : nullptr);
    n = cap = k;
  }
  // Appends one element, doubling the capacity when full (amortised O(1)).
  void push(const T& v) {
    if (n == cap) {
      const size_t c = cap ? 2 * cap : 16;
      std::unique_ptr<T[]> q(new T[c]);
      if (n) std::memcpy(q.get(), p.get(), n * sizeof(T));
      p = std::move(q);
      cap = c;
    }
    p[n++] = v;
  }
  void assign(const T* src, size_t k) {
    resize(k);
    if (k) std::memcpy(p.get(), src, k * sizeof(T));
  }
  void zeros(size_t k) {
    resize(k);
    if (k) std::memset(p.get(), 0, k * sizeof(T));
  }
  void clear() { resize(0); }
  T* data() { return p.get(); }
  const T* data() const { return p.get(); }
  size_t size() const { return n; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
};

struct DeviceMatrix;
void device_release(DeviceMatrix* d);

}  // namespace tbsla_impl

struct tbsla_matrix {
  int format = TBSLA_CSR;
  tbsla_info info{};
  // COO/SCOO: values, row (idx0), col (idx1)
  // CSR:      values, rowptr (idx0), colidx (idx1)
  // ELL:      values, columns (idx0), row-major ln_row x max_col
  // DENSE:    values, row-major ln_row x ln_col
  tbsla_impl::Buf<double> values;
  tbsla_impl::Buf<int> idx0, idx1;
  int precision = TBSLA_F64;
  int csr_tile = 2048;     // row-block budget (entries per block)
  int csr_algo = -1;       // -1: automatic (default), 0: merge path, 1: row blocks, 2: sliced ELL
  int merge_items = 8;     // merge path: items per thread
  int sell_short = 0;      // sliced ELL: rows up to this length, one lane each, sorted per window
                           // (0: 128 for FP64 values with several column blocks, else 64)
  int sell_long = 0;       // longer rows: fewest lanes keeping a slice this many steps wide (0: as short)
  int sell_sigma = 16384;  // window of consecutive rows sorted together
  int sell_unroll = 0;     // steps per lane in flight (0: 8)
  int sell_colblock = 0;   // columns per block (0: 8,388,608 = 64 MiB of x)
  int pr_gather = 8;       // batched PageRank (FP32 / BF16 values): X-row gathers in flight per warp, 8 or 16
  int pr_stream = 1;       // batched PageRank (FP32 / BF16 values): 1 a warp walks a row block's entries as one stream, 0 a warp per row
  int pr_fused = 1;        // PageRank on the sliced-ELL kernel: epilogue inside the SpMV (1) or a pass of its own (0)
  int device = 0;
  mutable tbsla_impl::DeviceMatrix* dev = nullptr;

  void invalidate() const {
    if (dev) {
      tbsla_impl::device_release(dev);
      dev = nullptr;
    }
  }
  void reset_info(int n_row, int n_col) {
    info = tbsla_info{};
    info.n_row = info.ln_row = n_row;
    info.n_col = info.ln_col = n_col;
    info.NR = info.NC = 1;
  }
  ~tbsla_matrix() { invalidate(); }
};

namespace tbsla_impl {

// Length of the value array for the handle's format.
size_t value_len(const tbsla_matrix* m);
// Host-side validation of index ranges and row pointers (status code).
int validate(const tbsla_matrix* m);
// Block partition helpers of tbsla::utils::range (range.cpp:7-26).
long range_lnv(long size, int local_pos, int number_pos);
long range_pflv(long size, int local_pos, int number_pos);

// Generators (generators.cpp).
int fill_cdiag(tbsla_matrix* m, int n_row, int n_col, int cdiag, int pr, int pc, int NR, int NC);
int fill_cqmat(tbsla_matrix* m, int n_row, int n_col, int c, double q, unsigned seed_mult,
               int pr, int pc, int NR, int NC);
int fill_random(tbsla_matrix* m, int n_row, int n_col, double ratio, unsigned seed_mult,
                int pr, int pc, int NR, int NC);
int fill_uniform_rows(tbsla_matrix* m, int n, int k, unsigned long long seed);
int fill_powerlaw(tbsla_matrix* m, int n, double mean_len, double zipf_s, int max_len,
                  double local_frac, int band, unsigned long long seed);
int fill_dense_uniform(tbsla_matrix* m, int n_row, int n_col, unsigned long long seed);
int fill_pa_graph(tbsla_matrix* m, int n, double mean_deg, double zipf_s, int max_deg,
                  double dangling_frac, unsigned long long seed);
int fill_diffusion7(tbsla_matrix* m, int n, double sigma, double corr_len,
                    unsigned long long seed);
void fill_uniform(double* out, long n, double lo, double hi, unsigned long long seed);

// Conversions (formats.cpp).
// device: order the entries with the GPU radix sort instead of the host sort
// (same result).
int convert_from_coo(tbsla_matrix* out, const tbsla_matrix* coo, int format, bool device = false);

// Binary I/O (io.cpp).
int write_file(const tbsla_matrix* m, const char* path, bool append);
int read_file(tbsla_matrix* m, const char* path, long offset);

// Runs fn(begin, end) over [0, n) split across hardware threads.
template <class F>
void parallel_for(long n, F fn);

}  // namespace tbsla_impl

#include "parallel.hpp"
