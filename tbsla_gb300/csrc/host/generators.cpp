// Matrix generators.
//
// Part 1 reproduces the reference's deterministic generators (fill_cdiag,
// fill_cqmat, fill_random of every format) so that a handle filled here holds
// the same arrays, byte for byte, as the reference object after the same
// call.  The entry-index -> (row, col) maps and the libc rand_r streams they
// draw from are the reference's (src/cpp/utils/values_generation.cpp); the
// per-format assembly follows each format's fill_* (cited per function).
// Reference quirks that change the produced arrays are kept on purpose and
// named where they occur.
//
// Part 2 holds the synthetic workload generators of this library
// (uniform rows, power-law rows, dense uniform, preferential-attachment
// graph, 7-point diffusion).  They draw from a counter-based hash (SplitMix64
// finaliser), so each entry depends only on (seed, position) and the output
// is identical for any thread count and on any host.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "matrix.hpp"

namespace tbsla_impl {

long range_lnv(long size, int local_pos, int number_pos) {
  // tbsla::utils::range::lnv, src/cpp/utils/range.cpp:7-13
  long n = size / number_pos;
  long mod = size % number_pos;
  if (local_pos < mod) n++;
  return n;
}

long range_pflv(long size, int local_pos, int number_pos) {
  // tbsla::utils::range::pflv, src/cpp/utils/range.cpp:19-26
  long mod = size % number_pos;
  long n = range_lnv(size, local_pos, number_pos) * local_pos;
  if (local_pos >= mod) n += mod;
  return n;
}

namespace {

// ---------------------------------------------------------------------------
// Part 1: reference-compatible generators
// ---------------------------------------------------------------------------

struct Entry {
  uint64_t row, col;  // size_t in the reference; callers reinterpret as signed
  double val;
};

// Entry i of the cdiag matrix (ones on diagonals -c and +c), the map of
// values_generation.cpp:6-26.  The reference computes with size_t and long
// mixed; two's-complement int64 gives the same bits.
Entry cdiag_entry(int64_t i, int64_t nc, int64_t cdiag) {
  if (cdiag == 0) return {(uint64_t)i, (uint64_t)i, 1.0};
  int64_t lim1 = std::max<int64_t>(std::min<int64_t>(nc - cdiag, cdiag), 0);
  if (i < lim1) return {(uint64_t)i, (uint64_t)(i + cdiag), 1.0};
  int64_t lim2 = std::max<int64_t>(cdiag + 2 * (nc - 2 * cdiag), 0);
  if (i < lim2) {
    int64_t it = (i + cdiag) / 2;
    if (i % 2 == 0) return {(uint64_t)it, (uint64_t)(it - cdiag), 1.0};
    return {(uint64_t)it, (uint64_t)(it + cdiag), 1.0};
  }
  int64_t it = i - (nc - 2 * cdiag);
  if (cdiag > nc) it -= cdiag - nc;
  return {(uint64_t)it, (uint64_t)(it - cdiag), 1.0};
}

// Entry i of the cqmat matrix (c entries per row, each moved to a random
// column with probability q), the map of values_generation.cpp:28-47.
// Evaluated in uint64_t as the reference evaluates it in size_t, including
// the tail-row branch whose integer division rand_r()/RAND_MAX makes the
// probability test (0 < q) for every draw but RAND_MAX itself.
Entry cqmat_entry(uint64_t i, uint64_t nr, uint64_t nc, uint64_t c_in, double q,
                  unsigned seed_mult) {
  unsigned seed = (unsigned)i;
  if (seed_mult > 0) seed = (unsigned)(seed_mult * i);
  uint64_t c = std::min(nc, c_in);
  uint64_t full = std::min(nc - c + 1, nr);
  if (i < c * full) {
    uint64_t row = i / c;
    double u = (double)rand_r(&seed) / RAND_MAX;
    uint64_t col = u < q ? (uint64_t)(int64_t)rand_r(&seed) % nc : i / c + i % c;
    return {row, col, 1.0};
  }
  uint64_t it = i - c * full;
  uint64_t cur = 1;
  while (cur < nr - full && it >= c - cur) {
    it -= (c - cur);
    cur++;
  }
  cur += full - 1;
  double u = (double)(rand_r(&seed) / RAND_MAX);
  uint64_t col = u < q ? (uint64_t)(int64_t)rand_r(&seed) % nc : cur + it;
  return {cur, col, 1.0};
}

// random_columns + fix_list, values_generation.cpp:162-221: n draws
// rand_r() % nc from the seed of entry i, then each repeated draw is moved
// one step at a time towards the middle of [0, nc) until it lands on an
// unused column.  Where the reference runs out of room it leaves the slot
// uninitialised, which the caller's block test then (in practice) drops;
// here such a slot is -1, always dropped.
void random_columns(uint64_t i, int n, int nc, unsigned seed_mult, std::vector<int>& out) {
  unsigned seed = (unsigned)i;
  if (seed_mult > 0) seed = (unsigned)(seed_mult * i);
  std::vector<int> raw(n);
  for (int k = 0; k < n; k++) raw[k] = rand_r(&seed) % nc;
  out.assign(n, 0);
  std::vector<int> used;  // small: n is the row length
  used.reserve(2 * n);
  auto is_used = [&](int v) { return std::find(used.begin(), used.end(), v) != used.end(); };
  std::vector<char> dup(n, 0);
  for (int k = 0; k < n; k++) {
    if (is_used(raw[k])) dup[k] = 1;
    else used.push_back(raw[k]);
  }
  for (int k = 0; k < n; k++) {
    if (!dup[k]) {
      out[k] = raw[k];
      continue;
    }
    int v = raw[k];
    int step = (uint64_t)(int64_t)v > (uint64_t)nc / 2 ? -1 : 1;
    while (is_used(v) && v > 0 && v < nc - 1) v += step;
    if (!is_used(v)) {
      out[k] = v;
      used.push_back(v);
    } else {
      out[k] = -1;
    }
  }
}

struct Block {
  int n_row, n_col, ln_row, ln_col, f_row, f_col;
  bool in(int64_t ii, int64_t jj) const {
    return ii >= f_row && ii < f_row + ln_row && jj >= f_col && jj < f_col + ln_col;
  }
};

Block set_block(tbsla_matrix* m, int n_row, int n_col, int pr, int pc, int NR, int NC) {
  tbsla_info& I = m->info;
  I = tbsla_info{};
  I.n_row = n_row;
  I.n_col = n_col;
  I.pr = pr;
  I.pc = pc;
  I.NR = NR;
  I.NC = NC;
  I.ln_row = (int)range_lnv(n_row, pr, NR);
  I.f_row = (int)range_pflv(n_row, pr, NR);
  I.ln_col = (int)range_lnv(n_col, pc, NC);
  I.f_col = (int)range_pflv(n_col, pc, NC);
  m->values.clear();
  m->idx0.clear();
  m->idx1.clear();
  return Block{I.n_row, I.n_col, I.ln_row, I.ln_col, I.f_row, I.f_col};
}

struct Trip {
  int64_t row, col;
  double val;
};

// CSR from per-row entry lists in generation order.
void assemble_csr(tbsla_matrix* m, const std::vector<std::vector<Trip>>& rows, long nnz_field,
                  long alloc) {
  int ln_row = m->info.ln_row;
  m->idx0.zeros(ln_row + 1);
  m->values.zeros(alloc);
  m->idx1.zeros(alloc);
  long k = 0;
  for (int r = 0; r < ln_row; r++) {
    for (const Trip& t : rows[r]) {
      m->idx1[k] = (int)t.col;
      m->values[k] = t.val;
      k++;
    }
    m->idx0[r + 1] = (int)k;
  }
  m->info.nnz = nnz_field;
}

// cqmat row-block prologue shared by the CSR/ELL/SCOO/DENSE fills
// (e.g. MatrixCSR.cpp:390-420): first entry index of the block and the
// number of generated entries in its rows.
void cqmat_prologue(const Block& B, int c, long& incr, long& nv, int& min_) {
  int cc = std::min(c, B.n_col);
  min_ = std::min(B.n_col - cc + 1, B.n_row);
  incr = 0;
  nv = 0;
  for (long i = 0; i < min_; i++) {
    if (i < B.f_row) incr += cc;
    if (i >= B.f_row && i < B.f_row + B.ln_row) nv += cc;
    if (i >= B.f_row + B.ln_row) break;
  }
  long tail = (long)std::min(B.n_row, B.n_col) - min_;
  for (long i = 0; i < tail; i++) {
    if (i + min_ < B.f_row) incr += cc - i - 1;
    if (i + min_ >= B.f_row && i + min_ < B.f_row + B.ln_row) nv += cc - i - 1;
    if (i + min_ >= B.f_row + B.ln_row) break;
  }
}

// Walks the generated entries of the block's rows in the reference's order:
// full rows [f_row, min(min_, row_end)) with cc entries, then tail rows up to
// `tail_end` with cc - i + min_ - 1 entries.  fn(i, entry) per entry.
template <class F>
void cqmat_walk(const Block& B, int c, double q, unsigned s, long incr, int min_, long tail_end,
                F fn) {
  int cc = std::min(c, B.n_col);
  long i = B.f_row;
  long full_end = std::min<long>(min_, (long)B.f_row + B.ln_row);
  for (; i < full_end; i++)
    for (long j = 0; j < cc; j++) fn(i, cqmat_entry(incr++, B.n_row, B.n_col, c, q, s));
  for (; i < tail_end; i++)
    for (long j = 0; j < cc - i + min_ - 1; j++)
      fn(i, cqmat_entry(incr++, B.n_row, B.n_col, c, q, s));
}

}  // namespace

int fill_cdiag(tbsla_matrix* m, int n_row, int n_col, int cdiag, int pr, int pc, int NR, int NC) {
  m->invalidate();
  if (m->format == TBSLA_COO) {
    // MatrixCOO::fill_cdiag, MatrixCOO.cpp:280-318: the global entry list
    // is split evenly by entry index over the NR*NC blocks.
    tbsla_info& I = m->info;
    I = tbsla_info{};
    I.n_row = I.ln_row = n_row;
    I.n_col = I.ln_col = n_col;
    I.pr = pr; I.pc = pc; I.NR = NR; I.NC = NC;
    m->values.clear(); m->idx0.clear(); m->idx1.clear();
    long gnv = std::max(std::min(n_row, n_col - cdiag), 0) + std::max(std::min(n_row - cdiag, n_col), 0);
    if (cdiag == 0) gnv /= 2;
    if (gnv == 0) return TBSLA_OK;
    long s = range_pflv(gnv, pr * NC + pc, NR * NC);
    long n = range_lnv(gnv, pr * NC + pc, NR * NC);
    m->values.resize(n); m->idx0.resize(n); m->idx1.resize(n);
    for (long i = 0; i < n; i++) {
      Entry e = cdiag_entry(i + s, n_col, cdiag);
      m->idx0[i] = (int)e.row;
      m->idx1[i] = (int)e.col;
      m->values[i] = e.val;
    }
    I.nnz = n;
    return TBSLA_OK;
  }
  Block B = set_block(m, n_row, n_col, pr, pc, NR, NC);
  // The row-block formats take (i, i-c) then (i, i+c) for each local row,
  // kept when inside the block (MatrixCSR.cpp:297-371, MatrixSCOO.cpp:228-290,
  // MatrixELL.cpp:263-333, MatrixDENSE.cpp:128-186).
  std::vector<std::vector<Trip>> rows(B.ln_row);
  long nv = 0;
  for (long i = B.f_row; i < (long)B.f_row + B.ln_row; i++) {
    if (B.in(i, i - cdiag)) { rows[i - B.f_row].push_back({i, i - cdiag, 1.0}); nv++; }
    if (cdiag != 0 && B.in(i, i + cdiag)) { rows[i - B.f_row].push_back({i, i + cdiag, 1.0}); nv++; }
  }
  m->info.nnz = nv;
  switch (m->format) {
    case TBSLA_CSR:
      if (nv == 0) { m->idx0.zeros(B.ln_row + 1); return TBSLA_OK; }
      assemble_csr(m, rows, nv, nv);
      return TBSLA_OK;
    case TBSLA_SCOO: {
      if (nv == 0) return TBSLA_OK;
      m->values.resize(nv); m->idx0.resize(nv); m->idx1.resize(nv);
      long k = 0;
      for (auto& r : rows)
        for (auto& t : r) { m->idx0[k] = (int)t.row; m->idx1[k] = (int)t.col; m->values[k] = t.val; k++; }
      return TBSLA_OK;
    }
    case TBSLA_ELL: {
      // Fixed slots: slot 0 holds (i, i-c), slot 1 (i, i+c); a slot whose
      // entry falls outside the block is a pad (0, 0) -- entries are not
      // packed left here, unlike the other ELL fills.
      int mc = cdiag == 0 ? 1 : 2;
      m->info.max_col = mc;
      if (nv == 0) return TBSLA_OK;
      m->values.zeros((size_t)B.ln_row * mc);
      m->idx0.zeros((size_t)B.ln_row * mc);
      long idx = 0;
      for (long i = B.f_row; i < (long)B.f_row + B.ln_row; i++) {
        if (B.in(i, i - cdiag)) { m->idx0[idx] = (int)(i - cdiag); m->values[idx] = 1; }
        idx++;
        if (cdiag != 0) {
          if (B.in(i, i + cdiag)) { m->idx0[idx] = (int)(i + cdiag); m->values[idx] = 1; }
          idx++;
        }
      }
      return TBSLA_OK;
    }
    case TBSLA_DENSE: {
      if (nv == 0) return TBSLA_OK;
      m->values.zeros((size_t)B.ln_row * B.ln_col);
      for (auto& r : rows)
        for (auto& t : r) m->values[(size_t)(t.row - B.f_row) * B.ln_col + (t.col - B.f_col)] = 1;
      return TBSLA_OK;
    }
  }
  return TBSLA_ERR_UNSUPPORTED;
}

int fill_cqmat(tbsla_matrix* m, int n_row, int n_col, int c, double q, unsigned seed_mult,
               int pr, int pc, int NR, int NC) {
  m->invalidate();
  if (m->format == TBSLA_COO) {
    // MatrixCOO::fill_cqmat, MatrixCOO.cpp:320-354: global entry list split
    // by entry index; entries kept whatever block they fall in.
    tbsla_info& I = m->info;
    I = tbsla_info{};
    I.n_row = I.ln_row = n_row;
    I.n_col = I.ln_col = n_col;
    I.pr = pr; I.pc = pc; I.NR = NR; I.NC = NC;
    m->values.clear(); m->idx0.clear(); m->idx1.clear();
    int cc = std::min(c, n_col);
    long gnv = 0;
    int min_ = std::min(n_col - cc + 1, n_row);
    for (long i = 0; i < min_; i++) gnv += cc;
    for (long i = 0; i < (long)std::min(n_row, n_col) - min_; i++) gnv += cc - i - 1;
    if (gnv == 0) return TBSLA_OK;
    long s = range_pflv(gnv, pr * NC + pc, NR * NC);
    long n = range_lnv(gnv, pr * NC + pc, NR * NC);
    // MatrixCOO::init (MatrixCOO.cpp:14-34) resets the block position and
    // grid to 0 / 1x1 and fill_cqmat does not set them again.
    I.pr = 0; I.pc = 0; I.NR = 1; I.NC = 1;
    m->values.resize(n); m->idx0.resize(n); m->idx1.resize(n);
    for (long i = 0; i < n; i++) {
      Entry e = cqmat_entry(i + s, n_row, n_col, c, q, seed_mult);
      m->idx0[i] = (int)e.row;
      m->idx1[i] = (int)e.col;
      m->values[i] = e.val;
    }
    I.nnz = n;
    return TBSLA_OK;
  }
  Block B = set_block(m, n_row, n_col, pr, pc, NR, NC);
  long incr, nv;
  int min_;
  cqmat_prologue(B, c, incr, nv, min_);
  int cc = std::min(c, n_col);
  long row_end = (long)B.f_row + B.ln_row;
  long nr_nc_end = std::min<long>({(long)n_row, (long)n_col, row_end});

  // The count pass of CSR / ELL / SCOO walks cc entries for every row up to
  // min(n_row, n_col, row_end) (MatrixCSR.cpp:425-437), so for tail rows it
  // counts entries past the ones the fill pass stores: CSR reports that
  // count as nnz and sizes its arrays with it.
  long first_pass = 0;
  {
    long k = incr;
    for (long i = B.f_row; i < nr_nc_end; i++)
      for (long j = 0; j < cc; j++) {
        Entry e = cqmat_entry(k++, n_row, n_col, c, q, seed_mult);
        if (B.in((int64_t)e.row, (int64_t)e.col)) first_pass++;
      }
  }
  switch (m->format) {
    case TBSLA_CSR: {
      // MatrixCSR::fill_cqmat, MatrixCSR.cpp:373-486
      m->info.nnz = first_pass;
      if (nv == 0) { m->idx0.zeros(B.ln_row + 1); return TBSLA_OK; }
      std::vector<std::vector<Trip>> rows(B.ln_row);
      cqmat_walk(B, c, q, seed_mult, incr, min_, nr_nc_end, [&](long i, const Entry& e) {
        if (B.in((int64_t)e.row, (int64_t)e.col))
          rows[i - B.f_row].push_back({(int64_t)e.row, (int64_t)e.col, e.val});
      });
      assemble_csr(m, rows, first_pass, first_pass);
      return TBSLA_OK;
    }
    case TBSLA_SCOO: {
      // MatrixSCOO::fill_cqmat, MatrixSCOO.cpp:292-403: nnz is the stored count.
      m->info.nnz = first_pass;
      if (nv == 0) return TBSLA_OK;
      std::vector<Trip> t;
      cqmat_walk(B, c, q, seed_mult, incr, min_, nr_nc_end, [&](long, const Entry& e) {
        if (B.in((int64_t)e.row, (int64_t)e.col)) t.push_back({(int64_t)e.row, (int64_t)e.col, e.val});
      });
      long n = (long)t.size();
      m->values.resize(n); m->idx0.resize(n); m->idx1.resize(n);
      for (long k = 0; k < n; k++) { m->idx0[k] = (int)t[k].row; m->idx1[k] = (int)t[k].col; m->values[k] = t[k].val; }
      m->info.nnz = n;
      return TBSLA_OK;
    }
    case TBSLA_ELL: {
      // MatrixELL::fill_cqmat, MatrixELL.cpp:335-466.  max_col comes from a
      // count pass in which tail rows also count every j in
      // [cc - i + min_ - 1, cc) that lies in [f_col, f_col + ln_col), j being
      // a slot number compared as a column (MatrixELL.cpp:393-397).
      long nnz = 0;
      int mc = 0;
      {
        long k = incr;
        long i = B.f_row;
        long full_end = std::min<long>(min_, row_end);
        for (; i < full_end; i++) {
          int nbc = 0;
          for (long j = 0; j < cc; j++) {
            Entry e = cqmat_entry(k++, n_row, n_col, c, q, seed_mult);
            if (B.in((int64_t)e.row, (int64_t)e.col)) { nnz++; nbc++; }
          }
          mc = std::max(mc, nbc);
        }
        for (; i < nr_nc_end; i++) {
          int nbc = 0;
          long j = 0;
          for (; j < cc - i + min_ - 1; j++) {
            Entry e = cqmat_entry(k++, n_row, n_col, c, q, seed_mult);
            if (B.in((int64_t)e.row, (int64_t)e.col)) { nbc++; nnz++; }
          }
          for (; j < cc; j++)
            if (j >= B.f_col && j < B.f_col + B.ln_col) nbc++;
          mc = std::max(mc, nbc);
        }
      }
      m->info.nnz = nnz;
      m->info.max_col = mc;
      if (nv == 0) return TBSLA_OK;
      m->values.zeros((size_t)B.ln_row * mc);
      m->idx0.zeros((size_t)B.ln_row * mc);
      std::vector<int> fill(B.ln_row, 0);
      // The store pass runs tail rows up to min(n_row, row_end) (n_col not
      // included), MatrixELL.cpp:440.
      long tail_end = std::min<long>((long)n_row, row_end);
      cqmat_walk(B, c, q, seed_mult, incr, min_, tail_end, [&](long i, const Entry& e) {
        if (B.in((int64_t)e.row, (int64_t)e.col)) {
          size_t slot = (size_t)(i - B.f_row) * mc + fill[i - B.f_row]++;
          m->idx0[slot] = (int)e.col;
          m->values[slot] = e.val;
        }
      });
      return TBSLA_OK;
    }
    case TBSLA_DENSE: {
      // MatrixDENSE::fill_cqmat, MatrixDENSE.cpp:187-270: duplicates add up.
      if (nv == 0) return TBSLA_OK;
      m->values.zeros((size_t)B.ln_row * B.ln_col);
      long nnz = 0;
      long tail_end = std::min<long>((long)n_row, row_end);
      cqmat_walk(B, c, q, seed_mult, incr, min_, tail_end, [&](long, const Entry& e) {
        if (B.in((int64_t)e.row, (int64_t)e.col)) {
          m->values[(size_t)((int64_t)e.row - B.f_row) * B.ln_col + ((int64_t)e.col - B.f_col)] += e.val;
          nnz++;
        }
      });
      m->info.nnz = nnz;
      return TBSLA_OK;
    }
  }
  return TBSLA_ERR_UNSUPPORTED;
}

int fill_random(tbsla_matrix* m, int n_row, int n_col, double ratio, unsigned seed_mult,
                int pr, int pc, int NR, int NC) {
  m->invalidate();
  if (m->format == TBSLA_COO || m->format == TBSLA_DENSE) {
    // MatrixCOO.cpp:356-369 and MatrixDENSE.cpp:272-280 only record the
    // dimensions; the matrix stays empty.
    m->reset_info(n_row, n_col);
    m->info.pr = pr; m->info.pc = pc; m->info.NR = NR; m->info.NC = NC;
    m->values.clear(); m->idx0.clear(); m->idx1.clear();
    return TBSLA_OK;
  }
  // MatrixCSR.cpp:861-1005, MatrixELL.cpp:626-769, MatrixSCOO.cpp:559-686:
  // row i takes random_columns(i * cc, cc, n_col) in draw order, kept when
  // inside the block, value 1.  (The reference splits rows over OpenMP
  // threads; the per-row seed makes the split irrelevant.)
  Block B = set_block(m, n_row, n_col, pr, pc, NR, NC);
  int c = std::max(1, (int)(n_col * ratio));
  if (ratio > 1) c = (int)ratio;
  int cc = std::min(c, n_col);
  std::vector<std::vector<Trip>> rows(B.ln_row);
  parallel_for(B.ln_row, [&](long b, long e) {
    std::vector<int> cols;
    for (long r = b; r < e; r++) {
      long i = B.f_row + r;
      random_columns((uint64_t)i * cc, cc, n_col, seed_mult, cols);
      for (int j = 0; j < cc; j++)
        if (B.in(i, cols[j])) rows[r].push_back({i, cols[j], 1.0});
    }
  });
  long nnz = 0;
  int mc = 0;
  for (auto& r : rows) { nnz += (long)r.size(); mc = std::max(mc, (int)r.size()); }
  switch (m->format) {
    case TBSLA_CSR:
      assemble_csr(m, rows, nnz, nnz);
      return TBSLA_OK;
    case TBSLA_SCOO: {
      m->values.resize(nnz); m->idx0.resize(nnz); m->idx1.resize(nnz);
      long k = 0;
      for (auto& r : rows)
        for (auto& t : r) { m->idx0[k] = (int)t.row; m->idx1[k] = (int)t.col; m->values[k] = 1; k++; }
      m->info.nnz = nnz;
      return TBSLA_OK;
    }
    case TBSLA_ELL: {
      m->info.nnz = nnz;
      m->info.max_col = mc;
      m->values.zeros((size_t)B.ln_row * mc);
      m->idx0.zeros((size_t)B.ln_row * mc);
      for (int r = 0; r < B.ln_row; r++)
        for (size_t j = 0; j < rows[r].size(); j++) {
          m->idx0[(size_t)r * mc + j] = (int)rows[r][j].col;
          m->values[(size_t)r * mc + j] = 1;
        }
      return TBSLA_OK;
    }
  }
  return TBSLA_ERR_UNSUPPORTED;
}

// ---------------------------------------------------------------------------
// Part 2: synthetic workload generators
// ---------------------------------------------------------------------------

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Independent stream per (seed, a) indexed by b.
inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(seed ^ mix64(a + 0x632BE59BD9B4E019ull)) + b);
}
inline double u01(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }
inline double um11(uint64_t h) { return 2.0 * u01(h) - 1.0; }  // exact in FP64

// Truncated Zipf(s) on [1, kmax]: cumulative table for inverse sampling.
struct Zipf {
  std::vector<double> cdf;
  double mean = 0;
  Zipf(double s, int kmax) : cdf(kmax) {
    double z = 0, m = 0;
    for (int k = 1; k <= kmax; k++) {
      double p = std::pow((double)k, -s);
      z += p;
      m += k * p;
      cdf[k - 1] = z;
    }
    for (auto& v : cdf) v /= z;
    mean = m / z;
  }
  int draw(double u) const {
    return (int)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
  }
  // Length of a draw k after rescaling: k * scale rounded stochastically
  // (down, or up with probability equal to the fraction; u in [0,1) is the
  // draw's own uniform), clipped to [lo, kmax].  Stochastic rounding keeps
  // the expected length continuous in the scale, so the target mean is met
  // exactly although 60% of the draws are k = 1.
  static long rescale(int k, double scale, double u, long lo, long kmax) {
    const double y = k * scale;
    long r = (long)std::floor(y);
    if (u < y - (double)r) r++;
    return std::min<long>(std::max<long>(r, lo), kmax);
  }
  // Scale whose rescaled lengths have expectation `target` (bisection; the
  // expectation sum_k p_k clamp(k*scale, lo, kmax) is monotone in the scale).
  double scale_for(double target, long lo, long kmax) const {
    auto mean_at = [&](double sc) {
      double m = 0, prev = 0;
      for (size_t k = 1; k <= cdf.size(); k++) {
        m += (cdf[k - 1] - prev) * std::min<double>(std::max<double>(k * sc, (double)lo), (double)kmax);
        prev = cdf[k - 1];
      }
      return m;
    };
    double a = 0, b = 2.0 * target / mean + 1.0;
    while (mean_at(b) < target && b < 1e9) b *= 2;
    for (int it = 0; it < 200; it++) {
      double c = 0.5 * (a + b);
      (mean_at(c) < target ? a : b) = c;
    }
    return b;
  }
};

void finish_square_csr(tbsla_matrix* m, int n) {
  m->reset_info(n, n);
  m->info.nnz = (long)m->idx0[n];
}

}  // namespace

void fill_uniform(double* out, long n, double lo, double hi, unsigned long long seed) {
  parallel_for(n, [&](long b, long e) {
    for (long i = b; i < e; i++) out[i] = lo + (hi - lo) * u01(hash3(seed, 0x5eed, (uint64_t)i));
  });
}

int fill_uniform_rows(tbsla_matrix* m, int n, int k, unsigned long long seed) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  if (n <= 0 || k <= 0 || k > n) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  long nnz = (long)n * k;
  m->idx0.resize(n + 1);
  m->idx1.resize(nnz);
  m->values.resize(nnz);
  for (long i = 0; i <= n; i++) m->idx0[i] = (int)(i * k);
  parallel_for(n, [&](long b, long e) {
    std::vector<int> cols;
    for (long i = b; i < e; i++) {
      cols.assign(1, (int)i);
      uint64_t t = 0;
      while ((int)cols.size() < k) {
        int c = (int)(hash3(seed, (uint64_t)i, t++) % (uint64_t)n);
        if (std::find(cols.begin(), cols.end(), c) == cols.end()) cols.push_back(c);
      }
      std::sort(cols.begin(), cols.end());
      for (int j = 0; j < k; j++) {
        long p = i * k + j;
        m->idx1[p] = cols[j];
        m->values[p] = um11(hash3(seed ^ 0xA5A5A5A5ull, 1, (uint64_t)p));
      }
    }
  });
  finish_square_csr(m, n);
  return TBSLA_OK;
}

int fill_powerlaw(tbsla_matrix* m, int n, double mean_len, double zipf_s, int max_len,
                  double local_frac, int band, unsigned long long seed) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  if (n <= 0 || max_len <= 0 || max_len > n || band < 0) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  Zipf z(zipf_s, max_len);
  // scale chosen so that the expected length after rounding and clipping is
  // exactly mean_len
  const double scale = z.scale_for(mean_len, 1, max_len);
  m->idx0.resize(n + 1);
  std::vector<int> len(n);
  // with every column drawn near the diagonal (local_frac >= 1) a row holds
  // at most the columns of its band; capped there, the distinct-column draw
  // below always ends
  const bool all_local = local_frac >= 1.0;
  parallel_for(n, [&](long b, long e) {
    for (long i = b; i < e; i++) {
      int k = z.draw(u01(hash3(seed, 1, (uint64_t)i)));
      len[i] = (int)Zipf::rescale(k, scale, u01(hash3(seed, 12, (uint64_t)i)), 1, max_len);
      if (all_local) {
        const long cap = std::min<long>((long)n - 1, i + band) - std::max<long>(0, i - band) + 1;
        len[i] = (int)std::min<long>(len[i], cap);
      }
    }
  });
  long acc = 0;
  m->idx0[0] = 0;
  for (long i = 0; i < n; i++) {
    acc += len[i];
    if (acc > 0x7fffffffL) return TBSLA_ERR_INVALID_ARG;  // int32 row pointers
    m->idx0[i + 1] = (int)acc;
  }
  m->idx1.resize(acc);
  m->values.resize(acc);
  parallel_for(n, [&](long b, long e) {
    std::vector<int> cols;
    for (long i = b; i < e; i++) {
      int L = len[i];
      long lo = std::max<long>(0, i - band), hi = std::min<long>((long)n - 1, i + band);
      // distinct columns: draw a batch, sort + unique, draw again for the gap
      int want = std::min<long>(L, (long)n);
      cols.clear();
      uint64_t t = 0;
      while ((int)cols.size() < want) {
        int need = want - (int)cols.size();
        for (int d = 0; d < need; d++) {
          uint64_t h = hash3(seed, 2 + (uint64_t)i * 2, t++);
          bool local = u01(h) < local_frac;
          uint64_t h2 = hash3(seed, 3 + (uint64_t)i * 2, t);
          long c = local ? lo + (long)(h2 % (uint64_t)(hi - lo + 1)) : (long)(h2 % (uint64_t)n);
          cols.push_back((int)c);
        }
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
      }
      long p0 = m->idx0[i];
      for (int j = 0; j < want; j++) {
        m->idx1[p0 + j] = cols[j];
        m->values[p0 + j] = um11(hash3(seed ^ 0xC3C3C3C3ull, 4, (uint64_t)(p0 + j)));
      }
    }
  });
  finish_square_csr(m, n);
  return TBSLA_OK;
}

int fill_dense_uniform(tbsla_matrix* m, int n_row, int n_col, unsigned long long seed) {
  if (m->format != TBSLA_DENSE) return TBSLA_ERR_UNSUPPORTED;
  if (n_row <= 0 || n_col <= 0) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  long n = (long)n_row * n_col;
  m->values.resize(n);
  m->idx0.clear();
  m->idx1.clear();
  parallel_for(n, [&](long b, long e) {
    for (long i = b; i < e; i++) m->values[i] = um11(hash3(seed, 5, (uint64_t)i));
  });
  m->reset_info(n_row, n_col);
  m->info.nnz = n;
  return TBSLA_OK;
}

int fill_pa_graph(tbsla_matrix* m, int n, double mean_deg, double zipf_s, int max_deg,
                  double dangling_frac, unsigned long long seed) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  if (n <= 1 || max_deg <= 0 || max_deg >= n) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  Zipf z(zipf_s, max_deg);
  // Rescale so that the expected out-degree over all nodes (dangling ones
  // included) is mean_deg after rounding and clipping.
  const double scale = z.scale_for(mean_deg / (1.0 - dangling_frac), 1, max_deg);
  std::vector<int> outdeg(n);
  parallel_for(n, [&](long b, long e) {
    for (long j = b; j < e; j++) {
      if (u01(hash3(seed, 6, (uint64_t)j)) < dangling_frac) {
        outdeg[j] = 0;
        continue;
      }
      int k = z.draw(u01(hash3(seed, 7, (uint64_t)j)));
      outdeg[j] = (int)Zipf::rescale(k, scale, u01(hash3(seed, 13, (uint64_t)j)), 1, max_deg);
    }
  });
  long E = 0;
  for (int d : outdeg) E += d;
  if (E > 0x7fffffffL) return TBSLA_ERR_INVALID_ARG;
  // Edges in source order; each target drawn with probability proportional
  // to (in-degree so far + 1): with probability n / (e + n) a uniform node,
  // otherwise the target of a uniformly chosen earlier edge.  Self-loops and
  // repeated targets of one source are redrawn.  Sequential by construction.
  std::vector<int> target(E);
  std::vector<int> mark(n, -1);  // mark[t] == j: t is already a target of source j
  long e = 0;
  uint64_t draw = 0;
  for (int j = 0; j < n; j++) {
    for (int d = 0; d < outdeg[j]; d++) {
      int t = -1;
      for (int attempt = 0; attempt < 64; attempt++) {
        uint64_t h = hash3(seed, 8, draw++);
        double u = u01(h);
        uint64_t h2 = hash3(seed, 9, draw);
        if (e == 0 || u * (double)(e + n) < (double)n) t = (int)(h2 % (uint64_t)n);
        else t = target[h2 % (uint64_t)e];
        if (t != j && mark[t] != j) break;
        t = -1;
      }
      if (t < 0) {  // fall back to the next free node after j
        t = (j + 1) % n;
        while (t == j || mark[t] == j) t = (t + 1) % n;
      }
      mark[t] = j;
      target[e++] = t;
    }
  }
  // CSR of the transpose: row = target, column = source (ascending).
  m->idx0.zeros(n + 1);
  for (long k = 0; k < E; k++) m->idx0[target[k] + 1]++;
  for (int i = 0; i < n; i++) m->idx0[i + 1] += m->idx0[i];
  m->idx1.resize(E);
  m->values.resize(E);
  std::vector<int> fillp(m->idx0.data(), m->idx0.data() + n);
  long k = 0;
  for (int j = 0; j < n; j++)
    for (int d = 0; d < outdeg[j]; d++) {
      int t = target[k++];
      long p = fillp[t]++;
      m->idx1[p] = j;
      m->values[p] = 1.0;
    }
  finish_square_csr(m, n);
  return TBSLA_OK;
}

int fill_diffusion7(tbsla_matrix* m, int n, double sigma, double corr_len,
                    unsigned long long seed) {
  if (m->format != TBSLA_CSR) return TBSLA_ERR_UNSUPPORTED;
  if (n <= 0 || corr_len <= 0) return TBSLA_ERR_INVALID_ARG;
  long N = (long)n * n * n;
  if (N * 7 > 0x7fffffffL) return TBSLA_ERR_INVALID_ARG;
  m->invalidate();
  // Gaussian random field: white noise on a padded grid convolved with a
  // separable Gaussian kernel of standard deviation corr_len / sqrt(2) (so the
  // field's covariance has length corr_len), scaled to standard deviation
  // sigma by the kernel's exact norm.
  double a = corr_len / std::sqrt(2.0);
  int rad = (int)std::ceil(3.0 * a);
  std::vector<double> ker(2 * rad + 1);
  double ksq = 0;
  for (int t = -rad; t <= rad; t++) ker[t + rad] = std::exp(-0.5 * t * t / (a * a));
  for (double w : ker) ksq += w * w;
  double norm = sigma / std::pow(ksq, 1.5);
  int P = n + 2 * rad;
  long PP = (long)P * P * P;
  std::vector<double> buf(PP), tmp(PP);
  parallel_for(PP, [&](long b, long e) {
    for (long i = b; i < e; i++) {  // Box-Muller from two uniforms
      double u1 = 1.0 - u01(hash3(seed, 10, (uint64_t)i));
      double u2 = u01(hash3(seed, 11, (uint64_t)i));
      buf[i] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
  });
  auto conv = [&](std::vector<double>& src, std::vector<double>& dst, long stride) {
    parallel_for(PP, [&](long b, long e) {
      for (long i = b; i < e; i++) {
        long coord = (i / stride) % P;
        double s = 0;
        for (int t = -rad; t <= rad; t++) {
          long c2 = coord + t;
          if (c2 < 0 || c2 >= P) continue;
          s += ker[t + rad] * src[i + t * stride];
        }
        dst[i] = s;
      }
    });
  };
  conv(buf, tmp, 1);
  conv(tmp, buf, P);
  conv(buf, tmp, (long)P * P);
  std::vector<double> kc(N);
  parallel_for(N, [&](long b, long e) {
    for (long c = b; c < e; c++) {
      long x = c % n, y = (c / n) % n, zz = c / ((long)n * n);
      long p = ((zz + rad) * P + (y + rad)) * P + (x + rad);
      kc[c] = std::exp(norm * tmp[p]);
    }
  });
  // 7-point finite volume: face transmissibility = harmonic mean of the two
  // cell coefficients; a Dirichlet boundary face contributes 2 k_cell to the
  // diagonal.  Row c: lower neighbours, diagonal, upper neighbours (sorted).
  m->idx0.resize(N + 1);
  m->idx0[0] = 0;
  for (long c = 0; c < N; c++) {
    long x = c % n, y = (c / n) % n, zz = c / ((long)n * n);
    int cnt = 1 + (x > 0) + (x < n - 1) + (y > 0) + (y < n - 1) + (zz > 0) + (zz < n - 1);
    m->idx0[c + 1] = m->idx0[c] + cnt;
  }
  long nnz = m->idx0[N];
  m->idx1.resize(nnz);
  m->values.resize(nnz);
  const long sx = 1, sy = n, sz = (long)n * n;
  parallel_for(N, [&](long b, long e) {
    for (long c = b; c < e; c++) {
      long x = c % n, y = (c / n) % n, zz = c / ((long)n * n);
      double kcell = kc[c];
      auto T = [&](long nb) { return 2.0 * kcell * kc[nb] / (kcell + kc[nb]); };
      double diag = 0;
      long p = m->idx0[c];
      long nbs[6] = {zz > 0 ? c - sz : -1, y > 0 ? c - sy : -1, x > 0 ? c - sx : -1,
                     x < n - 1 ? c + sx : -1, y < n - 1 ? c + sy : -1, zz < n - 1 ? c + sz : -1};
      // boundary faces
      int nbound = (x == 0) + (x == n - 1) + (y == 0) + (y == n - 1) + (zz == 0) + (zz == n - 1);
      diag += nbound * 2.0 * kcell;
      for (int f = 0; f < 3; f++)
        if (nbs[f] >= 0) { double t = T(nbs[f]); m->idx1[p] = (int)nbs[f]; m->values[p] = -t; diag += t; p++; }
      long pd = p++;
      for (int f = 3; f < 6; f++)
        if (nbs[f] >= 0) { double t = T(nbs[f]); m->idx1[p] = (int)nbs[f]; m->values[p] = -t; diag += t; p++; }
      m->idx1[pd] = (int)c;
      m->values[pd] = diag;
    }
  });
  finish_square_csr(m, (int)N);
  return TBSLA_OK;
}

}  // namespace tbsla_impl
