// Minimal fork-join over std::thread for host-side preparation work
// (generation, validation, layout changes).  Deterministic results never
// depend on the split: every caller writes disjoint index ranges.
#pragma once

#include <algorithm>
#include <thread>
#include <vector>

namespace tbsla_impl {

inline int host_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)std::min(h, 64u) : 4;
}

template <class F>
void parallel_for(long n, F fn) {
  int nt = host_threads();
  if (n < 65536 || nt <= 1) {
    fn(0L, n);
    return;
  }
  nt = (int)std::min<long>(nt, n / 16384 + 1);
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; t++) {
    long b = n * t / nt, e = n * (t + 1) / nt;
    th.emplace_back([=] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

// The same over n heavy items (each worth thousands of elements, e.g. a
// window of rows to sort): split across threads whenever n > 1.
template <class F>
void parallel_for_items(long n, F fn) {
  const int nt = (int)std::min<long>(host_threads(), n);
  if (nt <= 1) {
    fn(0L, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; t++) {
    long b = n * t / nt, e = n * (t + 1) / nt;
    th.emplace_back([=] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

}  // namespace tbsla_impl
