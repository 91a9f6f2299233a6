/* Stand-in for tbb::parallel_for (see tbb.h in this folder). */
#pragma once
#include <cstdlib>
#include <thread>
#include <vector>
#include "blocked_range.h"
namespace tbb {
inline int oracle_ref_threads() {
  static int n = [] {
    const char *e = std::getenv("ORACLE_REF_THREADS");
    int v = e ? std::atoi(e) : 1;
    return v > 0 ? v : 1;
  }();
  return n;
}
// Built with ORACLE_REF_SERIAL the range runs in order on one thread (the
// reference's random boundary draws rand() inside a parallel_for, so only
// a serial run is reproducible).
template <class T, class F>
void parallel_for(const blocked_range<T> &r, const F &f) {
#ifdef ORACLE_REF_SERIAL
  f(r);
  return;
#endif
  const int nt = oracle_ref_threads();
  const long long len = (long long)(r.end() - r.begin());
  if (nt <= 1 || len < 2 * nt) {
    f(r);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; t++) {
    T b = r.begin() + (T)(len * t / nt);
    T e = r.begin() + (T)(len * (t + 1) / nt);
    pool.emplace_back([&f, b, e] { f(blocked_range<T>(b, e)); });
  }
  for (auto &th : pool) th.join();
}
}  // namespace tbb
