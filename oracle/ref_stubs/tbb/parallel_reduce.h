/* Stand-in for tbb::parallel_reduce (see tbb.h in this folder); serial. */
#pragma once
#include "blocked_range.h"
namespace tbb {
template <class R, class V, class F, class J>
V parallel_reduce(const R &r, V init, const F &f, const J &) {
  return (V)f(r, init);
}
}  // namespace tbb
