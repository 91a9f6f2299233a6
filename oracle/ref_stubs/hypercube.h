/* Stand-in for the SEP `hypercube` type (an ordered list of axes) used by
 * the reference's hypercube_float and geometry code.  Test infrastructure
 * only.  Axes are numbered from 1, as the reference's getAxis(1) is the
 * fastest axis. */
#pragma once
#include <memory>
#include <sstream>
#include <vector>

#include "axis.h"
namespace SEP {
class hypercube {
 public:
  hypercube() {}
  explicit hypercube(const std::vector<axis> &a) { initNd(a); }
  virtual ~hypercube() {}
  void initNd(const std::vector<axis> &a) { axes_ = a; }
  axis getAxis(int i) const {
    return (i >= 1 && i <= (int)axes_.size()) ? axes_[i - 1] : axis();
  }
  std::vector<axis> getAxes() const { return axes_; }
  std::vector<axis> getAxes(int n) const {
    std::vector<axis> a;
    for (int i = 1; i <= n; ++i) a.push_back(getAxis(i));
    return a;
  }
  int getNdim() const { return (int)axes_.size(); }
  // description text; the reference prints it only on paths not taken here
  void infoStream(std::stringstream &) const {}
  long long getN123() const {
    long long n = 1;
    for (const axis &a : axes_) n *= a.n;
    return n;
  }

 private:
  std::vector<axis> axes_;
};
}  // namespace SEP
