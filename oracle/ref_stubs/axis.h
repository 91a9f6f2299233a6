/* Stand-in for the SEP `axis` type used by the reference's geometry code
 * (SEP libraries are not installed).  Test infrastructure only: an axis is
 * a sample count, origin and spacing (floats, as the reference's
 * arithmetic on o and d takes them). */
#pragma once
#include <string>
namespace SEP {
class axis {
 public:
  axis() : n(1), o(0.f), d(1.f) {}
  axis(int n_, float o_ = 0.f, float d_ = 1.f, const std::string &l = "",
       const std::string &u = "")
      : n(n_), o(o_), d(d_), label(l), unit(u) {}
  int n;
  float o, d;
  std::string label, unit;
};
}  // namespace SEP
