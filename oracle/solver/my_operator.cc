// my_operator members (base/my_operator.cc:5-59) -- TEST INFRASTRUCTURE ONLY.
#include "my_operator.h"

#include <cmath>
#include <cstdio>

// my_operator.cc:5-12: the spaces are kept as clones
void my_operator::set_domain(std::shared_ptr<my_vector> dom) {
  scale = 1;
  domain = dom->clone_space();
}
void my_operator::set_range(std::shared_ptr<my_vector> ran) {
  scale = 1;
  range = ran->clone_space();
}

// my_operator.cc:13-59: <L m1, d2> = <m1, L' d2> for random m1, d2, first
// with add = false, then once more accumulating (add = true); relative
// tolerance 1e-4 on both
bool my_operator::dot_test(bool verb) {
  std::shared_ptr<my_vector> m1 = domain->clone_vec();
  std::shared_ptr<my_vector> m2 = m1->clone_vec();
  std::shared_ptr<my_vector> d1 = range->clone_vec();
  std::shared_ptr<my_vector> d2 = d1->clone_vec();
  m1->random();
  d2->random();
  forward(false, m1, d1);
  const double a = d1->dot(d2);
  adjoint(false, m2, d2);
  const double b = m2->dot(m1);
  if (verb) std::fprintf(stderr, "Dot(add=false) %g %g \n", a, b);
  forward(true, m1, d1);
  adjoint(true, m2, d2);
  const double c = m1->dot(m2);
  const double d = d1->dot(d2);
  if (verb) std::fprintf(stderr, "Dot(add=true) %g %g \n", d, c);
  if (std::fabs(a) < 1e-12 || std::fabs(c) < 1e-12) return false;
  if (std::fabs((a - b) / a) > .0001) return false;
  if (std::fabs((c - d) / c) > .0001) return false;
  return true;
}
