// Runs the least-squares loop of whichever solver classes it is compiled
// against (the reference's base/lin_solver.cc + cgstep.cc, or the
// restatement in oracle/solver) on a small dense operator with host vectors
// that follow hypercube_float's arithmetic (base/hypercube_float.cc), and
// prints rr.rr after every iteration, the final model's dot with itself and
// the dot-product test, all with 17 significant digits.  The two builds must
// print the same text.
//   pin_solver <niter>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "cgstep.h"
#include "lin_solver.h"
#include "my_operator.h"
#include "my_vector.h"

class host_vector : public my_vector {
 public:
  explicit host_vector(size_t n) : v(n, 0.f) { name = "host_vector"; }
  std::vector<float> v;
  static host_vector *of(const std::shared_ptr<my_vector> &p) {
    return dynamic_cast<host_vector *>(p.get());
  }
  std::shared_ptr<my_vector> clone_vec() {
    auto c = std::make_shared<host_vector>(v.size());
    c->v = v;
    return c;
  }
  std::shared_ptr<my_vector> clone_space() {
    return std::make_shared<host_vector>(v.size());
  }
  void scale(const double r) {
    for (auto &x : v) x = x * r;
  }
  void scale_add(const double mes, std::shared_ptr<my_vector> vec,
                 const double other) {
    const host_vector *o = of(vec);
    for (size_t i = 0; i < v.size(); ++i) v[i] = v[i] * mes + other * o->v[i];
  }
  void scale_add(const double sc1, std::shared_ptr<my_vector> v1, double sc2,
                 std::shared_ptr<my_vector> v2) {
    const host_vector *a = of(v1), *b = of(v2);
    for (size_t i = 0; i < v.size(); ++i) v[i] = a->v[i] * sc1 + b->v[i] * sc2;
  }
  void set_val(double val) {
    for (auto &x : v) x = val;
  }
  void add(std::shared_ptr<my_vector> vec) {
    const host_vector *o = of(vec);
    for (size_t i = 0; i < v.size(); ++i) v[i] += o->v[i];
  }
  double dot(std::shared_ptr<my_vector> vec) {
    const host_vector *o = of(vec);
    double s = 0;
    for (size_t i = 0; i < v.size(); ++i) s += (double)v[i] * (double)o->v[i];
    return s;
  }
  void info(char *, int) {}
  void random() {
    for (auto &x : v) x = (float)rand() / (float)RAND_MAX - .5f;
  }
  bool check_match(const std::shared_ptr<my_vector> v2) {
    return of(v2) && of(v2)->v.size() == v.size();
  }
};

// d = A m with A (nd x nm) of fixed pseudo-random entries, sums in double
class dense_op : public my_operator {
 public:
  dense_op(int nd_, int nm_) : nd(nd_), nm(nm_), a((size_t)nd_ * nm_) {
    unsigned s = 12345u;
    for (auto &x : a) {
      s = s * 1103515245u + 12345u;
      x = (float)((s >> 8) & 0xffff) / 65536.f - .5f;
    }
    set_domain(std::make_shared<host_vector>(nm));
    set_range(std::make_shared<host_vector>(nd));
  }
  bool forward(bool add, std::shared_ptr<my_vector> model,
               std::shared_ptr<my_vector> data, int iter = 1) {
    (void)iter;
    const host_vector *m = host_vector::of(model);
    host_vector *d = host_vector::of(data);
    for (int i = 0; i < nd; ++i) {
      double s = add ? d->v[i] : 0.0;
      for (int j = 0; j < nm; ++j) s += (double)a[(size_t)i * nm + j] * m->v[j];
      d->v[i] = (float)s;
    }
    return true;
  }
  bool adjoint(bool add, std::shared_ptr<my_vector> model,
               std::shared_ptr<my_vector> data, int iter = 1) {
    (void)iter;
    host_vector *m = host_vector::of(model);
    const host_vector *d = host_vector::of(data);
    for (int j = 0; j < nm; ++j) {
      double s = add ? m->v[j] : 0.0;
      for (int i = 0; i < nd; ++i) s += (double)a[(size_t)i * nm + j] * d->v[i];
      m->v[j] = (float)s;
    }
    return true;
  }
  int nd, nm;
  std::vector<float> a;
};

int main(int argc, char **argv) {
  const int niter = argc > 1 ? std::atoi(argv[1]) : 6;
  auto op = std::make_shared<dense_op>(60, 40);
  auto mtrue = std::make_shared<host_vector>(40);
  for (int j = 0; j < 40; ++j) mtrue->v[j] = (j % 7 == 3) ? 1.f : 0.f;
  auto data = std::make_shared<host_vector>(60);
  op->forward(false, mtrue, data);
  cgstep cg;
  simple_solver solver(&cg, data, op);
  std::printf("rr0 %.17g\n", solver.rr->dot(solver.rr));
  for (int it = 0; it < niter; ++it) {
    if (!solver.solve(1)) {
      std::printf("stopped %d\n", it);
      break;
    }
    std::printf("rr%d %.17g\n", it + 1, solver.rr->dot(solver.rr));
  }
  std::printf("mm %.17g\n", solver.m->dot(solver.m));
  srand(7);
  std::printf("dot_test %d\n", op->dot_test(false) ? 1 : 0);
  return 0;
}
