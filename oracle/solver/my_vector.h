// Restatement of the reference's vector interface, base/my_vector.h:7-91 --
// TEST INFRASTRUCTURE ONLY (with my_operator.h, step.h, cgstep.h and
// lin_solver.h of this folder it lets the reference's least-squares loop
// run where the reference's sources are absent; tests pin it against the
// reference's own lin_solver/cgstep where they are present).  Only the
// virtuals the solver loop and the operator adapter use are declared; their
// names and signatures are the reference's, because the adapter overrides
// them.  Default bodies fail as the reference's assert(0 == 1) bodies do.
#ifndef ORACLE_SOLVER_MY_VECTOR_H
#define ORACLE_SOLVER_MY_VECTOR_H
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

class my_vector {
 public:
  my_vector() {}
  virtual ~my_vector() {}
  virtual std::shared_ptr<my_vector> clone_vec() { return nullptr; }
  virtual std::shared_ptr<my_vector> clone_space() { return nullptr; }
  virtual std::shared_ptr<my_vector> clone_zero() {
    std::shared_ptr<my_vector> v = clone_vec();
    v->zero();
    return v;
  }
  virtual void scale(const double) { unimplemented("scale"); }
  virtual void scale_add(const double, std::shared_ptr<my_vector>,
                         const double) {
    unimplemented("scale_add");
  }
  // base/my_vector.h:64-68: two passes of the three-argument form
  virtual void scale_add(const double sc1, std::shared_ptr<my_vector> v1,
                         double sc2, std::shared_ptr<my_vector> v2) {
    scale_add(0., v1, sc1);
    scale_add(1., v2, sc2);
  }
  virtual void set_val(double) { unimplemented("set_val"); }
  virtual void add(std::shared_ptr<my_vector>) { unimplemented("add"); }
  virtual double dot(std::shared_ptr<my_vector>) {
    unimplemented("dot");
    return 0.;
  }
  virtual void info(char *, int level = 0) {
    (void)level;
    unimplemented("info");
  }
  virtual void random() { unimplemented("random"); }
  virtual bool check_match(const std::shared_ptr<my_vector> v2) {
    return name != v2->name;  // as base/my_vector.h:82-87 returns it
  }
  void zero() { set_val(0.); }
  std::string name;

 private:
  static void unimplemented(const char *what) {
    std::fprintf(stderr, "my_vector::%s is not implemented\n", what);
    std::abort();
  }
};
#endif
