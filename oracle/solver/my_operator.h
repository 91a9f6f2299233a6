// Restatement of the reference's operator interface, base/my_operator.h:6-50
// (and the members defined in base/my_operator.cc) -- TEST INFRASTRUCTURE
// ONLY; see my_vector.h of this folder.
#ifndef ORACLE_SOLVER_MY_OPERATOR_H
#define ORACLE_SOLVER_MY_OPERATOR_H
#include <memory>

#include "my_vector.h"

class my_operator {
 public:
  my_operator() {}
  virtual ~my_operator() {}
  virtual bool forward(bool add, std::shared_ptr<my_vector> model,
                       std::shared_ptr<my_vector> data, int iter = 1) {
    (void)add, (void)model, (void)data, (void)iter;
    return false;
  }
  virtual bool adjoint(bool add, std::shared_ptr<my_vector> model,
                       std::shared_ptr<my_vector> data, int iter = 1) {
    (void)add, (void)model, (void)data, (void)iter;
    return false;
  }
  void set_domain(std::shared_ptr<my_vector> dom);
  void set_range(std::shared_ptr<my_vector> ran);
  bool dot_test(bool verb);
  virtual void set_scale(float s) { scale = s; }

  float scale = 1.f;
  std::shared_ptr<my_vector> domain, range;
  bool solver_own = false;
};
#endif
