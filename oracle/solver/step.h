// Restatement of base/step.h:5-16 -- TEST INFRASTRUCTURE ONLY.
#ifndef ORACLE_SOLVER_STEP_H
#define ORACLE_SOLVER_STEP_H
#include "my_vector.h"

class step {
 public:
  step() {}
  virtual ~step() {}
  virtual void alloc_step(std::shared_ptr<my_vector> mod,
                          std::shared_ptr<my_vector> dat) {
    (void)mod, (void)dat;
  }
  virtual bool step_it(int iter, std::shared_ptr<my_vector> x,
                       std::shared_ptr<my_vector> g,
                       std::shared_ptr<my_vector> rr,
                       std::shared_ptr<my_vector> gg, double *sc) {
    (void)iter, (void)x, (void)g, (void)rr, (void)gg, (void)sc;
    return false;
  }
};
#endif
