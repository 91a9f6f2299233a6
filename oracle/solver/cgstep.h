// Restatement of base/cgstep.h:5-26 -- TEST INFRASTRUCTURE ONLY.
#ifndef ORACLE_SOLVER_CGSTEP_H
#define ORACLE_SOLVER_CGSTEP_H
#include "step.h"

class cgstep : public step {
 public:
  virtual bool step_it(int iter, std::shared_ptr<my_vector> x,
                       std::shared_ptr<my_vector> g,
                       std::shared_ptr<my_vector> rr,
                       std::shared_ptr<my_vector> gg, double *sc);
  virtual void alloc_step(std::shared_ptr<my_vector> mod,
                          std::shared_ptr<my_vector> dat);
  void forget_it();

 private:
  std::shared_ptr<my_vector> s, ss;
  bool forget = true;
  double small = 1e-20;
};
#endif
