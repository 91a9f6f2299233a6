// Restatement of the reference's solver driver, base/lin_solver.h:6-44
// (lin_solver and simple_solver without weights) -- TEST INFRASTRUCTURE
// ONLY.
#ifndef ORACLE_SOLVER_LIN_SOLVER_H
#define ORACLE_SOLVER_LIN_SOLVER_H
#include "cgstep.h"
#include "my_operator.h"

class lin_solver {
 public:
  lin_solver() {}
  virtual ~lin_solver() {}
  void set_verbose(int iv) { verb = iv; }
  bool solve(int niter);
  void init_solve(step *s);
  void create_solver_vecs();
  std::shared_ptr<my_vector> init_rr(std::shared_ptr<my_vector> data,
                                     std::shared_ptr<my_operator> op,
                                     std::shared_ptr<my_vector> m0);
  virtual void update_model(std::shared_ptr<my_vector> mod) { mod->add(m); }
  virtual std::shared_ptr<my_vector> return_model() { return m->clone_vec(); }

  std::shared_ptr<my_vector> g, m, gg, rr;
  std::shared_ptr<my_operator> oper;
  int verb = 0;
  step *st = nullptr;
};

class simple_solver : public lin_solver {
 public:
  simple_solver(step *s, std::shared_ptr<my_vector> data,
                std::shared_ptr<my_operator> op,
                std::shared_ptr<my_vector> m0 = nullptr);
};
#endif
