// The reference's least-squares loop restated from base/lin_solver.cc --
// TEST INFRASTRUCTURE ONLY.
#include "lin_solver.h"

#include <cstdio>

// lin_solver.cc:6-16 (no weighting operator: the operator itself is used)
simple_solver::simple_solver(step *s, std::shared_ptr<my_vector> data,
                             std::shared_ptr<my_operator> op,
                             std::shared_ptr<my_vector> m0) {
  init_solve(s);
  rr = init_rr(data, op, m0);
  oper = op;
  create_solver_vecs();
}

void lin_solver::init_solve(step *s) {
  st = s;
  verb = 0;
}

// lin_solver.cc:62-68: residual image, model, gradient, then the step's
// own vectors
void lin_solver::create_solver_vecs() {
  gg = rr->clone_zero();
  m = oper->domain->clone_zero();
  g = oper->domain->clone_zero();
  st->alloc_step(m, rr);
}

// lin_solver.cc:79-103 without weights: rr = -d (+ L m0)
std::shared_ptr<my_vector> lin_solver::init_rr(
    std::shared_ptr<my_vector> data, std::shared_ptr<my_operator> op,
    std::shared_ptr<my_vector> m0) {
  std::shared_ptr<my_vector> r = data->clone_vec();
  r->scale(-1.);
  if (m0) op->forward(true, m0, r);
  return r;
}

// lin_solver.cc:104-132: per iteration g = L' rr, gg = L g, then the step
bool lin_solver::solve(int niter) {
  for (int iter = 0; iter < niter; iter++) {
    oper->adjoint(false, g, rr, iter);
    oper->forward(false, g, gg, iter);
    double val = 0.;
    const bool valid = st->step_it(iter, m, g, rr, gg, &val);
    if (verb > 0) std::fprintf(stderr, "iteration %d rr.rr %g\n", iter, val);
    if (!valid) return false;
  }
  return true;
}
