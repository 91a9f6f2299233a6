// Claerbout's conjugate-gradient step, restated from base/cgstep.cc:1-54 --
// TEST INFRASTRUCTURE ONLY.  The first step is a steepest descent
// (alfa = -<gg, rr> / <gg, gg>); later steps solve the 2 x 2 system for the
// combination of the new direction g (data-space image gg) and the previous
// step s (image ss) that minimises |rr + alfa gg + beta ss|, with the
// reference's determinant form and its 1e-20 guards.
#include "cgstep.h"

#include <cmath>
#include <cstdio>

void cgstep::alloc_step(std::shared_ptr<my_vector> mod,
                        std::shared_ptr<my_vector> dat) {
  s = mod->clone_vec();
  ss = dat->clone_vec();
  forget_it();
}

void cgstep::forget_it() {
  forget = true;
  s->zero();
  ss->zero();
  small = 1e-20;
}

bool cgstep::step_it(int iter, std::shared_ptr<my_vector> m,
                     std::shared_ptr<my_vector> g,
                     std::shared_ptr<my_vector> rr,
                     std::shared_ptr<my_vector> gg, double *vv) {
  (void)iter;
  double alfa, beta;
  const double gg_gg = gg->dot(gg);
  if (forget) {
    if (std::fabs(gg_gg) < small) return false;
    beta = 0;
    alfa = -gg->dot(rr) / gg_gg;
  } else {
    const double ss_ss = ss->dot(ss);
    const double gg_ss = gg->dot(ss);
    if (std::fabs(gg_gg) < small || std::fabs(ss_ss) < small) return false;
    const double det = gg_gg * ss_ss * (1.0 - gg_ss / gg_gg * gg_ss / ss_ss);
    const double gr = -gg->dot(rr);
    const double sr = -ss->dot(rr);
    alfa = (ss_ss * gr - gg_ss * sr) / det;
    beta = (-gg_ss * gr + gg_gg * sr) / det;
  }
  s->scale_add(beta, g, alfa);    // s  = beta s  + alfa g
  ss->scale_add(beta, gg, alfa);  // ss = beta ss + alfa gg
  m->add(s);
  rr->add(ss);
  *vv = rr->dot(rr);
  forget = false;
  return true;
}
