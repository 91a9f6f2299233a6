// born_my_operatorT / born_device_vectorT: the GB300 Born operator behind the
// reference's solver classes.
//
// The reference's least-squares code reaches an operator only through
//   bool my_operator::forward/adjoint(bool add, std::shared_ptr<my_vector>
//        model, std::shared_ptr<my_vector> data, int iter)
// (base/my_operator.h:18-25) and vectors only through the my_vector virtuals
// (base/my_vector.h:7-91).  lin_solver::solve (base/lin_solver.cc:104-132)
// and cgstep::step_it (base/cgstep.cc:11-54) call clone_vec, clone_space,
// clone_zero (via set_val), scale, scale_add, add, dot and info;
// my_operator::dot_test (base/my_operator.cc:13-59) adds random.  This header
// implements exactly those over the C ABI of libborn_gb300.so:
//
//  * born_device_vectorT<V> is a V (the reference's my_vector) whose values
//    live on the GPU; its algebra is hypercube_float's (double factors,
//    elements formed in double and stored as float, FP64 dot products), run
//    on the operator's stream by born_vec_* and born_dot_f64;
//  * born_my_operatorT<O, V> is an O (the reference's my_operator) whose
//    forward/adjoint are born_op_forward/born_op_adjoint on those vectors
//    (born_op honours the model and data vectors, which rtm_zero_op does
//    not: rtm_zero_op_3d.cc:161,193,295).
//
// In the reference tree:
//   typedef born_device_vectorT<my_vector> born_device_vector;
//   typedef born_my_operatorT<my_operator, my_vector> born_my_operator;
//   auto op = std::make_shared<born_my_operator>(born_op_handle);
//   auto data = op->data_vector();  data->upload(host_traces);
//   cgstep cg;  simple_solver solver(&cg, data, op);  solver.solve(niter);
// runs the reference's CG unchanged with every operator application and
// vector operation on the device.  The my_vector virtuals return void, so a
// failing call throws std::runtime_error (the reference asserts);
// forward/adjoint return false on failure and keep the status (status()).
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/born_gb300.h"

template <class V>
class born_device_vectorT : public V {
 public:
  born_device_vectorT(born_op *op, long long n) : op_(op), n_(n) {
    check(born_vec_create(op, n, &x_), "born_vec_create");
    this->name = "born_device_vector";
  }
  ~born_device_vectorT() { born_vec_destroy(op_, x_); }
  born_device_vectorT(const born_device_vectorT &) = delete;
  born_device_vectorT &operator=(const born_device_vectorT &) = delete;

  float *data() const { return x_; }
  long long size() const { return n_; }
  born_op *op() const { return op_; }
  void upload(const float *host) {
    check(born_vec_upload(op_, x_, host, n_), "born_vec_upload");
  }
  void download(float *host) const {
    check(born_vec_download(op_, host, x_, n_), "born_vec_download");
  }

  // ---- the my_vector virtuals lin_solver, cgstep and dot_test call ----
  virtual std::shared_ptr<V> clone_vec() {
    auto v = std::make_shared<born_device_vectorT>(op_, n_);
    check(born_vec_copy(op_, v->x_, x_, n_), "born_vec_copy");
    return v;
  }
  virtual std::shared_ptr<V> clone_space() {
    return std::make_shared<born_device_vectorT>(op_, n_);
  }
  virtual void scale(const double r) {
    check(born_vec_scale(op_, x_, n_, r), "born_vec_scale");
  }
  virtual void scale_add(const double mes, std::shared_ptr<V> vec,
                         const double other) {
    check(born_vec_scale_add(op_, x_, mes, of(vec)->x_, other, n_),
          "born_vec_scale_add");
  }
  virtual void scale_add(const double sc1, std::shared_ptr<V> v1, double sc2,
                         std::shared_ptr<V> v2) {
    check(born_vec_lincomb(op_, x_, sc1, of(v1)->x_, sc2, of(v2)->x_, n_),
          "born_vec_lincomb");
  }
  virtual void set_val(double val) {
    check(born_vec_fill(op_, x_, n_, val), "born_vec_fill");
  }
  virtual void add(std::shared_ptr<V> vec) {
    check(born_vec_add(op_, x_, of(vec)->x_, n_), "born_vec_add");
  }
  virtual double dot(std::shared_ptr<V> vec) {
    double out = 0.0;
    check(born_dot_f64(op_, x_, of(vec)->x_, n_, &out), "born_dot_f64");
    return out;
  }
  // hypercube_float::random (hypercube_float.cc:115-119), drawn on the host
  virtual void random() {
    std::vector<float> h((size_t)n_);
    for (auto &v : h) v = (float)rand() / (float)RAND_MAX - .5f;
    upload(h.data());
  }
  // the name and size (and, at level > 0, the L2 norm) on stderr
  virtual void info(char *str, int level = 0) {
    if (level > 0) {
      const double nrm = std::sqrt(dot_self());
      std::fprintf(stderr, "    NAME=%s TYPE=%s N=%lld |x|=%g\n", str,
                   this->name.c_str(), n_, nrm);
    } else {
      std::fprintf(stderr, "    NAME=%s TYPE=%s N=%lld\n", str,
                   this->name.c_str(), n_);
    }
  }
  virtual bool check_match(const std::shared_ptr<V> v2) {
    auto *o = dynamic_cast<born_device_vectorT *>(v2.get());
    return o && o->n_ == n_ && o->op_ == op_;
  }

  static born_device_vectorT *of(const std::shared_ptr<V> &v) {
    auto *p = dynamic_cast<born_device_vectorT *>(v.get());
    if (!p)
      throw std::invalid_argument(
          "born_gb300: vector is not a born_device_vector");
    return p;
  }

 private:
  double dot_self() {
    double out = 0.0;
    check(born_dot_f64(op_, x_, x_, n_, &out), "born_dot_f64");
    return out;
  }
  static void check(int rc, const char *what) {
    if (rc != BORN_OK)
      throw std::runtime_error(std::string("born_gb300: ") + what +
                               " failed (status " + std::to_string(rc) + ")");
  }

  born_op *op_ = nullptr;
  long long n_ = 0;
  float *x_ = nullptr;
};

template <class O, class V>
class born_my_operatorT : public O {
 public:
  typedef born_device_vectorT<V> vector_type;

  // op: an operator made by born_op_create (owned by the caller, which
  // destroys it after this object).  Domain: the model [n3][n2][n1]; range:
  // the data [nshots][rec_ny][rec_nx][nt_data].
  explicit born_my_operatorT(born_op *op) : op_(op) {
    int nt = 0;
    float dt = 0.f;
    status_ = born_op_sizes(op, &model_n_, &data_n_, &nt, &dt);
    if (status_ != BORN_OK)
      throw std::runtime_error("born_gb300: born_op_sizes failed");
    this->set_domain(model_vector());
    this->set_range(data_vector());
  }

  std::shared_ptr<vector_type> model_vector() const {
    return std::make_shared<vector_type>(op_, model_n_);
  }
  std::shared_ptr<vector_type> data_vector() const {
    return std::make_shared<vector_type>(op_, data_n_);
  }

  // my_operator.h:18-25; add = false overwrites the output
  virtual bool forward(bool add, std::shared_ptr<V> model,
                       std::shared_ptr<V> data, int iter = 1) {
    (void)iter;
    status_ = born_op_forward(op_, add ? 1 : 0, vector_type::of(model)->data(),
                              vector_type::of(data)->data());
    return status_ == BORN_OK;
  }
  virtual bool adjoint(bool add, std::shared_ptr<V> model,
                       std::shared_ptr<V> data, int iter = 1) {
    (void)iter;
    status_ = born_op_adjoint(op_, add ? 1 : 0, vector_type::of(model)->data(),
                              vector_type::of(data)->data());
    return status_ == BORN_OK;
  }

  int status() const { return status_; }
  born_op *op() const { return op_; }

 private:
  born_op *op_ = nullptr;
  long long model_n_ = 0, data_n_ = 0;
  int status_ = BORN_OK;
};
