// gb300PropT<Base>: the GB300 propagator behind the reference's C++
// propagator interface.
//
// The reference's operator talks to a propagator only through the virtuals
// of baseProp (base/base_prop.h:4-72): createSpace, transferSincTableS/D,
// setNtblock, transferSourceFunc, transferVelFunc1/2, transferReceiverFunc,
// sourceProp, rtmAdjoint, rtmForward.  This header implements exactly those
// signatures over the C ABI of libborn_gb300.so, with the semantics of the
// reference CPU propagator cpuProp (base/cpu_prop.cc):
//
//  * transferReceiverFunc retains the trace array; rtmForward accumulates the
//    modelled traces into it (cpu_prop.cc:205-212);
//  * sourceProp leaves the final two levels in p0/p1, as cpuProp does
//    whatever getLast says (cpu_prop.cc:106-129), and keeps them on the
//    device;
//  * rtmAdjoint reads the levels through born_rtm_adjoint_host: by default
//    the arrays sourceProp filled (in either order) select the
//    device-resident levels without a copy and any other host arrays are
//    uploaded; born_set_host_levels(handle(), ...) makes it verify the
//    arrays' contents by checksum or always upload them.  The image is
//    accumulated into img (cpu_prop.cc:101).
//
// Base is the class to derive from: in the reference tree,
//   typedef gb300PropT<baseProp> gb300Prop;
// gives a drop-in replacement for cpuProp/gpuProp.  The virtuals are declared
// without `override` so that any Base with these virtuals (or none) works.
// The reference's virtuals return void and never report errors; this class
// records the status of every call (status(), error()) and, if
// set_throw(true), throws std::runtime_error instead.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/born_gb300.h"

template <class Base>
class gb300PropT : public Base {
 public:
  explicit gb300PropT(int device = 0) {
    status_ = born_create(device, &h_);
    if (status_ != BORN_OK) h_ = nullptr;
  }
  ~gb300PropT() { born_destroy(h_); }
  gb300PropT(const gb300PropT &) = delete;
  gb300PropT &operator=(const gb300PropT &) = delete;

  int status() const { return status_; }
  std::string error() const { return h_ ? born_error_string(h_) : "no device"; }
  void set_throw(bool t) { throw_ = t; }
  born_handle *handle() { return h_; }

  virtual void setNtblock(int nb) { (void)nb; }

  virtual void createSpace(float d1, float d2, float d3, float bc_a,
                           float bc_b, float bc_y, int nx, int ny, int nz) {
    if (!ready()) return;
    done(born_create_space(h_, d1, d2, d3, bc_a, bc_b, bc_y, nx, ny, nz));
  }

  virtual void transferSincTableS(int nsinc, int jts,
                                  std::vector<std::vector<float>> &table) {
    if (!ready()) return;
    std::vector<float> flat = flatten(table);
    done(born_set_sinc_table(h_, 0, nsinc, jts, flat.data()));
  }

  virtual void transferSincTableD(int nsinc, int jtd,
                                  std::vector<std::vector<float>> &table) {
    if (!ready()) return;
    std::vector<float> flat = flatten(table);
    done(born_set_sinc_table(h_, 1, nsinc, jtd, flat.data()));
  }

  virtual void transferSourceFunc(int npts, int nt_big, std::vector<int> &locs,
                                  float *vals) {
    if (!ready()) return;
    done(born_set_source_func(h_, npts, nt_big, locs.data(), vals));
  }

  virtual void transferVelFunc1(int nx, int ny, int nz, float *vloc) {
    if (!ready()) return;
    done(born_set_velocity(h_, 1, nx, ny, nz, vloc));
  }

  virtual void transferVelFunc2(int nx, int ny, int nz, float *vloc) {
    if (!ready()) return;
    done(born_set_velocity(h_, 2, nx, ny, nz, vloc));
  }

  virtual void transferReceiverFunc(int nx, int ny, int nt,
                                    std::vector<int> &locs, float *rec) {
    if (!ready()) return;
    rec_ = rec;
    done(born_set_receiver_func(h_, nx, ny, nt, locs.data(), rec));
  }

  virtual void sourceProp(int nx, int ny, int nz, bool damp, bool getLast,
                          float *p0, float *p1, int jts, int npts, int nt) {
    (void)nx, (void)ny, (void)nz, (void)damp, (void)npts;
    if (!ready()) return;
    (void)getLast;
    done(born_source_prop(h_, jts, nt, p0, p1));
  }

  virtual void rtmAdjoint(int n1, int n2, int n3, int jtd, float *p0,
                          float *p1, float *img, int npts_s, int nt) {
    (void)n1, (void)n2, (void)n3, (void)npts_s;
    if (!ready()) return;
    // the handle's host-level policy decides whether p0/p1 are read or the
    // device-resident levels source_prop left are used
    done(born_rtm_adjoint_host(h_, jtd, nt, p0, p1, img));
  }

  virtual void rtmForward(int n1, int n2, int n3, int jt, float *img,
                          float *rec, int npts, int nt, int nt_big,
                          int rec_nx, int rec_ny) {
    (void)n1, (void)n2, (void)n3, (void)npts, (void)nt_big, (void)rec_nx,
        (void)rec_ny;
    if (!ready()) return;
    if (!done(born_set_reflectivity(h_, img))) return;
    done(born_rtm_forward(h_, jt, nt, rec_ ? rec_ : rec));
  }

 private:
  static std::vector<float> flatten(
      const std::vector<std::vector<float>> &table) {
    std::vector<float> flat;  // row-major, as gpu_prop.cc:15-24 flattens
    for (const auto &row : table) flat.insert(flat.end(), row.begin(), row.end());
    return flat;
  }
  bool ready() {
    if (h_) return true;
    status_ = BORN_ENODEV;
    if (throw_) throw std::runtime_error("born_gb300: no device handle");
    return false;
  }
  bool done(int rc) {
    status_ = rc;
    if (rc != BORN_OK && throw_)
      throw std::runtime_error(std::string("born_gb300: ") +
                               born_error_string(h_));
    return rc == BORN_OK;
  }

  born_handle *h_ = nullptr;
  int status_ = BORN_OK;
  bool throw_ = false;
  float *rec_ = nullptr;
};
