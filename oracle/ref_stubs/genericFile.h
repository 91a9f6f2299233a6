/* Stand-in for the SEP regular-file interface the reference's velocity and
 * wavelet readers use.  Test infrastructure only: a "file" is an in-memory
 * hypercube and its floats (see genericIO.h). */
#pragma once
#include <cstring>
#include <memory>
#include <vector>

#include "hypercube.h"
namespace SEP {
enum usage_code { usageIn, usageOut, usageInOut, usageScr };
class genericRegFile {
 public:
  genericRegFile(std::shared_ptr<hypercube> h, std::vector<float> v)
      : hyper_(h), vals_(std::move(v)) {}
  std::shared_ptr<hypercube> getHyper() { return hyper_; }
  void readFloatStream(float *out, long long n) {
    std::memcpy(out, vals_.data() + pos_, sizeof(float) * (size_t)n);
    pos_ += n;
  }
  void writeFloatStream(const float *in, long long n) {
    if ((long long)vals_.size() < pos_ + n) vals_.resize(pos_ + n);
    std::memcpy(vals_.data() + pos_, in, sizeof(float) * (size_t)n);
    pos_ += n;
  }
  // byte offset, whence 0 (from the start) as the reference uses it
  void seekTo(long long bytes, int) { pos_ = bytes / (long long)sizeof(float); }

 private:
  std::shared_ptr<hypercube> hyper_;
  std::vector<float> vals_;
  long long pos_ = 0;  // in floats
};
}  // namespace SEP
