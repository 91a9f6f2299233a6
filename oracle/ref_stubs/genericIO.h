/* Minimal stand-in for the SEP genericIO header that the reference's
 * base/base_prop.h includes (SEP libraries are not installed).  Test
 * infrastructure only: cpuProp needs the type names and nothing else. */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <vector>
namespace SEP {
class paramObj {
 public:
  int getInt(const std::string &, int def) const { return def; }
  float getFloat(const std::string &, float def) const { return def; }
};
class genericIO {
 public:
  std::shared_ptr<paramObj> getParamObj() {
    return std::make_shared<paramObj>();
  }
};
}  // namespace SEP
