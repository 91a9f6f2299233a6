/* Minimal stand-in for the SEP genericIO header (SEP libraries are not
 * installed).  Test infrastructure only: cpuProp needs the parameter-object
 * type names; the geometry code reads "files", which here are in-memory
 * arrays registered by tag (register_file) before the reference code opens
 * them. */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "genericFile.h"
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
  std::shared_ptr<genericRegFile> getRegFile(const std::string &tag,
                                             usage_code) {
    return files()[tag];
  }
  static void register_file(const std::string &tag,
                            const std::vector<axis> &axes, const float *v) {
    const auto h = std::make_shared<hypercube>(axes);
    files()[tag] = std::make_shared<genericRegFile>(
        h, std::vector<float>(v, v + h->getN123()));
  }

 private:
  static std::map<std::string, std::shared_ptr<genericRegFile>> &files() {
    static std::map<std::string, std::shared_ptr<genericRegFile>> f;
    return f;
  }
};
}  // namespace SEP
