// SEP regular-file I/O for the arrays that cross the operator boundary
// (velocity, wavelet, shot data, image), so reference datasets can be used
// as they are.  The reference reads and writes them through SEP genericIO
// (vel_fd_3d.cc:7-14, data_rtm_3d.cc:4-20, image_rtm_3d.cc:4-16), which is
// not part of this build.  A SEP header is text made of key=value pairs
// (later pairs override earlier ones): n1..n6, o1..o6, d1..d6, label1..,
// esize, data_format ("xdr_float" = big-endian IEEE, "native_float" = host
// order) and in= the path of the binary data (relative paths are taken
// relative to the header's folder; "stdin" is not supported).
#include "born_host.h"

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/born_gb300.h"

namespace {

std::map<std::string, std::string> parse_header(const std::string &text) {
  std::map<std::string, std::string> kv;
  size_t i = 0;
  const size_t n = text.size();
  while (i < n) {
    while (i < n && (std::isspace((unsigned char)text[i]))) ++i;
    if (i < n && text[i] == '#') {  // comment to end of line
      while (i < n && text[i] != '\n') ++i;
      continue;
    }
    size_t k0 = i;
    while (i < n && !std::isspace((unsigned char)text[i]) && text[i] != '=')
      ++i;
    std::string key = text.substr(k0, i - k0);
    if (i < n && text[i] == '=' && !key.empty()) {
      ++i;
      std::string val;
      if (i < n && (text[i] == '"' || text[i] == '\'')) {
        const char q = text[i++];
        size_t v0 = i;
        while (i < n && text[i] != q) ++i;
        val = text.substr(v0, i - v0);
        if (i < n) ++i;
      } else {
        size_t v0 = i;
        while (i < n && !std::isspace((unsigned char)text[i])) ++i;
        val = text.substr(v0, i - v0);
      }
      kv[key] = val;
    } else {
      while (i < n && !std::isspace((unsigned char)text[i])) ++i;
    }
  }
  return kv;
}

std::string dirname_of(const std::string &p) {
  const size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

bool little_endian_host() {
  const unsigned int one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

void swap4(float *v, long long n) {
  for (long long i = 0; i < n; ++i) {
    unsigned char *b = reinterpret_cast<unsigned char *>(v + i);
    std::swap(b[0], b[3]);
    std::swap(b[1], b[2]);
  }
}

int read_info(const char *path, born_sep_info *info, std::string *data_path) {
  std::ifstream f(path);
  if (!f) return BORN_EINVAL;
  std::stringstream ss;
  ss << f.rdbuf();
  auto kv = parse_header(ss.str());
  std::memset(info, 0, sizeof(*info));
  info->ndim = 0;
  for (int a = 0; a < 6; ++a) {
    const std::string na = "n" + std::to_string(a + 1);
    info->n[a] = kv.count(na) ? std::atoll(kv[na].c_str()) : 1;
    info->o[a] = kv.count("o" + std::to_string(a + 1))
                     ? (float)std::atof(kv["o" + std::to_string(a + 1)].c_str())
                     : 0.f;
    info->d[a] = kv.count("d" + std::to_string(a + 1))
                     ? (float)std::atof(kv["d" + std::to_string(a + 1)].c_str())
                     : 1.f;
    if (kv.count(na)) info->ndim = a + 1;
  }
  const std::string fmt = kv.count("data_format") ? kv["data_format"]
                                                  : std::string("xdr_float");
  if (fmt == "xdr_float")
    info->big_endian = 1;
  else if (fmt == "native_float")
    info->big_endian = little_endian_host() ? 0 : 1;
  else
    return BORN_EINVAL;  // only 4-byte IEEE floats are supported
  if (kv.count("esize") && kv["esize"] != "4") return BORN_EINVAL;
  if (!kv.count("in")) return BORN_EINVAL;
  std::string in = kv["in"];
  if (in == "stdin" || in == "-") return BORN_EINVAL;
  if (!in.empty() && in[0] != '/') in = dirname_of(path) + "/" + in;
  if (data_path) *data_path = in;
  std::snprintf(info->in, sizeof(info->in), "%s", in.c_str());
  return BORN_OK;
}

}  // namespace

extern "C" {

int born_sep_read_info(const char *header, born_sep_info *info) {
  if (!header || !info) return BORN_EINVAL;
  return read_info(header, info, nullptr);
}

int born_sep_read(const char *header, float *out, long long count) {
  if (!header || !out || count < 0) return BORN_EINVAL;
  born_sep_info info;
  std::string data;
  int rc = read_info(header, &info, &data);
  if (rc) return rc;
  long long total = 1;
  for (int a = 0; a < 6; ++a) total *= info.n[a];
  if (count != total) return BORN_EINVAL;
  std::FILE *f = std::fopen(data.c_str(), "rb");
  if (!f) return BORN_EINVAL;
  const size_t got = std::fread(out, 4, (size_t)count, f);
  std::fclose(f);
  if ((long long)got != count) return BORN_EINVAL;
  if (info.big_endian == (little_endian_host() ? 1 : 0)) swap4(out, count);
  return BORN_OK;
}

int born_sep_write(const char *header, const born_sep_info *info,
                   const float *data, int big_endian) {
  if (!header || !info || !data || info->ndim < 1 || info->ndim > 6)
    return BORN_EINVAL;
  long long total = 1;
  for (int a = 0; a < info->ndim; ++a) total *= info->n[a];
  std::string bin = std::string(header) + "@";
  std::FILE *hf = std::fopen(header, "w");
  if (!hf) return BORN_EINVAL;
  for (int a = 0; a < info->ndim; ++a)
    std::fprintf(hf, "n%d=%lld o%d=%.9g d%d=%.9g\n", a + 1, info->n[a], a + 1,
                 (double)info->o[a], a + 1, (double)info->d[a]);
  const size_t slash = bin.find_last_of('/');
  const std::string rel = slash == std::string::npos ? bin : bin.substr(slash + 1);
  std::fprintf(hf, "esize=4 data_format=\"%s\" in=\"%s\"\n",
               big_endian ? "xdr_float" : "native_float", rel.c_str());
  std::fclose(hf);
  std::FILE *df = std::fopen(bin.c_str(), "wb");
  if (!df) return BORN_EINVAL;
  const bool swap = (big_endian != 0) == little_endian_host();
  std::vector<float> buf(1 << 16);
  long long done = 0;
  while (done < total) {
    const long long m = std::min<long long>((long long)buf.size(), total - done);
    std::memcpy(buf.data(), data + done, (size_t)m * 4);
    if (swap) swap4(buf.data(), m);
    if (std::fwrite(buf.data(), 4, (size_t)m, df) != (size_t)m) {
      std::fclose(df);
      return BORN_EINVAL;
    }
    done += m;
  }
  std::fclose(df);
  return BORN_OK;
}

}  // extern "C"
