// Regular-file I/O for the arrays that cross the operator boundary
// (velocity, wavelet, shot data, image), so reference datasets can be used
// as they are.  The reference reads and writes them through SEP genericIO
// (vel_fd_3d.cc:7-14, data_rtm_3d.cc:4-20, image_rtm_3d.cc:4-16), which is
// not part of this build; its two regular-file kinds are read and written
// here:
//  * SEP: a text header of key=value pairs (later pairs override earlier
//    ones): n1..n6, o1..o6, d1..d6, label1.., esize, data_format
//    ("xdr_float" = big-endian IEEE, "native_float" = host order) and in=
//    the path of the binary data (relative paths are taken relative to the
//    header's folder; "stdin" is not supported);
//  * JSON: a JSON object with the same axis keys (numbers), label1.. and
//    "filename", the binary data file (the form scripts/run.py:20-36 writes
//    for the images it adds), 4-byte floats in host order unless
//    "data_format" says "xdr_float".
// util/Add (util/Add.cc:1-41) becomes born_add_regfiles: the sum of two
// regular files of the same size, streamed in blocks, into a third.
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

// ---- JSON regular files ----

// Values of a flat JSON object: strings unescaped, numbers and literals as
// their text; nested arrays and objects are skipped.  Returns false on a
// syntax error.
bool parse_json_object(const std::string &t, std::map<std::string, std::string> *kv) {
  size_t i = 0;
  const size_t n = t.size();
  auto ws = [&]() {
    while (i < n && std::isspace((unsigned char)t[i])) ++i;
  };
  auto str = [&](std::string *out) {
    if (i >= n || t[i] != '"') return false;
    ++i;
    std::string v;
    while (i < n && t[i] != '"') {
      if (t[i] == '\\' && i + 1 < n) {
        const char c = t[++i];
        v += c == 'n' ? '\n' : c == 't' ? '\t' : c;
      } else {
        v += t[i];
      }
      ++i;
    }
    if (i >= n) return false;
    ++i;
    *out = v;
    return true;
  };
  ws();
  if (i >= n || t[i] != '{') return false;
  ++i;
  ws();
  if (i < n && t[i] == '}') return true;
  while (i < n) {
    ws();
    std::string key;
    if (!str(&key)) return false;
    ws();
    if (i >= n || t[i] != ':') return false;
    ++i;
    ws();
    std::string val;
    if (i < n && t[i] == '"') {
      if (!str(&val)) return false;
    } else if (i < n && (t[i] == '[' || t[i] == '{')) {
      int depth = 0;
      bool in_str = false;
      for (; i < n; ++i) {
        const char c = t[i];
        if (in_str) {
          if (c == '\\') ++i;
          else if (c == '"') in_str = false;
        } else if (c == '"') {
          in_str = true;
        } else if (c == '[' || c == '{') {
          ++depth;
        } else if (c == ']' || c == '}') {
          if (--depth == 0) {
            ++i;
            break;
          }
        }
      }
    } else {
      const size_t v0 = i;
      while (i < n && t[i] != ',' && t[i] != '}' &&
             !std::isspace((unsigned char)t[i]))
        ++i;
      val = t.substr(v0, i - v0);
    }
    (*kv)[key] = val;
    ws();
    if (i < n && t[i] == ',') {
      ++i;
      continue;
    }
    if (i < n && t[i] == '}') return true;
    return false;
  }
  return false;
}

int read_json_info(const char *path, born_sep_info *info,
                   std::string *data_path) {
  std::ifstream f(path);
  if (!f) return BORN_EINVAL;
  std::stringstream ss;
  ss << f.rdbuf();
  std::map<std::string, std::string> kv;
  if (!parse_json_object(ss.str(), &kv)) return BORN_EINVAL;
  std::memset(info, 0, sizeof(*info));
  for (int a = 0; a < 6; ++a) {
    const std::string k = std::to_string(a + 1);
    info->n[a] = kv.count("n" + k) ? std::atoll(kv["n" + k].c_str()) : 1;
    info->o[a] = kv.count("o" + k) ? (float)std::atof(kv["o" + k].c_str()) : 0.f;
    info->d[a] = kv.count("d" + k) ? (float)std::atof(kv["d" + k].c_str()) : 1.f;
    if (kv.count("n" + k)) info->ndim = a + 1;
    if (info->n[a] < 1) return BORN_EINVAL;
  }
  if (kv.count("esize") && kv["esize"] != "4") return BORN_EINVAL;
  const std::string fmt =
      kv.count("data_format") ? kv["data_format"] : std::string("native_float");
  if (fmt == "xdr_float")
    info->big_endian = 1;
  else if (fmt == "native_float" || fmt == "float")
    info->big_endian = little_endian_host() ? 0 : 1;
  else
    return BORN_EINVAL;
  std::string in = kv.count("filename") ? kv["filename"]
                                        : std::string(path) + ".dat";
  if (!in.empty() && in[0] != '/') in = dirname_of(path) + "/" + in;
  if (data_path) *data_path = in;
  std::snprintf(info->in, sizeof(info->in), "%s", in.c_str());
  return BORN_OK;
}

bool is_json_path(const char *path) {
  const std::string p(path);
  return p.size() >= 5 && p.compare(p.size() - 5, 5, ".json") == 0;
}

int read_any_info(const char *path, born_sep_info *info, std::string *data) {
  return is_json_path(path) ? read_json_info(path, info, data)
                            : read_info(path, info, data);
}

// Elements of a file: the product of the first ndim axis lengths (a
// description made by a caller may leave the higher axes unset).
long long total_of(const born_sep_info &info) {
  long long t = 1;
  for (int a = 0; a < info.ndim && a < 6; ++a) t *= info.n[a];
  return t;
}

// Writes count floats from data into an open file, byte-swapped when the
// file's order is not the host's.
bool write_floats(std::FILE *f, const float *data, long long count,
                  bool swap) {
  std::vector<float> buf(1 << 16);
  long long done = 0;
  while (done < count) {
    const long long m = std::min<long long>((long long)buf.size(), count - done);
    std::memcpy(buf.data(), data + done, (size_t)m * 4);
    if (swap) swap4(buf.data(), m);
    if (std::fwrite(buf.data(), 4, (size_t)m, f) != (size_t)m) return false;
    done += m;
  }
  return true;
}

// The description of a regular file: SEP header (data in path + "@",
// big-endian) or JSON (data in path + ".dat", host order).
int write_description(const char *path, const born_sep_info *info,
                      bool *swap, std::string *data_path) {
  const bool json = is_json_path(path);
  std::string bin = std::string(path) + (json ? ".dat" : "@");
  const size_t slash = bin.find_last_of('/');
  const std::string rel =
      slash == std::string::npos ? bin : bin.substr(slash + 1);
  std::FILE *hf = std::fopen(path, "w");
  if (!hf) return BORN_EINVAL;
  if (json) {
    std::fprintf(hf, "{\n");
    for (int a = 0; a < info->ndim; ++a)
      std::fprintf(hf,
                   "    \"n%d\": %lld,\n    \"o%d\": %.9g,\n    \"d%d\": "
                   "%.9g,\n    \"label%d\": \"Undefined\",\n",
                   a + 1, info->n[a], a + 1, (double)info->o[a], a + 1,
                   (double)info->d[a], a + 1);
    std::fprintf(hf, "    \"esize\": 4,\n    \"data_format\": \"native_float\",\n"
                     "    \"filename\": \"%s\"\n}\n",
                 rel.c_str());
    *swap = false;
  } else {
    for (int a = 0; a < info->ndim; ++a)
      std::fprintf(hf, "n%d=%lld o%d=%.9g d%d=%.9g\n", a + 1, info->n[a],
                   a + 1, (double)info->o[a], a + 1, (double)info->d[a]);
    std::fprintf(hf, "esize=4 data_format=\"xdr_float\" in=\"%s\"\n",
                 rel.c_str());
    *swap = little_endian_host();
  }
  std::fclose(hf);
  *data_path = bin;
  return BORN_OK;
}

}  // namespace

extern "C" {

int born_json_read_info(const char *path, born_sep_info *info) {
  if (!path || !info) return BORN_EINVAL;
  return read_json_info(path, info, nullptr);
}

int born_regfile_read_info(const char *path, born_sep_info *info) {
  if (!path || !info) return BORN_EINVAL;
  return read_any_info(path, info, nullptr);
}

int born_regfile_read(const char *path, float *out, long long count) {
  if (!path || !out || count < 0) return BORN_EINVAL;
  born_sep_info info;
  std::string data;
  int rc = read_any_info(path, &info, &data);
  if (rc) return rc;
  if (count != total_of(info)) return BORN_EINVAL;
  std::FILE *f = std::fopen(data.c_str(), "rb");
  if (!f) return BORN_EINVAL;
  const size_t got = std::fread(out, 4, (size_t)count, f);
  std::fclose(f);
  if ((long long)got != count) return BORN_EINVAL;
  if (info.big_endian == (little_endian_host() ? 1 : 0)) swap4(out, count);
  return BORN_OK;
}

int born_regfile_write(const char *path, const born_sep_info *info,
                       const float *data) {
  if (!path || !info || !data || info->ndim < 1 || info->ndim > 6)
    return BORN_EINVAL;
  bool swap = false;
  std::string bin;
  int rc = write_description(path, info, &swap, &bin);
  if (rc) return rc;
  std::FILE *df = std::fopen(bin.c_str(), "wb");
  if (!df) return BORN_EINVAL;
  const bool ok = write_floats(df, data, total_of(*info), swap);
  std::fclose(df);
  return ok ? BORN_OK : BORN_EINVAL;
}

// util/Add (util/Add.cc:5-41): out = in1 + in2, both of the same size
// (the reference asserts sameSize), streamed in blocks of 2^26 floats; out
// takes in1's axes and is SEP or JSON by its name.
int born_add_regfiles(const char *in1, const char *in2, const char *out) {
  if (!in1 || !in2 || !out) return BORN_EINVAL;
  born_sep_info a, b;
  std::string da, db;
  int rc = read_any_info(in1, &a, &da);
  if (!rc) rc = read_any_info(in2, &b, &db);
  if (rc) return rc;
  for (int k = 0; k < 6; ++k)
    if (a.n[k] != b.n[k]) return BORN_EINVAL;
  bool swap_out = false;
  std::string dout;
  born_sep_info o = a;
  if (o.ndim < 1) o.ndim = 1;
  // read both inputs before creating the output (out may be in1 or in2)
  const long long total = total_of(a);
  const long long block = 1LL << 26;
  std::FILE *fa = std::fopen(da.c_str(), "rb");
  std::FILE *fb = std::fopen(db.c_str(), "rb");
  if (!fa || !fb) {
    if (fa) std::fclose(fa);
    if (fb) std::fclose(fb);
    return BORN_EINVAL;
  }
  const bool swap_a = a.big_endian == (little_endian_host() ? 1 : 0);
  const bool swap_b = b.big_endian == (little_endian_host() ? 1 : 0);
  std::vector<float> sum((size_t)total);
  std::vector<float> buf((size_t)std::min(block, total > 0 ? total : 1));
  long long done = 0;
  bool ok = true;
  while (ok && done < total) {
    const long long m = std::min(block, total - done);
    ok = std::fread(sum.data() + done, 4, (size_t)m, fa) == (size_t)m &&
         std::fread(buf.data(), 4, (size_t)m, fb) == (size_t)m;
    if (!ok) break;
    if (swap_a) swap4(sum.data() + done, m);
    if (swap_b) swap4(buf.data(), m);
    for (long long i = 0; i < m; ++i) sum[(size_t)(done + i)] += buf[(size_t)i];
    done += m;
  }
  std::fclose(fa);
  std::fclose(fb);
  if (!ok) return BORN_EINVAL;
  rc = write_description(out, &o, &swap_out, &dout);
  if (rc) return rc;
  std::FILE *fo = std::fopen(dout.c_str(), "wb");
  if (!fo) return BORN_EINVAL;
  ok = write_floats(fo, sum.data(), total, swap_out);
  std::fclose(fo);
  return ok ? BORN_OK : BORN_EINVAL;
}

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
