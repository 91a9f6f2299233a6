// Drives gb300PropT through the reference operator's call sequence
// (rtm_zero_op_3d.cc:249-282 adjoint, then :147-185 forward) from C++, on a
// case stored as raw files by tests/test_cpp_boundary.py:
//   params.txt : nx ny nz d nt jt nt_big rec_nx rec_ny
//   table.f32 locs_s.i32 src.f32 vel1.f32 vel2.f32 locs_r.i32 rec_in.f32
//   refl.f32
// Writes src_p0.f32 src_p1.f32 image.f32 traces.f32 into the same folder.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "gb300_prop.h"

struct NoBase {
  virtual ~NoBase() {}
};

template <class T>
static std::vector<T> load(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const size_t n = (size_t)f.tellg() / sizeof(T);
  std::vector<T> v(n);
  f.seekg(0);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(T));
  return v;
}

template <class T>
static void save(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  int nx, ny, nz, nt, jt, nt_big, rec_nx, rec_ny;
  float d;
  {
    std::ifstream p(dir + "/params.txt");
    p >> nx >> ny >> nz >> d >> nt >> jt >> nt_big >> rec_nx >> rec_ny;
  }
  auto flat = load<float>(dir + "/table.f32");
  std::vector<std::vector<float>> table(jt, std::vector<float>(8));
  for (int r = 0; r < jt; ++r)
    for (int c = 0; c < 8; ++c) table[r][c] = flat[r * 8 + c];
  auto locs_s = load<int>(dir + "/locs_s.i32");
  auto src = load<float>(dir + "/src.f32");
  auto vel1 = load<float>(dir + "/vel1.f32");
  auto vel2 = load<float>(dir + "/vel2.f32");
  auto locs_r = load<int>(dir + "/locs_r.i32");
  auto rec_in = load<float>(dir + "/rec_in.f32");
  auto refl = load<float>(dir + "/refl.f32");
  const size_t n123 = (size_t)nx * ny * nz;

  gb300PropT<NoBase> prop(0);
  prop.set_throw(true);
  try {
    prop.createSpace(d, d, d, 50.f, .0005f, .0005f, nx, ny, nz);
    prop.transferSincTableS(8, jt, table);
    prop.setNtblock(50);
    prop.transferSincTableD(8, jt, table);
    prop.transferSourceFunc((int)locs_s.size(), nt_big, locs_s, src.data());
    prop.transferVelFunc1(nx, ny, nz, vel1.data());
    prop.transferVelFunc2(nx, ny, nz, vel2.data());
    prop.transferReceiverFunc(rec_nx, rec_ny, nt_big, locs_r, rec_in.data());
    std::vector<float> p0(n123, 0.f), p1(n123, 0.f), img(n123, 0.f);
    prop.sourceProp(nx, ny, nz, false, true, p0.data(), p1.data(), jt, 9, nt);
    save(dir + "/src_p0.f32", p0);
    save(dir + "/src_p1.f32", p1);
    prop.rtmAdjoint(nx, ny, nz, jt, p1.data(), p0.data(), img.data(), 9, nt);
    save(dir + "/image.f32", img);
    std::vector<float> rec(rec_in.size(), 0.f);
    prop.transferReceiverFunc(rec_nx, rec_ny, nt_big, locs_r, rec.data());
    prop.rtmForward(nx, ny, nz, jt, refl.data(), rec.data(), 9, nt, nt_big,
                    rec_nx, rec_ny);
    save(dir + "/traces.f32", rec);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
