// Least-squares RTM through the reference's solver classes: lin_solver's
// simple_solver with cgstep (base/lin_solver.cc:6-16,104-132,
// base/cgstep.cc:11-54) driving the Born operator through
// born_my_operatorT / born_device_vectorT (csrc/born_my_operator.h), against
// born_cg_solve on the same operator.  Built against the reference's solver
// sources where they are present, else against the restatement in
// oracle/solver; linked against libborn_gb300.so (or, for a CPU check of
// the adapter, a host stand-in of its C ABI).
//   drive_solver <dir> <niter> [skip_cg]
// <dir>/params.txt: n1 n2 n3 o1 o2 o3 d1 d2 d3 nt_data dt_data rec_nx rec_ny
//   rec_ox rec_dx rec_oy rec_dy rec_depth nshots nt_wavelet dt_wavelet nbound
//   exact ckpt_interval; velocity.f32, shots.f32, wavelet.f32, m_true.f32.
// Prints "solver <k> <rr.rr>" for k = 0..niter, "cg <k> <rr.rr>", and
// "dot_test <0|1>"; writes model_solver.f32 and model_cg.f32.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "born_my_operator.h"
#include "cgstep.h"
#include "lin_solver.h"
#include "my_operator.h"
#include "my_vector.h"

typedef born_my_operatorT<my_operator, my_vector> born_my_operator;

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
  if (argc < 3) return 2;
  const std::string dir = argv[1];
  const int niter = std::atoi(argv[2]);
  const bool skip_cg = argc > 3 && std::atoi(argv[3]) != 0;
  born_op_params p{};
  {
    std::ifstream f(dir + "/params.txt");
    f >> p.n1 >> p.n2 >> p.n3 >> p.o1 >> p.o2 >> p.o3 >> p.d1 >> p.d2 >>
        p.d3 >> p.nt_data >> p.dt_data >> p.rec_nx >> p.rec_ny >> p.rec_ox >>
        p.rec_dx >> p.rec_oy >> p.rec_dy >> p.rec_depth >> p.nshots >>
        p.nt_wavelet >> p.dt_wavelet >> p.nbound >> p.exact >>
        p.ckpt_interval;
    if (!f) return 2;
  }
  auto vel = load<float>(dir + "/velocity.f32");
  auto shots = load<float>(dir + "/shots.f32");
  auto wav = load<float>(dir + "/wavelet.f32");
  auto mtrue = load<float>(dir + "/m_true.f32");
  born_handle *h = nullptr;
  born_op *bop = nullptr;
  if (born_create(0, &h) != BORN_OK ||
      born_op_create(h, &p, vel.data(), shots.data(), wav.data(), &bop) !=
          BORN_OK) {
    std::fprintf(stderr, "operator set-up failed: %s\n",
                 h ? born_error_string(h) : "no device");
    return 3;
  }
  int rc = 0;
  try {
    auto op = std::make_shared<born_my_operator>(bop);
    auto mt = op->model_vector();
    mt->upload(mtrue.data());
    auto data = op->data_vector();
    if (!op->forward(false, mt, data)) throw std::runtime_error("forward");
    {
      cgstep cg;
      simple_solver solver(&cg, data, op);
      std::printf("solver 0 %.17g\n", solver.rr->dot(solver.rr));
      for (int it = 0; it < niter; ++it) {
        if (!solver.solve(1)) throw std::runtime_error("solver stopped");
        std::printf("solver %d %.17g\n", it + 1, solver.rr->dot(solver.rr));
      }
      std::vector<float> m((size_t)mt->size());
      born_device_vectorT<my_vector>::of(solver.m)->download(m.data());
      save(dir + "/model_solver.f32", m);
    }
    if (!skip_cg) {
      auto m0 = op->model_vector();
      std::vector<double> res((size_t)niter + 1, 0.0);
      if (born_cg_solve(bop, data->data(), m0->data(), niter, res.data()) !=
          BORN_OK)
        throw std::runtime_error("born_cg_solve");
      for (int k = 0; k <= niter; ++k)
        std::printf("cg %d %.17g\n", k, res[(size_t)k]);
      std::vector<float> m((size_t)m0->size());
      m0->download(m.data());
      save(dir + "/model_cg.f32", m);
    }
    srand(7);
    std::printf("dot_test %d\n", op->dot_test(false) ? 1 : 0);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    rc = 1;
  }
  born_op_destroy(bop);
  born_destroy(h);
  return rc;
}
