"""The Born operator behind the reference's solver classes.

csrc/born_my_operator.h wraps the operator in a my_operator subclass and
its vectors in a my_vector subclass (base/my_operator.h:18-25,
base/my_vector.h:7-91), so that the reference's least-squares loop,
lin_solver's simple_solver with cgstep (base/lin_solver.cc:6-16,104-132,
base/cgstep.cc:11-54), drives the GPU operator unchanged.

* CPU: the restatement of lin_solver/cgstep in oracle/solver (used where the
  reference's sources are absent, e.g. on the GPU machine) prints the same
  residuals, model and dot-product test as the reference's own classes,
  bit for bit (oracle/_ref/pin_solver_ref, built from the reference's
  sources by oracle/Makefile).
* CPU: the adapter under the reference's own classes, over a host stand-in
  of the library's C ABI (oracle/_ref/drive_solver_ref_fake), gives the
  same residuals and model as under the restatement; the adapter also
  compiles and links against the real library.
* GPU: the reference's loop (restated) on the adapter and the library's own
  born_cg_solve on the same exact-mode operator give the same rr.rr per
  iteration (relative 1e-6; the arithmetic is the same, so they agree to
  the last bit in practice) and the same model; the dot-product test of
  my_operator passes.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "sc17-born_gb300", "csrc")
INC = os.path.join(ROOT, "include")
SOLVER = os.path.join(ROOT, "oracle", "solver")
TCPP = os.path.join(ROOT, "tests", "cpp")
FLAGS = ["g++", "-std=c++14", "-O2", "-fno-fast-math", "-ffp-contract=off",
         "-Wall", "-Wextra"]
SOLVER_SRC = [os.path.join(SOLVER, f) for f in
              ("my_operator.cc", "cgstep.cc", "lin_solver.cc")]


def build_restated(tmp_path, name, sources, libborn=None):
    exe = str(tmp_path / name)
    cmd = FLAGS + ["-I", SOLVER, "-I", INC, "-I", CSRC] + sources + \
        SOLVER_SRC + ["-o", exe]
    if libborn:
        lib_dir = os.path.dirname(libborn)
        cmd += ["-L", lib_dir, "-lborn_gb300", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True)
    return exe


def write_problem(d, kw, m_true):
    vel = kw["velocity"]
    n3, n2, n1 = vel.shape
    with open(d / "params.txt", "w") as f:
        f.write(" ".join(str(v) for v in (
            n1, n2, n3, *kw["o"], *kw["d"], kw["nt_data"], kw["dt_data"],
            kw["rec_n"][0], kw["rec_n"][1], kw["rec_o"][0], kw["rec_d"][0],
            kw["rec_o"][1], kw["rec_d"][1], kw["rec_depth"],
            len(kw["shots"]), kw["wavelet"].size, kw["dt_wavelet"],
            kw["nbound"], 1, kw.get("ckpt_interval", 50))) + "\n")
    np.ascontiguousarray(vel, np.float32).tofile(d / "velocity.f32")
    np.ascontiguousarray(kw["shots"], np.float32).tofile(d / "shots.f32")
    np.ascontiguousarray(kw["wavelet"], np.float32).tofile(d / "wavelet.f32")
    np.ascontiguousarray(m_true, np.float32).tofile(d / "m_true.f32")


def parse(out):
    res = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] in ("solver", "cg"):
            res.setdefault(parts[0], []).append(float(parts[2]))
        elif len(parts) == 2 and parts[0] == "dot_test":
            res["dot_test"] = int(parts[1])
    return res


GOLDEN = os.path.join(ROOT, "tests", "golden", "solver_ref.npz")


def fake_problem():
    """The small problem the adapter runs on over the host stand-in."""
    from test_operator import setup_problem
    kw = setup_problem(seed=3, n=(6, 7, 8), nt_data=12, nshots=1)
    m_true = np.zeros(kw["velocity"].shape, np.float32)
    m_true.ravel()[::5] = 1.0
    return kw, m_true


def test_restated_solver_matches_reference_solver(po, tmp_path):
    """Against the reference classes' output stored by
    tests/golden/make_golden.py, and against the live build where the
    reference's sources are present."""
    mine = build_restated(tmp_path, "pin_solver",
                          [os.path.join(TCPP, "pin_solver.cc")])
    b = subprocess.run([mine, "10"], capture_output=True, text=True,
                       check=True).stdout
    want = str(np.load(GOLDEN)["pin_stdout"])
    assert "rr10 " in want and "dot_test 1" in want
    assert b == want
    ref = po.ref_program("pin_solver_ref")
    if ref is not None:
        a = subprocess.run([ref, "10"], capture_output=True, text=True,
                           check=True).stdout
        assert a == b


def test_adapter_under_reference_solver_cpu(po, tmp_path):
    """The adapter over the host stand-in: under the restated classes it
    prints what it printed under the reference's own (stored fixture, and
    the live build where the reference's sources are present)."""
    mine = build_restated(tmp_path, "drive_solver_fake",
                          [os.path.join(TCPP, "drive_solver.cc"),
                           os.path.join(TCPP, "fake_born.cc")])
    kw, m_true = fake_problem()
    g = np.load(GOLDEN)
    outs = [(parse(str(g["adapter_stdout"])), g["adapter_model"])]
    exes = [mine]
    ref = po.ref_program("drive_solver_ref_fake")
    if ref is not None:
        exes.append(ref)
    for exe in exes:
        d = tmp_path / ("run_" + os.path.basename(exe))
        d.mkdir()
        write_problem(d, kw, m_true)
        r = subprocess.run([exe, str(d), "6", "1"], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append((parse(r.stdout),
                     np.fromfile(d / "model_solver.f32", np.float32)))
    a, ma = outs[0]
    assert len(a["solver"]) == 7 and a["solver"][-1] < a["solver"][0]
    assert a["dot_test"] == 1
    for b, mb in outs[1:]:
        assert a == b
        assert np.array_equal(ma, mb)


def test_adapter_compiles_and_links_against_library(born, tmp_path):
    exe = build_restated(tmp_path, "drive_solver",
                         [os.path.join(TCPP, "drive_solver.cc")],
                         libborn=born.LIB_PATH)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_adapter_under_solver_matches_cg_solve(born, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from test_operator import setup_problem
    kw = setup_problem(seed=9, nshots=2, nt_data=50)
    kw["ckpt_interval"] = 16
    rng = np.random.default_rng(1002)
    m_true = np.zeros(kw["velocity"].shape, np.float32)
    m_true[10:12] = rng.choice([-1.0, 1.0], size=m_true[10:12].shape) * 1e-3
    exe = build_restated(tmp_path, "drive_solver",
                         [os.path.join(TCPP, "drive_solver.cc")],
                         libborn=born.LIB_PATH)
    write_problem(tmp_path, kw, m_true)
    niter = 5
    r = subprocess.run([exe, str(tmp_path), str(niter)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = parse(r.stdout)
    s, c = res["solver"], res["cg"]
    assert len(s) == len(c) == niter + 1
    for k in range(niter + 1):
        assert abs(s[k] - c[k]) <= 1e-6 * c[k], (k, s[k], c[k])
    assert all(s[k + 1] < s[k] for k in range(niter)), s
    ms = np.fromfile(tmp_path / "model_solver.f32", np.float32)
    mc = np.fromfile(tmp_path / "model_cg.f32", np.float32)
    assert np.linalg.norm(ms - mc) <= 1e-6 * np.linalg.norm(mc)
    assert res["dot_test"] == 1
