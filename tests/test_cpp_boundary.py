"""The C++ drop-in class (csrc/gb300_prop.h, gb300PropT<Base>) compiles
against the library, and on the GPU reproduces the reference fixtures when
driven from C++ in the reference operator's call order."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_oracle_golden import GOLDEN_FILES, load_golden

CSRC = os.path.join(ROOT, "sc17-born_gb300", "csrc")
DRIVER = os.path.join(ROOT, "tests", "cpp", "drive_prop.cc")


def build_driver(born, tmp_path):
    lib_dir = os.path.dirname(born.LIB_PATH)
    exe = str(tmp_path / "drive_prop")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-Wextra",
                    "-I", CSRC, DRIVER, "-o", exe, "-L", lib_dir,
                    "-lborn_gb300", f"-Wl,-rpath,{lib_dir}"], check=True)
    return exe


def test_cpp_drop_in_compiles_and_links(born, tmp_path):
    exe = build_driver(born, tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN_FILES[:2], ids=os.path.basename)
def test_cpp_drop_in_matches_reference_fixture(born, tmp_path, path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    exe = build_driver(born, tmp_path)
    case, out = load_golden(path)
    nz, ny, nx = case["shape"]
    d = tmp_path
    with open(d / "params.txt", "w") as f:
        f.write(f"{nx} {ny} {nz} {case['d']} {case['nt']} {case['jts']} "
                f"{case['nt_big']} {case['rec_nx']} {case['rec_ny']}\n")
    for k, dt in (("table_s", np.float32), ("locs_s", np.int32),
                  ("src", np.float32), ("vel1", np.float32),
                  ("vel2", np.float32), ("locs_r", np.int32),
                  ("rec_in", np.float32), ("refl", np.float32)):
        name = "table" if k == "table_s" else k
        ext = "i32" if dt == np.int32 else "f32"
        np.ascontiguousarray(case[k], dt).tofile(d / f"{name}.{ext}")
    subprocess.run([exe, str(d)], check=True)
    for k in ("src_p0", "src_p1", "image"):
        got = np.fromfile(d / f"{k}.f32", np.float32).reshape(case["shape"])
        assert np.array_equal(got, out[k]), k
    tr = np.fromfile(d / "traces.f32", np.float32).reshape(out["traces"].shape)
    err = np.linalg.norm(tr - out["traces"]) / np.linalg.norm(out["traces"])
    assert err <= 1e-5, err
