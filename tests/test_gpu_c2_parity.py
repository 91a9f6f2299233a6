"""Parity at the benchmark's own case.

bench.py times the c2 shot: a 256^3 model at 10 m with a 50-cell boundary
(368^3 compute grid), 128 x 128 receivers, 12 Hz Ricker, a layered velocity
with a dipping interface and a Gaussian salt blob.  Here the same shot,
truncated to nt = 150 FD steps so that the oracle finishes in well under a
minute on the host cores, runs through Gb300Prop and through the oracle
port in rtm_zero_op's call order (sourceProp, rtmAdjoint, then rtmForward;
cpu_prop.cc:22-129):

* the shot's inputs made by the product's host geometry equal those made by
  the oracle's restatement (sinc table, source and receiver cells, source
  traces, random-boundary and plain v^2 dt^2 models, reflectivity);
* source levels and image are bit-identical, Born traces within 1e-5
  relative L2 under FP32 storage (the reference forms the 1e-6 Born
  coupling in double, that storage in float) and bit-identical under the
  exact-coupling storage (the same shot again, "f32exact").
"""
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NT = 150


def workload():
    spec = importlib.util.spec_from_file_location(
        "born_gb300_workload",
        os.path.join(ROOT, "sc17-born_gb300", "workload.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) /
                 max(np.linalg.norm(b.ravel()), 1e-30))


def test_c2_shot_matches_oracle(born, po):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    wl = workload()
    case = wl.prepare_shot(born, "c2", nt=NT)
    assert case["shape"] == (368, 368, 368) and case["nt"] == NT
    assert case["rec_nx"] == case["rec_ny"] == 128
    ref_case = wl.prepare_shot(po.Geometry(), "c2", nt=NT)
    for k in ("table_s", "locs_s", "src", "vel1", "vel2", "locs_r", "rec_in",
              "refl"):
        assert np.array_equal(case[k], ref_case[k]), k

    po.set_threads(os.cpu_count() or 1)
    want = po.run_case(po.PortProp(), ref_case)
    got = po.run_case(born.Gb300Prop(0), case)
    for k in ("src_p0", "src_p1", "image"):
        assert np.array_equal(got[k], want[k]), (k, rel(got[k], want[k]))
    assert np.linalg.norm(want["image"]) > 0
    e = rel(got["traces"], want["traces"])
    assert np.linalg.norm(want["traces"]) > 0
    assert e <= 1e-5, e
    prop = born.Gb300Prop(0)
    nz, ny, nx = case["shape"]
    prop.createSpace(case["d"], case["d"], case["d"], 50, .0005, .0005, nx,
                     ny, nz)
    prop.set_storage("f32exact")
    got = po.run_case(prop, case)
    for k in ("src_p0", "src_p1", "image", "traces"):
        assert np.array_equal(got[k], want[k]), (k, rel(got[k], want[k]))
