"""bench.py's roofline inputs on CPU: the committed ncu traffic figure, the
algorithmic bytes per cell-update of each step, and the peak lookup with its
fallback (the JSON line's denominators)."""
import importlib.util
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location(
        "bench_helpers_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes_per_cell(bench):
    # compulsory FP32 traffic per interior cell-update: source 3 reads + 1
    # write, forward 6 + 2 (velocity shared), adjoint 7 + 3 (image RMW)
    assert bench.BYTES_PER_CELL == {"source": 16, "forward": 32, "adjoint": 40}


def test_traffic_figure_from_committed_profile(bench):
    tpc = bench.traffic_per_cell("adjoint_step")
    assert tpc is not None
    # ncu's DRAM bytes per cell sit at or just above the compulsory 40
    assert 40.0 <= tpc <= 44.0
    assert bench.traffic_per_cell("no_such_kernel") is None


def test_peak_lookup_and_fallback(bench, tmp_path, monkeypatch):
    peak, kind = bench.measured_peak()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        assert kind == "measured" and peak == float(d["hbm_gbs"])
    else:
        assert kind == "fallback"
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peak() == (bench.FALLBACK_HBM_GBS, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 1234.5}))
    assert bench.measured_peak() == (1234.5, "measured")
    (tmp_path / "MEASURED_PEAKS.json").write_text("not json")
    assert bench.measured_peak() == (bench.FALLBACK_HBM_GBS, "fallback")


def test_aggregate_rate_counts_all_ranks(bench):
    # 2 ranks, 3 steps of 1e9 cell-updates each in 1.5 s: 4 G cell-updates/s
    assert bench.aggregate_rate(1e9, 3, 1500.0, 2) == pytest.approx(4.0, rel=1e-3)


def test_reference_arm_inputs_equal_gpu_arm_inputs(bench, born, po):
    """The reference arm builds the shot from the oracle's geometry (so it
    loads no product library); the arrays equal those the GPU arm builds
    with the product's host geometry, bit for bit (reduced c2 model)."""
    import numpy as np
    wl = bench.workload_module()
    a = wl.prepare_shot(born, "c2", nt=30, n=48)
    b = wl.prepare_shot(po.Geometry(), "c2", nt=30, n=48)
    for k, v in a.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(v, b[k]), k
        else:
            assert v == b[k], k
    # both arms print the same config object
    assert bench.arm_config(a, "f32", 1) == bench.arm_config(b, "f32", 1)
