"""The RTM3D driver (sc17-born_gb300/cli.py rtm, rtm.cc:10-41) on files: a
5-axis data file (t, rx, ry, sx, sy), a wavelet and a velocity in SEP and
JSON form give the image of BornOperator.adjoint over the same shots bit
for bit, and migrating the shots in two round-robin halves (two ranks of
the shot farm) and summing the halves gives the same image to rounding."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cli_rtm_matches_operator(born, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    spec = importlib.util.spec_from_file_location(
        "born_gb300_cli", os.path.join(ROOT, "sc17-born_gb300", "cli.py"))
    cli = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cli)
    rng = np.random.default_rng(31)
    n3, n2, n1, d = 20, 22, 24, 10.0
    z = np.arange(n3)[:, None, None]
    vel = (2000.0 + 40.0 * z + 100 * rng.random((n3, n2, n1))).astype(
        np.float32)
    t = -0.02 + np.arange(80) * 0.001
    a = (np.pi * 25.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    nt, rnx, rny, nsx, nsy = 60, 12, 11, 3, 1
    data = (1e-3 * rng.standard_normal((nsy, nsx, rny, rnx, nt))).astype(
        np.float32)
    born.write_regfile(str(tmp_path / "velocity.json"), vel, o=(0, 0, 0),
                       d=(d, d, d))
    born.write_regfile(str(tmp_path / "wavelet.H"), wav, o=(0,), d=(0.001,))
    born.write_regfile(str(tmp_path / "data.json"), data,
                       o=(0.0, 10.0, 10.0, 100.0, 110.0),
                       d=(0.001, 20.0, 20.0, 10.0, 10.0))
    pars = dict(data=str(tmp_path / "data.json"),
                wavelet=str(tmp_path / "wavelet.H"),
                velocity=str(tmp_path / "velocity.json"),
                image=str(tmp_path / "image.json"), src_depth="20",
                rec_depth="10", nbound="6")
    assert cli.cmd_rtm(pars) == 0
    got, o, dd = born.read_regfile(str(tmp_path / "image.json"))
    assert got.shape == vel.shape and dd == pytest.approx((d, d, d))
    shots = np.array([[100.0 + 10.0 * k, 110.0, 20.0] for k in range(nsx)],
                     np.float32)
    op = born.BornOperator(vel, (0., 0., 0.), (d, d, d), shots, wav, 0.001,
                           nt, 0.001, (rnx, rny), (10.0, 10.0), (20.0, 20.0),
                           10.0, 6)
    want = torch.zeros(vel.shape, device="cuda")
    op.adjoint(False, want,
               torch.from_numpy(data.reshape(nsx, rny, rnx, nt)).cuda())
    assert np.linalg.norm(got) > 0
    assert np.array_equal(got, want.cpu().numpy())
    # rank 0 migrates shots 0 and 2, rank 1 shot 1: the same images summed
    # in another order (float addition), so equal to rounding
    halves = [cli.migrate(pars, r, 2)[0] for r in range(2)]
    s = halves[0] + halves[1]
    assert np.linalg.norm(s - got) <= 1e-6 * np.linalg.norm(got)
