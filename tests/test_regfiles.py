"""Regular files and the command-line drivers on CPU: JSON regular files
(the form scripts/run.py:20-36 writes) next to SEP ones, util/Add
(util/Add.cc) for either kind and in place, the json=<file> parameter
convention (scripts/run.py:66-77), and the round-robin shot split of the
shot farm (scripts/split.py:12-27)."""
import importlib.util
import json
import os

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def cli(born):
    spec = importlib.util.spec_from_file_location(
        "born_gb300_cli", os.path.join(ROOT, "sc17-born_gb300", "cli.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_json_round_trip(born, tmp_path):
    a = np.random.default_rng(1).standard_normal((5, 6, 7)).astype(np.float32)
    p = str(tmp_path / "img.json")
    born.write_regfile(p, a, o=(1.5, -2.0, 0.0), d=(10.0, 12.5, 8.0))
    desc = json.load(open(p))
    assert desc["n1"] == 7 and desc["n2"] == 6 and desc["n3"] == 5
    assert desc["filename"] == "img.json.dat"
    b, o, d = born.read_regfile(p)
    assert np.array_equal(a, b)
    assert o == pytest.approx((1.5, -2.0, 0.0)) and d == pytest.approx(
        (10.0, 12.5, 8.0))


def test_json_file_in_the_run_script_form(born, tmp_path):
    """A description as scripts/run.py writes it (labels, its 'i1' key,
    the data file named by 'filename') reads as a 1 x 1 x 1 cube."""
    params = {"d1": 1, "d2": 1, "d3": 1, "n1": 1, "n2": 1, "n3": 1, "i1": 1,
              "o2": 1, "o3": 1, "label1": "Undefined", "label2": "Undefined",
              "label3": "Undefined", "filename": "image.7.json.dat"}
    with open(tmp_path / "image.7.json", "w") as f:
        json.dump(params, f, indent=4)
    np.array([3.25], np.float32).tofile(tmp_path / "image.7.json.dat")
    a, o, d = born.read_regfile(str(tmp_path / "image.7.json"))
    assert a.shape == (1, 1, 1) and a.ravel()[0] == np.float32(3.25)
    assert o == pytest.approx((0.0, 1.0, 1.0))


def test_sep_and_json_add(born, tmp_path):
    rng = np.random.default_rng(2)
    a = rng.standard_normal((4, 5, 6)).astype(np.float32)
    b = rng.standard_normal((4, 5, 6)).astype(np.float32)
    born.write_regfile(str(tmp_path / "a.H"), a, d=(10.0, 10.0, 10.0))
    born.write_regfile(str(tmp_path / "b.json"), b)
    born.add_regfiles(str(tmp_path / "a.H"), str(tmp_path / "b.json"),
                      str(tmp_path / "c.json"))
    c, o, d = born.read_regfile(str(tmp_path / "c.json"))
    assert np.array_equal(c, a + b)
    assert d == pytest.approx((10.0, 10.0, 10.0))  # in1's axes
    # in place, as the shot farm accumulates its final image
    born.add_regfiles(str(tmp_path / "a.H"), str(tmp_path / "c.json"),
                      str(tmp_path / "c.json"))
    c2, _, _ = born.read_regfile(str(tmp_path / "c.json"))
    assert np.array_equal(c2, a + (a + b))
    # SEP output is big-endian xdr data beside the header
    born.add_regfiles(str(tmp_path / "b.json"), str(tmp_path / "a.H"),
                      str(tmp_path / "s.H"))
    raw = np.fromfile(tmp_path / "s.H@", ">f4").reshape(a.shape)
    assert np.array_equal(raw, b + a)
    # different sizes are refused, as the reference asserts sameSize
    born.write_regfile(str(tmp_path / "x.H"), np.zeros((4, 5, 7), np.float32))
    with pytest.raises(born.BornError):
        born.add_regfiles(str(tmp_path / "a.H"), str(tmp_path / "x.H"),
                          str(tmp_path / "y.H"))


def test_cli_add_with_json_parameters(born, cli, tmp_path):
    a = np.arange(24, dtype=np.float32).reshape(2, 3, 4)
    born.write_regfile(str(tmp_path / "image.1.json"), a)
    born.write_regfile(str(tmp_path / "final.image.json"), 2 * a)
    with open(tmp_path / "add.P", "w") as f:
        json.dump({"out": str(tmp_path / "final.image.json"),
                   "in1": str(tmp_path / "image.1.json"),
                   "in2": str(tmp_path / "final.image.json")}, f, indent=4)
    assert cli.main(["add", f"json={tmp_path / 'add.P'}"]) == 0
    c, _, _ = born.read_regfile(str(tmp_path / "final.image.json"))
    assert np.array_equal(c, 3 * a)
    # later key=value arguments override the JSON's
    pars = cli.parse_params([f"json={tmp_path / 'add.P'}", "out=z.H"])
    assert pars["out"] == "z.H" and pars["in1"].endswith("image.1.json")


def test_shot_split_round_robin(cli):
    assert cli.shots_of_rank(7, 0, 3) == [0, 3, 6]
    assert cli.shots_of_rank(7, 2, 3) == [2, 5]
    got = sorted(s for r in range(4) for s in cli.shots_of_rank(10, r, 4))
    assert got == list(range(10))
