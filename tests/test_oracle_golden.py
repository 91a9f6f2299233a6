"""The oracle (C restatement of base/cpu_prop.cc) against the golden
fixtures made by running the reference's own compiled CPU path, and directly
against that compiled path where the reference sources are present."""
import glob
import os

import numpy as np
import pytest

import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(path):
    z = np.load(path)
    case = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    for k in z.files:
        if k.startswith("par_"):
            v = z[k]
            case[k[4:]] = tuple(int(x) for x in v) if v.ndim else v.item()
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return case, out


GOLDEN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "g*_*.npz")))


def test_golden_files_present():
    assert len(GOLDEN_FILES) >= 3


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=os.path.basename)
def test_port_matches_reference_fixture(po, path):
    case, out = load_golden(path)
    got = po.run_case(po.PortProp(), case)
    for k, v in out.items():
        assert np.array_equal(got[k], v), f"{k} differs from the reference"


def test_sinc_tables_match_reference_fixture(po):
    z = np.load(os.path.join(GOLDEN, "sinc_tables.npz"))
    for k in z.files:
        n = int(k.split("_")[1])
        assert np.array_equal(po.sinc_table(n), z[k]), k
    # known answer (sinc_bob(4, 8).table[1])
    ka = [-0.00954874, 0.0413194, -0.134028, 0.878098, 0.293563, -0.0965802,
          0.0343447, -0.00847994]
    np.testing.assert_allclose(z["sinc_4"][1], ka, rtol=2e-5, atol=1e-7)


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=os.path.basename)
def test_fp64_oracle_close_to_reference(po, path):
    case, out = load_golden(path)
    got = po.run_case(po.PortProp64(), case)
    for k, v in out.items():
        ref = got[k]
        err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err < 1e-4, (k, err)


def test_port_against_compiled_reference_random_cases(po):
    if po.ref_lib() is None:
        pytest.skip("reference sources not present")
    for seed, nt, jt, dup in ((21, 25, 1, 0), (22, 33, 3, 1), (23, 1, 1, 0),
                              (24, 2, 2, 0)):
        c = cases.make_case(seed, shape=(18, 20, 24), nt=nt, jt=jt,
                            dup_receivers=dup, sinc=po.sinc_table)
        a = po.run_case(po.RefProp(), c)
        b = po.run_case(po.PortProp(), c)
        for k in a:
            assert np.array_equal(a[k], b[k]), (seed, k)


def test_primitives_against_compiled_reference(po):
    if po.ref_lib() is None:
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(5)
    shape = (20, 22, 24)
    r, p = po.RefProp(), po.PortProp()
    for prop in (r, p):
        prop.createSpace(10.0, 10.0, 10.0, 50, .0005, .0005, shape[2],
                         shape[1], shape[0])
    p1 = rng.standard_normal(shape).astype(np.float32)
    vel = (rng.uniform(0.05, 0.15, shape)).astype(np.float32)
    outs = []
    for prop in (r, p):
        a = rng.standard_normal(shape).astype(np.float32) * 0
        a[...] = p1[::-1]
        b = p1.copy()
        prop.prop(a, b, vel)
        prop.damp(a, b)
        outs.append((a, b))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_geometry_matches_reference_fixture(po):
    """Source points and wavelet derivative, receiver cells, compute-grid
    sizes, the random boundary, the FD step and the linear glue (laplac,
    deriv, map_data) of the oracle against the outputs of the reference's
    own code on the same seeded inputs (tests/golden/geometry.npz)."""
    import geometry_cases as gc
    z = np.load(os.path.join(GOLDEN, "geometry.npz"))
    got = gc.run(gc.make_inputs(int(z["seed"])), po, ref=False)
    names = [k for k in z.files if k != "seed"]
    assert sorted(names) == sorted(got)
    for k in names:
        assert got[k].shape == z[k].shape, k
        assert np.array_equal(got[k], z[k]), f"{k} differs from the reference"


def test_geometry_against_compiled_reference_random_cases(po):
    if po.ref_geom_lib() is None:
        pytest.skip("reference sources not present")
    import geometry_cases as gc
    for seed in (1, 2):
        inp = gc.make_inputs(seed)
        a = gc.run(inp, po, ref=True)
        b = gc.run(inp, po, ref=False)
        for k in a:
            assert np.array_equal(a[k], b[k]), (seed, k)
