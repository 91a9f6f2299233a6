"""The oracle (C restatement of base/cpu_prop.cc) against the golden
fixtures made by running the reference's own compiled CPU path, and directly
against that compiled path where the reference sources are present."""
import ctypes as C
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


def test_port_against_compiled_reference_random_shapes(po):
    """Random grid shapes (odd sizes included), sinc ratios jt 1-4 and step
    counts, with and without duplicated receivers."""
    if po.ref_lib() is None:
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(77)
    for k in range(6):
        shape = tuple(int(x) for x in rng.integers(14, 27, 3))
        jt = int(rng.integers(1, 5))
        nt = int(rng.integers(2, 30))
        c = cases.make_case(100 + k, shape=shape, nt=nt, jt=jt,
                            dup_receivers=int(k % 2), sinc=po.sinc_table)
        a = po.run_case(po.RefProp(), c)
        b = po.run_case(po.PortProp(), c)
        for key in a:
            assert np.array_equal(a[key], b[key]), (shape, jt, nt, key)


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


def test_geometry_random_axes_against_compiled_reference(po):
    """Random axes, positions and sizes (not only random data): windows,
    source points, receiver cells, random boundaries, FD step and compute
    sizes of the oracle against the reference's own code."""
    if po.ref_geom_lib() is None:
        pytest.skip("reference sources not present")
    R, L = po.ref_geom_lib(), po.port_lib()
    f, i = po.fptr, po.iptr
    f32 = np.float32
    rng = np.random.default_rng(2024)
    # image windows
    for _ in range(25):
        wn = tuple(int(x) for x in rng.integers(5, 15, 3))
        wo = tuple(float(f32(x)) for x in rng.uniform(-50, 50, 3))
        wd = tuple(float(f32(x)) for x in rng.uniform(3, 15, 3))
        sn = tuple(int(x) for x in rng.integers(3, 17, 3))
        so = tuple(float(f32(f32(o) + f32(k) * f32(d)))
                   for o, k, d in zip(wo, rng.uniform(-8, 8, 3), wd))
        whole = rng.standard_normal(wn[::-1]).astype(np.float32)
        sub = rng.standard_normal(sn[::-1]).astype(np.float32)
        off = [L.oracle_window_offset(so[a], wo[a], wd[a]) for a in range(3)]
        a, b = np.zeros(sn[::-1], np.float32), np.zeros(sn[::-1], np.float32)
        R.ref_geom_image_window(1, f(whole.copy()), *wn, *wo, *wd, f(a), *sn,
                                *so, *wd)
        L.oracle_extract_sub(f(whole), *wn, f(b), *sn, *off)
        assert np.array_equal(a, b), (wn, wo, wd, sn, so)
        wa, wb = whole.copy(), whole.copy()
        R.ref_geom_image_window(0, f(wa), *wn, *wo, *wd, f(sub.copy()), *sn,
                                *so, *wd)
        L.oracle_add_image(f(wb), *wn, f(sub), *sn, *off)
        assert np.array_equal(wa, wb), (wn, wo, wd, sn, so)
    # source points and wavelet derivative on random grids
    raw = rng.standard_normal(64).astype(np.float32)
    for _ in range(12):
        n = tuple(int(x) for x in rng.integers(24, 48, 3))
        o = tuple(float(f32(x)) for x in rng.uniform(-200, 0, 3))
        d = tuple(float(f32(x)) for x in rng.uniform(5, 12, 3))
        pos = [float(f32(o[k] + rng.uniform(3, n[k] - 3) * d[k]))
               for k in range(3)]
        dt = float(f32(rng.uniform(5e-4, 2e-3)))
        nts = 70
        wd_ = np.zeros_like(raw)
        L.oracle_wavelet_deriv(f(raw), raw.size, dt, f(wd_))
        lr, lo = np.zeros(9, np.int32), np.zeros(9, np.int32)
        vr = np.zeros(9 * nts, np.float32)
        vo = np.zeros(9 * nts, np.float32)
        R.ref_geom_source(f(raw), raw.size, dt, *pos, *o, *d, *n, nts, i(lr),
                          f(vr))
        L.oracle_source_geometry(*pos, *o, *d, n[0], n[1], f(wd_), raw.size,
                                 nts, i(lo), f(vo))
        assert np.array_equal(lr, lo) and np.array_equal(vr, vo), (n, o, d)
    # receiver cells
    for _ in range(12):
        n = tuple(int(x) for x in rng.integers(40, 64, 3))
        o = tuple(float(f32(x)) for x in rng.uniform(-100, 0, 3))
        d = tuple(float(f32(x)) for x in rng.uniform(5, 12, 3))
        rnx, rny = (int(x) for x in rng.integers(2, 12, 2))
        rx0, ry0 = (float(f32(o[k] + rng.uniform(1, 5) * d[k]))
                    for k in range(2))
        rdx, rdy = (float(f32(x)) for x in rng.uniform(1, 3, 2) * d[0])
        rz = float(f32(o[2] + rng.uniform(2, 10) * d[2]))
        lr = np.zeros(rnx * rny, np.int32)
        lo = np.zeros_like(lr)
        R.ref_geom_receivers(rnx, rny, rx0, rdx, ry0, rdy, rz, *o, *d, *n, 40,
                             i(lr))
        L.oracle_receiver_geometry(rnx, rny, rx0, rdx, ry0, rdy, rz, *o, *d,
                                   n[0], n[1], i(lo))
        assert np.array_equal(lr, lo), (n, o, d, rnx, rny)
    # random boundary on random compute grids
    vel = (1500 + 2500 * rng.random((20, 22, 24))).astype(np.float32)
    for _ in range(6):
        n = tuple(int(x) for x in rng.integers(24, 36, 3))
        o = tuple(float(f32(x)) for x in rng.uniform(-80, 0, 3))
        d = (10.0, 10.0, 10.0)
        nr = int(rng.integers(0, 9))
        irand = int(rng.integers(0, 10000))
        a = np.zeros(n[::-1], np.float32)
        b = np.zeros_like(a)
        va = (24, 22, 20, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0)
        R.ref_geom_rand_subspace(f(vel), *va, irand, nr, nr, nr, 0.001, *n,
                                 *o, *d, f(a))
        L.oracle_rand_subspace(f(vel), *va, float(vel.max()), irand, nr, nr,
                               nr, 0.001, *n, *o, *d, f(b))
        assert np.array_equal(a, b), (n, o, nr, irand)
    # FD step and compute sizes
    for _ in range(20):
        vmax = float(f32(rng.uniform(1500, 6000)))
        dv = float(f32(rng.uniform(2, 20)))
        dtd = float(f32(rng.choice([5e-4, 1e-3, 2e-3, 4e-3])))
        ntd = int(rng.integers(100, 3000))
        v = np.full((6, 5, 4), 1500.0, np.float32)
        v[2, 2, 2] = vmax
        dt_r, nt_r = np.zeros(1, np.float32), np.zeros(1, np.int32)
        R.ref_geom_calc_stability(f(v), 4, 5, 6, dv, dv, dv, dtd, ntd,
                                  f(dt_r), i(nt_r))
        nt_o = C.c_int()
        dt_o = L.oracle_calc_stability(vmax, dv, dtd, ntd, C.byref(nt_o))
        assert np.float32(dt_o) == dt_r[0] and nt_o.value == nt_r[0], (
            vmax, dv, dtd, ntd)
        nm, nb, fat = (int(x) for x in (rng.integers(9, 700),
                                        rng.integers(0, 80),
                                        rng.integers(0, 6)))
        assert R.ref_geom_compute_size(nm, nb, fat) == \
            L.oracle_compute_size(nm, nb, fat)
