"""CPU-side checks of the product library: it loads, exports every symbol
the public headers declare, and its host geometry (the per-shot setup that
runs on the CPU) matches the oracle bit for bit.  No GPU compute here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", "born_gb300.h"),
           os.path.join(ROOT, "sc17-born_gb300", "csrc", "born_host.h")]


def declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    # return types of one or more words (long long, unsigned int, ...)
    names = re.findall(r"^\s*(?:const\s+)?(?:(?:unsigned|signed|long|short)"
                       r"\s+)*[a-z_]+(?:\s+|\s*\*+\s*)([a-z_0-9]+)\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(born):
    L = born.lib()
    names = []
    for h in HEADERS:
        names += declared_functions(h)
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the ctypes table covers the public header
    pub = set(declared_functions(HEADERS[0]))
    assert pub <= set(born.exported_symbols())


def test_no_device_gives_enodev_not_exit(born):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert born.lib().born_create(0, C.byref(h)) == -6
    # the reference-compatible entry points record instead of exiting
    born.lib().setup_cuda(1)
    assert born.lib().born_default_status() == -6


def test_stream_mix_rejects_bad_arguments(born):
    """Argument checks come before any CUDA call."""
    L, out = born.lib(), C.c_float()
    for args in ((0, 1, 16, 1), (9, 1, 16, 1), (1, 0, 16, 1), (1, 5, 16, 1),
                 (1, 1, 6, 1), (1, 1, 0, 1), (1, 1, 16, 0)):
        assert L.born_stream_mix_gbs(*args, C.byref(out)) == -1, args
    assert L.born_stream_mix_gbs(1, 1, 16, 1, None) == -1


def test_sinc_tables_match_oracle(born, po):
    for n in (1, 2, 3, 4, 5, 8, 16):
        assert np.array_equal(born.sinc_table(n), po.sinc_table(n)), n


def test_stability_and_compute_size_match_oracle(born, po):
    L = po.port_lib()
    for vmax, dmin, dtd, ntd in ((4000., 10., .001, 1000), (4500., 8., .001,
                                                           1501),
                                 (4500., 10., .004, 500)):
        nt = C.c_int()
        dt = L.oracle_calc_stability(vmax, dmin, dtd, ntd, C.byref(nt))
        assert born.calc_stability(vmax, dmin, dtd, ntd) == (dt, nt.value)
    for n in (128, 256, 512, 800, 1, 17):
        for nb in (0, 20, 50):
            assert born.compute_size(n, nb) == L.oracle_compute_size(n, nb, 4)
    assert born.compute_size(128, 20) == 176
    assert born.compute_size(256, 50) == 368
    assert born.compute_size(512, 50) == 624


def test_source_and_receiver_geometry_match_oracle(born, po):
    L = po.port_lib()
    wav = np.sin(np.arange(300) * 0.1).astype(np.float32)
    o = (-240.0, -240.0, -240.0)
    d = (10.0, 10.0, 10.0)
    locs, vals = born.source_geometry(640.0, 645.0, 20.0, o, d, 176, 176, wav,
                                      308)
    l2 = np.zeros(9, np.int32)
    v2 = np.zeros((9, 308), np.float32)
    L.oracle_source_geometry(640.0, 645.0, 20.0, *o, *d, 176, 176,
                             po.fptr(wav), wav.size, 308, po.iptr(l2),
                             po.fptr(v2))
    assert np.array_equal(locs, l2) and np.array_equal(vals, v2)
    r = born.receiver_geometry(64, 64, 0.0, 20.0, 0.0, 20.0, 10.0, o, d, 176,
                               176)
    r2 = np.zeros(64 * 64, np.int32)
    L.oracle_receiver_geometry(64, 64, 0.0, 20.0, 0.0, 20.0, 10.0, *o, *d,
                               176, 176, po.iptr(r2))
    assert np.array_equal(r, r2)
    wd = born.wavelet_deriv(wav, 0.001)
    wd2 = np.zeros_like(wav)
    L.oracle_wavelet_deriv(po.fptr(wav), wav.size, 0.001, po.fptr(wd2))
    assert np.array_equal(wd, wd2)


def test_random_boundary_matches_oracle(born, po):
    rng = np.random.default_rng(3)
    vel = (2000 + 500 * rng.random((12, 14, 16))).astype(np.float32)
    shape = (28, 30, 32)
    o, d = (-80.0, -80.0, -80.0), (10.0, 10.0, 10.0)
    vo, vd = (0.0, 0.0, 0.0), (10.0, 10.0, 10.0)
    for nrand in ((8, 8, 8), (0, 0, 0)):
        a = born.rand_subspace(vel, vo, vd, float(vel.max()), 123, nrand,
                               0.001, shape, o, d)
        b = np.zeros(shape, np.float32)
        po.port_lib().oracle_rand_subspace(
            po.fptr(vel), 16, 14, 12, *vo, *vd, float(vel.max()), 123,
            *nrand, 0.001, 32, 30, 28, *o, *d, po.fptr(b))
        assert np.array_equal(a, b), nrand


def test_linear_glue_matches_oracle(born, po):
    L, P = born.lib(), po.port_lib()
    rng = np.random.default_rng(4)
    n1, n2, n3 = 9, 7, 5
    m = rng.standard_normal((n3, n2, n1)).astype(np.float32)
    for add in (0, 1):
        for fb, fo in (("born_laplac_forward", "oracle_laplac_forward"),
                       ("born_laplac_adjoint", "oracle_laplac_adjoint")):
            a = rng.standard_normal(m.shape).astype(np.float32)
            b = a.copy()
            if "forward" in fb:
                getattr(L, fb)(add, born.fptr(m), born.fptr(a), n1, n2, n3)
                getattr(P, fo)(add, po.fptr(m), po.fptr(b), n1, n2, n3)
            else:
                getattr(L, fb)(add, born.fptr(a), born.fptr(m), n1, n2, n3)
                getattr(P, fo)(add, po.fptr(b), po.fptr(m), n1, n2, n3)
            assert np.array_equal(a, b), (fb, add)
        for fb, fo in (("born_deriv_forward", "oracle_deriv_forward"),
                       ("born_deriv_adjoint", "oracle_deriv_adjoint")):
            a = rng.standard_normal(m.shape).astype(np.float32)
            b = a.copy()
            if "forward" in fb:
                getattr(L, fb)(add, born.fptr(m), born.fptr(a), n1, n2, n3,
                               0.004)
                getattr(P, fo)(add, po.fptr(m), po.fptr(b), n1, n2, n3, 0.004)
            else:
                getattr(L, fb)(add, born.fptr(a), born.fptr(m), n1, n2, n3,
                               0.004)
                getattr(P, fo)(add, po.fptr(b), po.fptr(m), n1, n2, n3, 0.004)
            assert np.array_equal(a, b), (fb, add)
    nt, ntb = 20, 28
    traces = rng.standard_normal((3, 4, nt)).astype(np.float32)
    padded = rng.standard_normal((3, 4, ntb)).astype(np.float32)
    a, b = padded.copy(), padded.copy()
    L.born_map_data_adjoint(1, born.fptr(a), born.fptr(traces), nt, 4, 3, ntb)
    P.oracle_map_data_adjoint(1, po.fptr(b), po.fptr(traces), nt, 4, 3, ntb)
    assert np.array_equal(a, b)
    a, b = traces.copy(), traces.copy()
    L.born_map_data_forward(0, born.fptr(padded), born.fptr(a), nt, 4, 3, ntb)
    P.oracle_map_data_forward(0, po.fptr(padded), po.fptr(b), nt, 4, 3, ntb)
    assert np.array_equal(a, b)
    whole = rng.standard_normal((6, 7, 8)).astype(np.float32)
    sub_a = np.zeros((9, 9, 9), np.float32)
    sub_b = np.zeros((9, 9, 9), np.float32)
    L.born_extract_sub(born.fptr(whole), 8, 7, 6, born.fptr(sub_a), 9, 9, 9,
                       -2, -1, -3)
    P.oracle_extract_sub(po.fptr(whole), 8, 7, 6, po.fptr(sub_b), 9, 9, 9, -2,
                         -1, -3)
    assert np.array_equal(sub_a, sub_b)
    wa, wb = whole.copy(), whole.copy()
    L.born_add_image(born.fptr(wa), 8, 7, 6, born.fptr(sub_a), 9, 9, 9, -2,
                     -1, -3)
    P.oracle_add_image(po.fptr(wb), 8, 7, 6, po.fptr(sub_b), 9, 9, 9, -2, -1,
                       -3)
    assert np.array_equal(wa, wb)
    # window offsets from float origins (truncation toward zero on both
    # sides, and the compute grids of 4-55 boundary cells at odd spacings)
    f32 = np.float32
    trip = [(float(f32(o) - f32(d) * f32(k)), o, d)
            for o in (0.0, 13.7, -2.3) for d in (10.0, 10.1, 10.3, 8.33, 7.3)
            for k in range(4, 56)]
    trip += [tuple(float(f32(x)) for x in rng.uniform(-500, 500, 2)) +
             (float(f32(rng.uniform(1, 20))),) for _ in range(500)]
    got = [L.born_window_offset(*t) for t in trip]
    assert got == [P.oracle_window_offset(*t) for t in trip]
    assert L.born_window_offset(float(f32(-10.3) * f32(14)), 0.0, 10.3) == -13
    assert L.born_window_offset(-35.0, 0.0, 10.0) == -3  # not floor (-4)
