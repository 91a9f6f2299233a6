"""Exact Born coupling storage ("f32exact", BORN_STORE_F32_EXACT): the rtm
forward loop forms r += 1e-6 s img as the reference's double expression
(base/cpu_prop.cc:216-223), so Born traces, like the source levels and the
image, are bit-identical to the reference's fixtures and to the oracle; the
arithmetic itself is checked on the CPU in tests/test_couple_exact.py."""
import os

import numpy as np
import pytest

import cases
from test_oracle_golden import GOLDEN_FILES, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(born):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return born


def exact_prop(born, shape):
    nz, ny, nx = shape
    p = born.Gb300Prop()
    p.createSpace(10., 10., 10., 50, .0005, .0005, nx, ny, nz)
    p.set_storage("f32exact")
    assert p.storage == "f32exact"
    return p


def same(got, want):
    for k, v in want.items():
        assert np.array_equal(got[k], v), (k, float(np.abs(got[k] - v).max()))


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=os.path.basename)
def test_exact_coupling_matches_reference_fixture(gpu, po, path):
    case, out = load_golden(path)
    same(po.run_case(exact_prop(gpu, case["shape"]), case), out)


@pytest.mark.parametrize("seed,shape,nt,jt,dup", [
    (301, (40, 44, 56), 90, 1, 0), (302, (36, 30, 40), 61, 2, 3),
    (303, (72, 80, 96), 150, 2, 4)])
def test_exact_coupling_matches_oracle(gpu, po, seed, shape, nt, jt, dup):
    c = cases.make_case(seed, shape=shape, nt=nt, jt=jt, dup_receivers=dup,
                        sinc=po.sinc_table)
    want = po.run_case(po.PortProp(), c)
    same(po.run_case(exact_prop(gpu, shape), c), want)
    if seed == 303:
        # the float coupling of FP32 storage differs from it by a few ulps
        got = po.run_case(gpu.Gb300Prop(), c)
        assert not np.array_equal(got["traces"], want["traces"])


def test_exact_coupling_loop_tuning_keeps_results(gpu, po):
    # a loop of 400+ steps switches (tile, z segments) while timing itself
    c = cases.make_case(304, shape=(40, 44, 56), nt=420, jt=1,
                        sinc=po.sinc_table)
    p = exact_prop(gpu, c["shape"])
    same(po.run_case(p, c), po.run_case(po.PortProp(), c))
    ms = p.loop_tile_ms(1)
    assert all(v > 0 for v in ms), ms
