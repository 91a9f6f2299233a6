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


def adversarial_inputs(n, seed=0):
    """The input classes of tests/cpp/couple_check.cc, drawn with numpy."""
    rng = np.random.default_rng(seed)

    def rand_float(lo, hi, size):
        e = rng.integers(lo, hi + 1, size, dtype=np.uint32)
        mant = rng.integers(0, 1 << 23, size, dtype=np.uint32)
        sign = rng.integers(0, 2, size, dtype=np.uint32) << 31
        return (sign | (e << 23) | mant).view(np.float32)

    def log_uniform(lo10, hi10, size):
        v = 10.0 ** rng.uniform(lo10, hi10, size)
        return np.where(rng.integers(0, 2, size) == 1, v, -v)

    rs, ss, ms = [], [], []
    # wavefield-like magnitudes
    r = log_uniform(-48, 0, n)
    r[::4] = 0.0
    rs.append(r)
    ss.append(log_uniform(-40, 2, n))
    ms.append(log_uniform(-4, -1, n))
    # every finite exponent
    for lst in (rs, ss, ms):
        lst.append(rand_float(0, 254, n))
    # r + V near r + half an ulp of r
    r = rand_float(60, 200, n)
    s = log_uniform(-20, 2, n).astype(np.float32)
    er = ((r.view(np.uint32) >> 23) & 0xff).astype(np.int64) - 127
    half = np.ldexp(1.0, er - 24) * (
        1.0 + np.ldexp(rng.uniform(-0.5, 0.5, n), -rng.integers(0, 40, n)))
    sign = np.where(rng.integers(0, 2, n) == 1, 1.0, -1.0)
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        m = (sign * half / (1e-6 * s.astype(np.float64))).astype(np.float32)
    keep = np.isfinite(m) & (m != 0)
    rs.append(r[keep])
    ss.append(s[keep])
    ms.append(m[keep])
    # underflow thresholds
    r = rand_float(0, 70, n)
    r[::3] = 0.0
    rs.append(r)
    ss.append(rand_float(0, 60, n))
    ms.append(rand_float(90, 140, n))
    # results around the smallest normal floats
    rs.append(rand_float(0, 6, n))
    ss.append(rand_float(20, 100, n))
    ms.append(rand_float(100, 140, n))
    # signed zeros
    z = np.array([0.0, -0.0], np.float32)
    rz, sz, mz = np.meshgrid(z, z, np.array([0.0, -0.0, 1e-3, -1e-3],
                                            np.float32), indexing="ij")
    rs.append(rz.ravel())
    ss.append(sz.ravel())
    ms.append(mz.ravel())
    return [np.ascontiguousarray(np.concatenate(x).astype(np.float32))
            for x in (rs, ss, ms)]


def test_device_coupling_matches_double_expression(gpu):
    """The forward step's exact-coupling arithmetic (two cells per thread,
    packed pairs, out-of-line double fallback) on adversarial inputs equals
    the reference's double expression bit for bit."""
    import torch
    r, s, m = adversarial_inputs(1_000_000)
    want = (r.astype(np.float64) + 1e-6 * s.astype(np.float64) *
            m.astype(np.float64))
    with np.errstate(over="ignore"):
        want = want.astype(np.float32)
    dev = [torch.from_numpy(a).cuda() for a in (r, s, m)]
    out = torch.empty_like(dev[0])
    torch.cuda.synchronize()
    lib = gpu.lib()
    rc = lib.born_couple_exact_device(dev[0].data_ptr(), dev[1].data_ptr(),
                                      dev[2].data_ptr(), out.data_ptr(),
                                      out.numel(), None)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
    assert bad.size == 0, (bad.size, r[bad[:3]], s[bad[:3]], m[bad[:3]],
                           got[bad[:3]], want[bad[:3]])
