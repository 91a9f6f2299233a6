"""16-bit wavefield storage (BF16 / FP16 with a power-of-two scale per
stored level, FP32 arithmetic) against the FP64 oracle.

Reduced-precision storage is judged by its error, not by bit equality: the
RTM image and the Born traces of each storage are compared with an FP64
propagation of the same case (the oracle's double instance), and FP32
storage must stay at the parity bound.  The per-level scaling is checked by
scale invariance: multiplying the source and the receiver data by 2^40
(far beyond FP16's range of 65504) must multiply every result by the same
power of two exactly, which holds only if every stored level carries its
own power-of-two scale."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

SHAPE = (40, 44, 56)  # nz, ny, nx (16-bit rows need nx % 8 == 0)
NT = 240


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def gpu(born):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return born


@pytest.fixture(scope="module")
def case(po):
    return cases.make_case(71, shape=SHAPE, nt=NT, jt=1, sinc=po.sinc_table)


@pytest.fixture(scope="module")
def fp64(po, case):
    return po.run_case(po.PortProp64(), case)


def run_device(born, c, storage, amp=1.0):
    """The reference call order of rtm_zero_op on device-resident levels:
    source propagation, RTM adjoint (image), Born forward (traces)."""
    nz, ny, nx = c["shape"]
    p = born.Gb300Prop()
    p.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    p.transferSincTableS(8, c["jts"], c["table_s"])
    p.transferSincTableD(8, c["jtd"], c["table_d"])
    p.transferSourceFunc(9, c["nt_big"], c["locs_s"],
                         np.ascontiguousarray(c["src"] * np.float32(amp)))
    p.transferVelFunc1(nx, ny, nz, c["vel1"])
    p.transferVelFunc2(nx, ny, nz, c["vel2"])
    p.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"], c["locs_r"],
                           np.ascontiguousarray(c["rec_in"] * np.float32(amp)))
    p.check(p.lib.born_set_reflectivity(p.h, born.fptr(c["refl"])))
    p.set_storage(storage)
    assert p.storage == storage
    p.source_prop_device(c["jts"], c["nt"])
    p.rtm_adjoint_device(c["jtd"], c["nt"], swap=1)
    img = p.get_image()
    p.zero_traces()
    p.rtm_forward_device(c["jtd"], c["nt"])
    return img, p.get_traces(c["rec_in"])


# (image, traces) relative L2 bounds against FP64 after NT steps for 16-bit
# storage; FP32 storage is held to the FP32 oracle's own distance from FP64
# (its arithmetic is the reference's, so the two round alike)
BOUNDS = {"f16": 1e-2, "bf16": 6e-2}


def test_storage_errors_against_fp64(gpu, po, case, fp64):
    o32 = po.run_case(po.PortProp(), case)
    e32 = (rel(o32["image"], fp64["image"]), rel(o32["traces"], fp64["traces"]))
    print(f"oracle f32: image rel L2 {e32[0]:.3e}, traces rel L2 {e32[1]:.3e}")
    BOUNDS["f32"] = max(1e-5, 1.5 * max(e32))
    err = {}
    for st in ("f32", "f16", "bf16"):
        img, tr = run_device(gpu, case, st)
        assert np.isfinite(img).all() and np.isfinite(tr).all(), st
        err[st] = (rel(img, fp64["image"]), rel(tr, fp64["traces"]))
        print(f"storage {st}: image rel L2 {err[st][0]:.3e}, "
              f"traces rel L2 {err[st][1]:.3e}")
    for st in err:
        assert max(err[st]) <= BOUNDS[st], (st, err[st])
    # FP16 keeps 11 significant bits against BF16's 8
    assert err["f16"][0] < err["bf16"][0] and err["f16"][1] < err["bf16"][1]


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_per_level_scaling_is_exact(gpu, case, storage):
    k = 40  # 2^40 * typical amplitudes overflows FP16 without scaling
    img1, tr1 = run_device(gpu, case, storage)
    img2, tr2 = run_device(gpu, case, storage, amp=2.0 ** k)
    # the image is s * r (both scaled), the traces are linear in s
    assert np.array_equal(img2, img1 * np.float32(2.0 ** (2 * k)))
    want = tr1 * np.float32(2.0 ** k)
    if storage == "f16":
        assert np.array_equal(tr2, want)
    else:
        # BF16 keeps FP32's exponent range, so the far tails of the
        # scattered field (and the trace samples before the wave arrives)
        # reach FP32's gradual underflow at the unscaled amplitude, where
        # scaling by 2^k is no longer exact; FP16 flushes them at 2^-24 of
        # the level's scale first
        assert rel(tr2, want) <= 1e-6


def test_storage_rejects_fp32_only_paths(gpu, case):
    born = gpu
    nz, ny, nx = case["shape"]
    p = born.Gb300Prop()
    p.createSpace(case["d"], case["d"], case["d"], 50, .0005, .0005, nx, ny,
                  nz)
    p.set_storage("bf16")
    lv = np.zeros(case["shape"], np.float32)
    # host copies of the levels are FP32-only (BORN_ESTATE = -4)
    assert p.lib.born_get_source_levels(p.h, born.fptr(lv),
                                        born.fptr(lv)) == -4
    q = born.Gb300Prop()
    q.createSpace(case["d"], case["d"], case["d"], 50, .0005, .0005, 36, ny,
                  nz)
    with pytest.raises(born.BornError):  # 16-bit rows need nx % 8 == 0
        q.set_storage("f16")


def test_f16_odd_nt_and_jt2_against_fp64(gpu, po):
    # jt = 2 (sinc interpolation) and odd nt (the final level copy of the
    # source propagation and the last pending source injection of the
    # adjoint act on 16-bit levels and their records)
    c = cases.make_case(73, shape=(32, 36, 48), nt=121, jt=2,
                        sinc=po.sinc_table)
    want = po.run_case(po.PortProp64(), c)
    img, tr = run_device(gpu, c, "f16")
    e = (rel(img, want["image"]), rel(tr, want["traces"]))
    print(f"f16 jt=2 nt=121: image rel L2 {e[0]:.3e}, traces {e[1]:.3e}")
    assert max(e) <= 1e-2, e


@pytest.mark.parametrize("seed,shape,nt,jt,dup", [
    (81, (40, 44, 56), 120, 1, 0), (82, (36, 30, 40), 61, 2, 3)])
def test_fused_fp32_within_parity_bound(gpu, po, seed, shape, nt, jt, dup):
    # FP32 levels with fused multiply-adds: not bit-identical to the
    # reference order, but within the 1e-5 relative L2 bound of plain FP32
    c = cases.make_case(seed, shape=shape, nt=nt, jt=jt, dup_receivers=dup,
                        sinc=po.sinc_table)
    nz, ny, nx = shape
    prop = gpu.Gb300Prop()
    prop.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    prop.set_storage("f32fma")
    got = po.run_case(prop, c)
    want = po.run_case(po.PortProp(), c)
    for k, v in want.items():
        e = rel(got[k], v)
        print(f"f32fma {k}: rel L2 {e:.2e}")
        assert e <= 1e-5, (k, e)
