"""In-loop tiling refinement: the time loops time (tile, z segments)
candidates on their own steps, continue the sweep over later loops when one
loop is too short for it, and every candidate gives bit-identical results
(compared with a fixed tiling run on the same inputs)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(born):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return born


def setup(born, c, fixed=None):
    nz, ny, nx = c["shape"]
    p = born.Gb300Prop()
    if fixed is not None:
        p.set_tiling(*fixed)
    p.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    p.transferSincTableS(8, c["jts"], c["table_s"])
    p.transferSincTableD(8, c["jtd"], c["table_d"])
    p.transferSourceFunc(c["locs_s"].size, c["nt_big"], c["locs_s"], c["src"])
    p.transferVelFunc1(nx, ny, nz, c["vel1"])
    p.transferVelFunc2(nx, ny, nz, c["vel2"])
    p.check(p.lib.born_set_reflectivity(p.h, born.fptr(c["refl"])))
    return p


def shot(p, c):
    """rtm_zero_op order on device levels: receiver data, source, adjoint
    (image), Born forward (traces)."""
    p.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"], c["locs_r"],
                           np.ascontiguousarray(c["rec_in"]))
    p.source_prop_device(c["jts"], c["nt"])
    p.rtm_adjoint_device(c["jtd"], c["nt"], swap=1)
    img = p.get_image()
    p.zero_traces()
    p.rtm_forward_device(c["jtd"], c["nt"])
    return img, p.get_traces(c["rec_in"])


def complete(p):
    return [all(v > 0 for v in p.loop_tile_ms(m)) for m in (0, 1, 2)]


def test_tiling_sweep_spans_loops_and_keeps_results(gpu, po):
    # 128 interior planes: every tile has 8 z-segment candidates, one timed
    # group of 9 steps each plus two rounds over the best 8; a 400-step
    # loop holds 44 groups
    c = cases.make_case(77, shape=(136, 28, 32), nt=400, jt=1,
                        sinc=po.sinc_table)
    want = shot(setup(gpu, c, fixed=(1, 0)), c)
    p = setup(gpu, c)
    done = None
    for k in range(6):
        got = shot(p, c)
        assert np.array_equal(got[0], want[0]), k
        assert np.array_equal(got[1], want[1]), k
        if k == 0:
            assert not any(complete(p)), [p.loop_tile_ms(m) for m in (0, 1, 2)]
        if all(complete(p)):
            done = k
            break
    assert done is not None and done >= 1
    for m in (0, 1, 2):
        ms = p.loop_tile_ms(m)
        cfg, t = p.tuned_config(m)
        assert ms[cfg] == min(ms) and t == ms[cfg], (m, cfg, t, ms)
        assert 8 <= p.tuned_zseg(m) <= 128, p.tuned_zseg(m)
    # the tuned tiling keeps giving the same results
    got = shot(p, c)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_new_space_on_same_grid_keeps_tuning(gpu, po):
    c = cases.make_case(78, shape=(40, 44, 56), nt=420, jt=1,
                        sinc=po.sinc_table)
    p = setup(gpu, c)
    shot(p, c)
    assert all(complete(p))
    before = [(p.tuned_config(m), p.tuned_zseg(m)) for m in (0, 1, 2)]
    nz, ny, nx = c["shape"]
    p.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    assert all(complete(p))
    assert [(p.tuned_config(m), p.tuned_zseg(m)) for m in (0, 1, 2)] == before
    # another grid starts over
    p.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz + 4)
    assert not any(complete(p))


def test_launch_overlap_keeps_results(gpu, po):
    """Programmatic dependent launch of the steps (default) and plain
    launches give the same levels, image and traces, equal to the oracle."""
    c = cases.make_case(79, shape=(40, 44, 56), nt=90, jt=2,
                        sinc=po.sinc_table)
    want = po.run_case(po.PortProp(), c)
    got = {}
    for overlap in (True, False):
        p = gpu.Gb300Prop()
        p.set_launch_overlap(overlap)
        got[overlap] = po.run_case(p, c)
    for k in ("src_p0", "src_p1", "image", "traces"):
        assert np.array_equal(got[True][k], got[False][k]), k
    for k in ("src_p0", "src_p1", "image"):
        assert np.array_equal(got[True][k], want[k]), k
