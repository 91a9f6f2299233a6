"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference fixtures, on the reference's own call sequence.

Tolerances.  The stencil, taper, injection and imaging kernels keep the
reference's operation order with separately rounded multiplies and adds, so
source levels and RTM images are expected to be identical bit for bit.  The
Born coupling r += 1e-6 s img is formed in double by the reference
(cpu_prop.cc:220) and in float here, so Born traces are compared at a
relative L2 of 1e-5, the parity bound of the task."""
import glob
import os

import numpy as np
import pytest

import cases
from test_oracle_golden import GOLDEN_FILES, load_golden

pytestmark = pytest.mark.gpu
TRACE_RTOL = 1e-5


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def gpu(born):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return born


def check(got, ref, exact=("src_p0", "src_p1", "image")):
    for k, v in ref.items():
        if k in exact:
            assert np.array_equal(got[k], v), (k, rel(got[k], v))
        else:
            assert rel(got[k], v) <= TRACE_RTOL, (k, rel(got[k], v))


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=os.path.basename)
def test_gpu_matches_reference_fixture(gpu, po, path):
    case, out = load_golden(path)
    got = po.run_case(gpu.Gb300Prop(), case)
    check(got, out)


@pytest.mark.parametrize("cfg", range(8))
def test_gpu_matches_oracle_all_tile_configs(gpu, po, cfg):
    # 48 interior columns: a partial second 32- or 64-wide tile
    if cfg >= gpu.lib().born_tile_config_count():
        pytest.skip("no such tile configuration")
    c = cases.make_case(31 + cfg, shape=(40, 44, 56), nt=60, jt=1,
                        sinc=po.sinc_table)
    prop = gpu.Gb300Prop()
    prop.set_tiling(cfg, 0)
    got = po.run_case(prop, c)
    check(got, po.run_case(po.PortProp(), c))


@pytest.mark.parametrize("zseg", [1, 5, 16])
def test_gpu_z_segments(gpu, po, zseg):
    c = cases.make_case(41, shape=(36, 30, 40), nt=30, jt=2,
                        sinc=po.sinc_table)
    prop = gpu.Gb300Prop()
    prop.set_tiling(1, zseg)
    check(po.run_case(prop, c), po.run_case(po.PortProp(), c))


@pytest.mark.parametrize("nt", [1, 2, 3])
def test_gpu_short_time_loops(gpu, po, nt):
    # nt = 1, 2 exercise the adjoint steps without one or both propagations
    c = cases.make_case(50 + nt, shape=(20, 24, 28), nt=nt, jt=1,
                        sinc=po.sinc_table)
    check(po.run_case(gpu.Gb300Prop(), c), po.run_case(po.PortProp(), c))


def test_gpu_larger_grid_against_oracle(gpu, po):
    c = cases.make_case(61, shape=(72, 80, 96), nt=150, jt=2,
                        dup_receivers=4, sinc=po.sinc_table)
    check(po.run_case(gpu.Gb300Prop(), c), po.run_case(po.PortProp(), c))


def test_gpu_fp64_accuracy(gpu, po):
    c = cases.make_case(62, shape=(40, 44, 56), nt=80, jt=1,
                        sinc=po.sinc_table)
    got = po.run_case(gpu.Gb300Prop(), c)
    ref = po.run_case(po.PortProp64(), c)
    for k in got:
        assert rel(got[k], ref[k]) < 1e-4, (k, rel(got[k], ref[k]))


def test_reference_c_abi_sequence(gpu, po):
    """The gpu_funcs_3d.h entry points, called the way gpu_prop.cc does."""
    import ctypes as C
    L = gpu.lib()
    c = cases.make_case(71, shape=(24, 28, 32), nt=40, jt=1,
                        sinc=po.sinc_table)
    nz, ny, nx = c["shape"]
    f = gpu.fptr
    L.setup_cuda(1)
    L.create_gpu_space(10.0, 10.0, 10.0, 50.0, .0005, .0005, nx, ny, nz)
    ts = np.ascontiguousarray(c["table_s"], np.float32)
    L.transfer_sinc_table_s(8, 1, f(ts))
    L.set_ntblock(50)
    L.transfer_sinc_table_d(8, 1, f(ts))
    locs_s = np.ascontiguousarray(c["locs_s"], np.int32)
    L.transfer_source_func(9, c["nt_big"], gpu.iptr(locs_s), f(c["src"]))
    L.transfer_vel_func1(nx, ny, nz, f(c["vel1"]))
    L.transfer_vel_func2(nx, ny, nz, f(c["vel2"]))
    rec = np.ascontiguousarray(c["rec_in"], np.float32)
    L.transfer_receiver_func(c["rec_nx"], c["rec_ny"], c["nt_big"],
                             gpu.iptr(c["locs_r"]), f(rec))
    p0 = np.zeros(c["shape"], np.float32)
    p1 = np.zeros(c["shape"], np.float32)
    L.source_prop(nx, ny, nz, False, True, f(p0), f(p1), 1, 9, c["nt"])
    assert L.born_default_status() == 0, L.born_default_error()
    img = np.zeros(c["shape"], np.float32)
    L.rtm_adjoint(nx, ny, nz, 1, f(p1), f(p0), f(img), 9, c["nt"])
    assert L.born_default_status() == 0, L.born_default_error()
    ref = po.run_case(po.PortProp(), c, which="adjoint")
    assert np.array_equal(p0, ref["src_p0"])
    assert np.array_equal(img, ref["image"])
    # bad input is reported, not fatal
    L.create_gpu_space(10.0, 10.0, 10.0, 50.0, .0005, .0005, 30, 28, 24)
    assert L.born_default_status() == -1


def test_invalid_points_rejected(gpu):
    prop = gpu.Gb300Prop()
    prop.createSpace(10., 10., 10., 50, .0005, .0005, 32, 28, 24)
    with pytest.raises(gpu.BornError):
        prop.transferSourceFunc(1, 16, np.array([0], np.int32),
                                np.zeros(16, np.float32))
    with pytest.raises(gpu.BornError):
        prop.rtm_adjoint_device(1, 10)  # no source levels yet


def test_call_sequence_errors_are_status_codes(gpu):
    # out-of-order calls and bad arguments return BORN_E* codes and leave the
    # handle usable (the reference exits the process instead)
    EINVAL, ESTATE = -1, -4
    prop = gpu.Gb300Prop()
    L, h = prop.lib, prop.h
    assert L.born_source_prop(h, 1, 10, None, None) == ESTATE  # no grid
    assert L.born_create_space(h, 10., 10., 10., 50., .0005, .0005,
                               30, 24, 20) == EINVAL          # nx % 4 != 0
    assert L.born_create_space(h, 10., 10., 10., 50., .0005, .0005,
                               32, 8, 20) == EINVAL           # n < 9
    prop.createSpace(10., 10., 10., 50, .0005, .0005, 32, 24, 20)
    assert L.born_source_prop(h, 1, 10, None, None) == ESTATE  # no vel1
    assert L.born_rtm_adjoint(h, 1, 10, 1, None) == ESTATE     # no velocities
    assert L.born_rtm_forward(h, 1, 10, None) == ESTATE        # no vel2/refl
    assert L.born_source_prop(h, 0, 10, None, None) == EINVAL  # jts < 1
    assert L.born_set_tiling(h, 99, 0) == EINVAL
    assert L.born_set_storage(h, 7) == EINVAL
    assert L.born_error_string(h)  # the last failure's message is kept
    # the handle still works after the errors
    vel = np.full((20, 24, 32), 0.1, np.float32)
    prop.transferVelFunc1(32, 24, 20, vel)
    prop.transferVelFunc2(32, 24, 20, vel)
    prop.transferSincTableS(8, 1, np.ones(8, np.float32) / 8)
    prop.transferSourceFunc(0, 16, np.zeros(0, np.int32),
                            np.zeros((0, 16), np.float32))
    prop.source_prop_device(1, 10)
    prop.synchronize()


def test_device_image_view_and_single_rank_stack(gpu, po):
    c = cases.make_case(91, shape=(20, 24, 28), nt=30, jt=1,
                        sinc=po.sinc_table)
    prop = gpu.Gb300Prop()
    got = po.run_case(prop, c, which="adjoint")
    t = prop.image_tensor()  # the handle's image buffer, no copy
    assert t.is_cuda and tuple(t.shape) == c["shape"]
    assert np.array_equal(t.cpu().numpy(), prop.get_image())
    assert np.array_equal(t.cpu().numpy(), got["image"])
    # without a process group the stack is the image itself
    assert np.array_equal(gpu.stack_image(prop).cpu().numpy(), got["image"])


def test_loop_tile_refinement_keeps_parity(gpu, po):
    """A loop of 400 steps or more switches tiles while it times its own
    steps; results stay bit-identical and each mode keeps the tile with the
    smallest measured time."""
    c = cases.make_case(41, shape=(40, 44, 56), nt=420, jt=1,
                        sinc=po.sinc_table)
    prop = gpu.Gb300Prop()
    got = po.run_case(prop, c)
    check(got, po.run_case(po.PortProp(), c))
    for mode in (0, 1, 2):  # source, forward, adjoint
        ms = prop.loop_tile_ms(mode)
        assert all(v > 0 for v in ms), (mode, ms)
        cfg, _ = prop.tuned_config(mode)
        assert ms[cfg] == min(ms), (mode, cfg, ms)


def test_stream_mix_ceiling_measures(gpu):
    """The streaming-ceiling probe runs and gives a plausible HBM rate for a
    mix larger than L2 (2 x 64 MiB for a copy, 10 x 64 MiB for the
    adjoint's mix)."""
    n = 1 << 24
    for r, w in ((1, 1), (7, 3)):
        gbs = gpu.stream_mix_gbs(r, w, n, reps=3)
        assert 500.0 < gbs < 20000.0, (r, w, gbs)


def test_gpu_matches_oracle_random_shapes(gpu, po):
    """Random grid shapes (nx a multiple of 4, the other axes any size >= 9
    plus the stencil halo), sinc ratios and step counts, default tiling."""
    rng = np.random.default_rng(91)
    for k in range(4):
        shape = (int(rng.integers(14, 40)), int(rng.integers(14, 40)),
                 4 * int(rng.integers(5, 12)))
        jt = int(rng.integers(1, 4))
        nt = int(rng.integers(3, 25))
        c = cases.make_case(200 + k, shape=shape, nt=nt, jt=jt,
                            dup_receivers=int(k % 2), sinc=po.sinc_table)
        got = po.run_case(gpu.Gb300Prop(), c)
        check(got, po.run_case(po.PortProp(), c))


def test_bounded_wait_gives_up_with_status_and_handle_stays_usable(gpu, po):
    """Failure detection without a GPU fault: a bounded wait on an mbarrier
    that nothing completes gives up (about 2 s), the host reads
    BORN_ETIMEOUT, and the same handle then propagates bit-exactly."""
    prop = gpu.Gb300Prop()
    c = cases.make_case(51, shape=(20, 24, 28), nt=12, jt=1,
                        sinc=po.sinc_table)
    po.run_case(prop, c, which="none")  # grid and inputs in place
    assert prop.lib.born_selftest_wait_timeout(prop.h) == -5
    assert prop.lib.born_synchronize(prop.h) == 0  # error word cleared
    check(po.run_case(prop, c), po.run_case(po.PortProp(), c))


@pytest.mark.parametrize("storage", ["f32", "f32exact"])
def test_points_on_the_interior_corners(gpu, po, storage):
    """Sources and receivers on the outermost interior cells (x, y, z = 4
    and n - 5: the taper, the tile and segment edges and the halo meet
    there), some cells holding several points, jt = 2, against the oracle:
    levels and image bit for bit, traces within the bound (bit for bit with
    the exact coupling)."""
    shape = (28, 36, 40)
    c = cases.make_case(97, shape=shape, nt=61, jt=2, sinc=po.sinc_table)
    nz, ny, nx = shape
    corners = [x + y * nx + z * nx * ny
               for z in (4, nz - 5) for y in (4, ny - 5) for x in (4, nx - 5)]
    # 8 corners, then 4 of them again (points sharing a cell)
    locs_r = np.array(corners + corners[:4], np.int32)
    c["locs_r"] = locs_r
    c["rec_nx"], c["rec_ny"] = 4, 3
    rng = np.random.default_rng(98)
    rec = np.zeros((12, c["nt_big"]), np.float32)
    rec[:, 4:-4] = 1e-3 * rng.standard_normal((12, c["nt_big"] - 8))
    c["rec_in"] = rec
    # the 9 sources: 6 corners and 3 of them again
    c["locs_s"] = np.array(corners[:6] + corners[:3], np.int32)
    prop = gpu.Gb300Prop()
    prop.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    prop.set_storage(storage)
    got = po.run_case(prop, c)
    want = po.run_case(po.PortProp(), c)
    assert np.linalg.norm(want["image"]) > 0
    assert np.linalg.norm(want["traces"]) > 0
    if storage == "f32exact":
        check(got, want, exact=("src_p0", "src_p1", "image", "traces"))
    else:
        check(got, want)
