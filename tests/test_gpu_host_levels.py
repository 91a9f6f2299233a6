"""How rtmAdjoint reads the host arrays of the source levels.

The reference's operator calls sourceProp(p0, p1) and then
rtmAdjoint(p1, p0) (rtm_zero_op_3d.cc:272-282).  cpuProp reads the arrays
it is given; the reference's GPU path ignores them and keeps the levels on
the device (gpu_funcs_3d.cu:14, 409-445).  A caller that rewrites the
arrays between the two calls gets different images from the two.  The
handle's host-level policy (born_set_host_levels) makes the choice
explicit, and these tests pin each policy on a modified and an unmodified
array, through Gb300Prop and through the reference-named C entry points:

* resident (default): the arrays sourceProp filled select the
  device-resident levels; their contents are not read, so the image is the
  unmodified one;
* verify: a checksum taken when sourceProp wrote the arrays shows the
  change, the arrays are uploaded and the image is the oracle's image for
  the modified levels; unmodified arrays give the resident image;
* upload: the arrays are always read (the oracle's image either way).
"""
import ctypes as C

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


def setup(prop, c):
    nz, ny, nx = c["shape"]
    prop.createSpace(c["d"], c["d"], c["d"], 50.0, .0005, .0005, nx, ny, nz)
    prop.transferSincTableS(8, c["jts"], c["table_s"])
    prop.transferSincTableD(8, c["jtd"], c["table_d"])
    prop.transferSourceFunc(9, c["nt_big"], c["locs_s"], c["src"])
    prop.transferVelFunc1(nx, ny, nz, c["vel1"])
    prop.transferVelFunc2(nx, ny, nz, c["vel2"])
    rec = np.ascontiguousarray(c["rec_in"])
    prop.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"],
                              c["locs_r"], rec)


def adjoint_after(prop, c, modify):
    """sourceProp, then (optionally) a change of the host p0, then
    rtmAdjoint(p1, p0); returns the image and the arrays."""
    nz, ny, nx = c["shape"]
    p0 = np.zeros(c["shape"], np.float32)
    p1 = np.zeros(c["shape"], np.float32)
    prop.sourceProp(nx, ny, nz, False, True, p0, p1, c["jts"], 9, c["nt"])
    if modify:
        p0 *= np.float32(0.5)
        p0[5, 6, 7] += np.float32(1e-3)
    img = np.zeros(c["shape"], np.float32)
    prop.rtmAdjoint(nx, ny, nz, c["jtd"], p1, p0, img, 9, c["nt"])
    return img, p0, p1


def oracle_adjoint(po, c, p0, p1):
    prop = po.PortProp()
    setup(prop, c)
    nz, ny, nx = c["shape"]
    # rtmAdjoint scales the receiver injection by the jt of the last
    # sourceProp (cpu_prop.cc:108,182), so one runs first
    q0 = np.zeros(c["shape"], np.float32)
    q1 = np.zeros(c["shape"], np.float32)
    prop.sourceProp(nx, ny, nz, False, True, q0, q1, c["jts"], 9, c["nt"])
    img = np.zeros(c["shape"], np.float32)
    prop.rtmAdjoint(nx, ny, nz, c["jtd"], p1.copy(), p0.copy(), img, 9,
                    c["nt"])
    return img


@pytest.mark.parametrize("policy", ["resident", "verify", "upload"])
def test_host_level_policy_gb300prop(gpu, po, policy):
    c = cases.make_case(41, shape=(28, 32, 36), nt=48, jt=1,
                        sinc=po.sinc_table)
    want_plain = po.run_case(po.PortProp(), c, which="adjoint")["image"]
    for modify in (False, True):
        prop = gpu.Gb300Prop()
        prop.set_host_levels(policy)
        setup(prop, c)
        img, p0, p1 = adjoint_after(prop, c, modify)
        if not modify or policy == "resident":
            assert np.array_equal(img, want_plain), (policy, modify)
        else:
            want = oracle_adjoint(po, c, p0, p1)
            assert not np.array_equal(want, want_plain)
            assert np.array_equal(img, want), (policy, modify)


def test_host_level_policy_reference_entry_points(gpu, po):
    """The gpu_funcs_3d.h names on the default handle follow the same
    policy (set on born_default_handle())."""
    L = gpu.lib()
    c = cases.make_case(43, shape=(24, 28, 32), nt=40, jt=1,
                        sinc=po.sinc_table)
    want_plain = po.run_case(po.PortProp(), c, which="adjoint")["image"]
    nz, ny, nx = c["shape"]
    fp = gpu.fptr
    L.setup_cuda(1)
    h = L.born_default_handle()
    for policy, code in (("resident", 0), ("verify", 1), ("upload", 2)):
        assert L.born_set_host_levels(h, code) == 0
        L.create_gpu_space(c["d"], c["d"], c["d"], 50.0, .0005, .0005, nx,
                           ny, nz)
        ts = np.ascontiguousarray(c["table_s"])
        L.transfer_sinc_table_s(8, c["jts"], fp(ts))
        L.transfer_sinc_table_d(8, c["jtd"], fp(ts))
        L.transfer_source_func(9, c["nt_big"], gpu.iptr(c["locs_s"]),
                               fp(c["src"]))
        L.transfer_vel_func1(nx, ny, nz, fp(c["vel1"]))
        L.transfer_vel_func2(nx, ny, nz, fp(c["vel2"]))
        rec = np.ascontiguousarray(c["rec_in"])
        L.transfer_receiver_func(c["rec_nx"], c["rec_ny"], c["nt_big"],
                                 gpu.iptr(c["locs_r"]), fp(rec))
        p0 = np.zeros(c["shape"], np.float32)
        p1 = np.zeros(c["shape"], np.float32)
        L.source_prop(nx, ny, nz, False, True, fp(p0), fp(p1), c["jts"], 9,
                      c["nt"])
        assert L.born_default_status() == 0, L.born_default_error()
        p0 *= np.float32(0.5)
        img = np.zeros(c["shape"], np.float32)
        L.rtm_adjoint(nx, ny, nz, c["jtd"], fp(p1), fp(p0), fp(img), 9,
                      c["nt"])
        assert L.born_default_status() == 0, L.born_default_error()
        if policy == "resident":
            assert np.array_equal(img, want_plain)
        else:
            assert np.array_equal(img, oracle_adjoint(po, c, p0, p1)), policy
    assert L.born_set_host_levels(h, 0) == 0


def test_host_level_policy_rejects_unknown(gpu):
    prop = gpu.Gb300Prop()
    with pytest.raises(gpu.BornError):
        prop.check(prop.lib.born_set_host_levels(prop.h, 7))
