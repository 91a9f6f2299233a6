"""The exact linearised Born pair on the GPU: nonlinear modelling and the
tangent-linear forward against the oracle, the dot-product test
<J m, d> = <m, J^T d>, central finite differences of nonlinear modelling
with respect to slowness squared, and a torch.autograd.Function wrapper
(test harness only) whose backward is the adjoint kernel.

Tolerances: modelling and the linearised forward keep the oracle's
operation order (bit-identical expected, checked at 1e-6 relative L2); the
dot test compares two FP64 sums of FP32 fields (1e-5); finite differences
in FP32 with eps = 1e-3 (1e-3 relative error)."""
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


def setup(prop, c, vel2=None):
    nz, ny, nx = c["shape"]
    prop.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    prop.transferSincTableS(8, c["jts"], c["table_s"])
    prop.transferSincTableD(8, c["jtd"], c["table_d"])
    prop.transferSourceFunc(9, c["nt_big"], c["locs_s"], c["src"])
    prop.transferVelFunc1(nx, ny, nz, c["vel1"])
    prop.transferVelFunc2(nx, ny, nz, c["vel2"] if vel2 is None else vel2)
    rec = np.zeros_like(c["rec_in"])
    prop.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"],
                              c["locs_r"], rec)
    return rec


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def case(po, seed=81, shape=(36, 40, 48), nt=90, jt=1):
    return cases.make_case(seed, shape=shape, nt=nt, jt=jt,
                           sinc=po.sinc_table)


def test_model_and_lin_forward_match_oracle(gpu, po):
    c = case(po)
    g = gpu.Gb300Prop()
    setup(g, c)
    o = po.PortProp()
    po.run_case(o, c, which="none")
    rec_o = np.zeros_like(c["rec_in"])
    o.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"], c["locs_r"],
                           rec_o)
    o.model(c["jts"], rec_o, c["nt"])
    d = g.model(c["jts"], c["nt"])
    assert rel(d, rec_o) <= 1e-6
    m = np.random.default_rng(3).standard_normal(c["shape"]).astype(np.float32)
    rec_o[...] = 0
    o.lin_forward(c["jts"], m, rec_o, c["nt"])
    dl = g.lin_forward(c["jts"], c["nt"], m)
    assert rel(dl, rec_o) <= 1e-6


@pytest.mark.parametrize("interval", [7, 50])
def test_dot_product(gpu, po, interval):
    c = case(po, seed=82, nt=80, jt=2)
    g = gpu.Gb300Prop()
    setup(g, c)
    rng = np.random.default_rng(1004)
    m = rng.standard_normal(c["shape"]).astype(np.float32)
    d = rng.standard_normal(c["rec_in"].shape).astype(np.float32)
    lm = g.lin_forward(c["jts"], c["nt"], m)
    ltd = g.lin_adjoint(c["jts"], c["nt"], d, interval=interval)
    a = float(np.dot(lm.astype(np.float64).ravel(), d.astype(np.float64).ravel()))
    b = float(np.dot(m.astype(np.float64).ravel(), ltd.astype(np.float64).ravel()))
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b)), (a, b)


def test_finite_differences_slowness_squared(gpu, po):
    """32 probes: J (dV/dm) p  vs  (F(m + eps m p) - F(m - eps m p)) / 2eps,
    m = slowness squared, V = v^2 dt^2 = dt^2 / m."""
    c = case(po, seed=83, shape=(32, 36, 40), nt=70)
    g = gpu.Gb300Prop()
    setup(g, c)
    V = c["vel2"].astype(np.float64)
    rng = np.random.default_rng(1005)
    eps = 1e-3
    nz, ny, nx = c["shape"]
    errs = []
    for k in range(32):
        p = rng.standard_normal(c["shape"])
        # smooth probes, interior only
        p[:4] = p[-4:] = 0
        p[:, :4] = p[:, -4:] = 0
        p[:, :, :4] = p[:, :, -4:] = 0
        plus = (V / (1 + eps * p)).astype(np.float32)
        minus = (V / (1 - eps * p)).astype(np.float32)
        g.transferVelFunc2(nx, ny, nz, plus)
        fp = g.model(c["jts"], c["nt"]).astype(np.float64)
        g.transferVelFunc2(nx, ny, nz, minus)
        fm = g.model(c["jts"], c["nt"]).astype(np.float64)
        fd = (fp - fm) / (2 * eps)
        g.transferVelFunc2(nx, ny, nz, c["vel2"])
        jd = g.lin_forward(c["jts"], c["nt"],
                           (-V * p).astype(np.float32)).astype(np.float64)
        errs.append(np.linalg.norm(fd - jd) / np.linalg.norm(jd))
    assert max(errs) < 1e-3, max(errs)


def test_autograd_function_uses_adjoint_kernel(gpu, po):
    import torch
    c = case(po, seed=84, shape=(28, 32, 36), nt=50)
    g = gpu.Gb300Prop()
    setup(g, c)
    jt, nt = c["jts"], c["nt"]

    class Born(torch.autograd.Function):
        @staticmethod
        def forward(ctx, m):
            return torch.from_numpy(g.lin_forward(jt, nt, m.detach().numpy()))

        @staticmethod
        def backward(ctx, grad):
            return torch.from_numpy(
                g.lin_adjoint(jt, nt, grad.contiguous().numpy(), interval=16))

    rng = np.random.default_rng(9)
    m = torch.tensor(rng.standard_normal(c["shape"]).astype(np.float32),
                     requires_grad=True)
    d_obs = torch.tensor(rng.standard_normal(c["rec_in"].shape)
                         .astype(np.float32))
    loss = 0.5 * ((Born.apply(m) - d_obs) ** 2).sum()
    loss.backward()
    # gradient of 0.5|Jm - d|^2 is J^T (Jm - d)
    r = g.lin_forward(jt, nt, m.detach().numpy()) - d_obs.numpy()
    expect = g.lin_adjoint(jt, nt, r, interval=16)
    assert rel(m.grad.numpy(), expect) <= 1e-6
    # directional derivative check of the loss along a probe
    q = rng.standard_normal(c["shape"]).astype(np.float32)
    jq = g.lin_forward(jt, nt, q)
    dd = float(np.dot(r.ravel().astype(np.float64), jq.ravel()))
    gq = float(np.dot(m.grad.numpy().ravel().astype(np.float64), q.ravel()))
    assert abs(dd - gq) <= 1e-5 * abs(dd)


def test_lin_adjoint_phase_timing(gpu, po):
    """Phase timing (born_time_phases) records events only: the gradient is
    bit-identical with it on, and the four phase times are positive and add
    up to no more than the call's own time."""
    import time
    c = case(po, seed=83, nt=120)
    g = gpu.Gb300Prop()
    setup(g, c)
    rng = np.random.default_rng(5)
    tr = rng.standard_normal(c["rec_in"].shape).astype(np.float32)
    want = g.lin_adjoint(c["jts"], c["nt"], tr, interval=25)
    g.time_phases(True)
    t0 = time.perf_counter()
    got = g.lin_adjoint(c["jts"], c["nt"], tr, interval=25)
    wall_ms = 1e3 * (time.perf_counter() - t0)
    ms = g.phase_times()
    g.time_phases(False)
    assert np.array_equal(got, want)
    assert all(v > 0 for v in ms), ms
    assert sum(ms) <= wall_ms, (ms, wall_ms)


def test_lin_adjoint_reuses_forward_checkpoints(gpu, po):
    """born_lin_forward stores the background's checkpoints as it computes
    the background; born_lin_adjoint then skips its own checkpointing sweep
    (born_checkpoints_reused) and gives the same gradient bit for bit as
    with the sweep.  Any change of vel2 or the source makes it sweep again."""
    c = case(po, seed=84, nt=110)
    g = gpu.Gb300Prop()
    setup(g, c)
    L = g.lib
    rng = np.random.default_rng(6)
    m = (1e-3 * rng.standard_normal(c["shape"])).astype(np.float32)
    tr = rng.standard_normal(c["rec_in"].shape).astype(np.float32)
    # without stored checkpoints: the adjoint sweeps
    g.check(L.born_set_checkpoint_interval(g.h, 0))
    d0 = g.lin_forward(c["jts"], c["nt"], m)
    want = g.lin_adjoint(c["jts"], c["nt"], tr, interval=20)
    assert L.born_checkpoints_reused(g.h) == 0
    # the adjoint's own checkpoints serve the next adjoint
    again = g.lin_adjoint(c["jts"], c["nt"], tr, interval=20)
    assert L.born_checkpoints_reused(g.h) == 1
    assert np.array_equal(again, want)
    # checkpoints stored by the forward
    g.check(L.born_set_checkpoint_interval(g.h, 20))
    d1 = g.lin_forward(c["jts"], c["nt"], m)
    assert np.array_equal(d0, d1)
    got = g.lin_adjoint(c["jts"], c["nt"], tr, interval=20)
    assert L.born_checkpoints_reused(g.h) == 1
    assert np.array_equal(got, want)
    # another interval, or a changed vel2: a fresh sweep, same gradient
    g.lin_forward(c["jts"], c["nt"], m)
    other = g.lin_adjoint(c["jts"], c["nt"], tr, interval=15)
    assert L.born_checkpoints_reused(g.h) == 0
    assert np.array_equal(other, want)
    nz, ny, nx = c["shape"]
    g.lin_forward(c["jts"], c["nt"], m)
    g.transferVelFunc2(nx, ny, nz, c["vel2"] * np.float32(1.01))
    g.lin_adjoint(c["jts"], c["nt"], tr, interval=20)
    assert L.born_checkpoints_reused(g.h) == 0
