"""The Born operator (rtm_zero_op behind the my_operator contract) and CG.

* reference mode against the same per-shot chain composed from the oracle
  (oracle geometry + oracle cpuProp restatement + oracle glue), following
  rtm_zero_op_3d.cc:101-299: the adjoint image must match bit for bit, the
  Born data to 1e-5 (the 1e-6 coupling is formed in double by the
  reference, in float here);
* add = 1 accumulates, add = 0 overwrites (my_operator.h:18-25);
* exact mode: dot-product test of the whole operator (1e-5);
* CG: the device cgstep reproduces an FP64 numpy restatement of
  cgstep.cc:11-54 driven by the same operator, and the residual decreases.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def torch_cuda(born):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def setup_problem(seed=7, n=(20, 22, 24), nbound=6, nt_data=60, nshots=2,
                  d=10.0):
    rng = np.random.default_rng(seed)
    n3, n2, n1 = n
    z = np.arange(n3)[:, None, None]
    vel = (2000.0 + 40.0 * z + 100 * rng.random(n)).astype(np.float32)
    shots = np.array([[d * (n1 // 2 + k), d * (n2 // 2), 20.0]
                      for k in range(nshots)], np.float32)
    t = -0.02 + np.arange(80) * 0.001
    a = (np.pi * 25.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    kw = dict(velocity=vel, o=(0., 0., 0.), d=(d, d, d), shots=shots,
              wavelet=wav, dt_wavelet=0.001, nt_data=nt_data, dt_data=0.001,
              rec_n=(n1 // 2, n2 // 2), rec_o=(10.0, 10.0),
              rec_d=(2 * d, 2 * d), rec_depth=10.0, nbound=nbound)
    return kw


def oracle_operator(po, kw, model=None, data=None):
    """rtm_zero_op forward (model -> data) or adjoint (data -> model),
    composed from oracle pieces only."""
    L = po.port_lib()
    vel = kw["velocity"]
    n3, n2, n1 = vel.shape
    d = kw["d"][0]
    nb = kw["nbound"]
    nt_c = C.c_int()
    dt = L.oracle_calc_stability(float(vel.max()), d, kw["dt_data"],
                                 kw["nt_data"], C.byref(nt_c))
    nt = nt_c.value
    jt = int(np.float32(kw["dt_data"]) / np.float32(dt))  # float / float
    nc = [L.oracle_compute_size(m, nb, 4) for m in (n1, n2, n3)]
    f = nb + 4
    # compute-grid origin o + (-d * f) in float (source_func_3d.cc:65-67) and
    # the image window's offset formed from it (image_rtm_3d.cc:33-35)
    oc = float(np.float32(0) + np.float32(-d) * np.float32(f))
    w = L.oracle_window_offset(oc, 0.0, d)
    tab = po.sinc_table(jt)
    wav = np.ascontiguousarray(kw["wavelet"])
    wd = np.zeros_like(wav)
    L.oracle_wavelet_deriv(po.fptr(wav), wav.size, kw["dt_wavelet"],
                           po.fptr(wd))
    rnx, rny = kw["rec_n"]
    locs_r = np.zeros(rnx * rny, np.int32)
    L.oracle_receiver_geometry(rnx, rny, kw["rec_o"][0], kw["rec_d"][0],
                               kw["rec_o"][1], kw["rec_d"][1],
                               kw["rec_depth"], oc, oc, oc, d, d, d, nc[0],
                               nc[1], po.iptr(locs_r))
    nt_data, nt_big = kw["nt_data"], kw["nt_data"] + 8
    shape_c = (nc[2], nc[1], nc[0])
    out = np.zeros((len(kw["shots"]), rny, rnx, nt_data), np.float32) \
        if model is not None else np.zeros(vel.shape, np.float32)
    for s, (sx, sy, sz) in enumerate(kw["shots"]):
        locs_s = np.zeros(9, np.int32)
        vals = np.zeros((9, nt_big), np.float32)
        L.oracle_source_geometry(float(sx), float(sy), float(sz), oc, oc, oc,
                                 d, d, d, nc[0], nc[1], po.fptr(wd), wd.size,
                                 nt_big, po.iptr(locs_s), po.fptr(vals))
        seed = int(locs_s[3] % 10000)
        vr = np.zeros(shape_c, np.float32)
        vn = np.zeros(shape_c, np.float32)
        for arr, nr in ((vr, nb), (vn, 0)):
            L.oracle_rand_subspace(po.fptr(vel), n1, n2, n3, 0., 0., 0., d, d,
                                   d, float(vel.max()), seed, nr, nr, nr, dt,
                                   nc[0], nc[1], nc[2], oc, oc, oc, d, d, d,
                                   po.fptr(arr))
        prop = po.PortProp()
        prop.createSpace(d, d, d, 50, .0005, .0005, nc[0], nc[1], nc[2])
        prop.transferSincTableS(8, jt, tab)
        prop.transferSincTableD(8, jt, tab)
        prop.transferSourceFunc(9, nt_big, locs_s, vals)
        prop.transferVelFunc1(nc[0], nc[1], nc[2], vr)
        prop.transferVelFunc2(nc[0], nc[1], nc[2], vn)
        if model is not None:
            img = np.zeros(shape_c, np.float32)
            L.oracle_extract_sub(po.fptr(model), n1, n2, n3, po.fptr(img),
                                 nc[0], nc[1], nc[2], w, w, w)
            lap = np.zeros(shape_c, np.float32)
            L.oracle_laplac_forward(0, po.fptr(img), po.fptr(lap), nc[0],
                                    nc[1], nc[2])
            rec = np.zeros((rnx * rny, nt_big), np.float32)
            prop.transferReceiverFunc(rnx, rny, nt_big, locs_r, rec)
            prop.rtmForward(nc[0], nc[1], nc[2], jt, lap, rec, 9, nt, nt_big,
                            rnx, rny)
            sd = np.zeros((rny, rnx, nt_data), np.float32)
            L.oracle_map_data_forward(0, po.fptr(rec), po.fptr(sd), nt_data,
                                      rnx, rny, nt_big)
            shot = np.zeros_like(sd)
            L.oracle_deriv_forward(0, po.fptr(sd), po.fptr(shot), nt_data,
                                   rnx, rny, kw["dt_data"])
            out[s] += shot
        else:
            sd = np.zeros((rny, rnx, nt_data), np.float32)
            ds = np.ascontiguousarray(data[s])
            L.oracle_deriv_adjoint(0, po.fptr(sd), po.fptr(ds), nt_data, rnx,
                                   rny, kw["dt_data"])
            rec = np.zeros((rnx * rny, nt_big), np.float32)
            L.oracle_map_data_adjoint(0, po.fptr(rec), po.fptr(sd), nt_data,
                                      rnx, rny, nt_big)
            prop.transferReceiverFunc(rnx, rny, nt_big, locs_r, rec)
            p0 = np.zeros(shape_c, np.float32)
            p1 = np.zeros(shape_c, np.float32)
            prop.sourceProp(nc[0], nc[1], nc[2], False, True, p0, p1, jt, 9,
                            nt)
            img = np.zeros(shape_c, np.float32)
            prop.rtmAdjoint(nc[0], nc[1], nc[2], jt, p1, p0, img, 9, nt)
            lap = np.zeros(shape_c, np.float32)
            L.oracle_laplac_adjoint(0, po.fptr(lap), po.fptr(img), nc[0],
                                    nc[1], nc[2])
            L.oracle_add_image(po.fptr(out), n1, n2, n3, po.fptr(lap), nc[0],
                               nc[1], nc[2], w, w, w)
    return out


def test_reference_operator_matches_oracle_chain(born, po, torch_cuda):
    torch = torch_cuda
    kw = setup_problem()
    op = born.BornOperator(**kw)
    rng = np.random.default_rng(11)
    m = rng.standard_normal(op.model_shape).astype(np.float32)
    dm = torch.from_numpy(m).cuda()
    dd = torch.zeros(op.data_shape, device="cuda")
    op.forward(False, dm, dd)
    want = oracle_operator(po, kw, model=m)
    assert rel(dd.cpu().numpy(), want) <= 1e-5
    data = rng.standard_normal(op.data_shape).astype(np.float32)
    ma = torch.zeros(op.model_shape, device="cuda")
    op.adjoint(False, ma, torch.from_numpy(data).cuda())
    want = oracle_operator(po, kw, data=data)
    got = ma.cpu().numpy()
    assert rel(got, want) <= 1e-6, rel(got, want)
    # add = 1 accumulates onto the output, add = 0 overwrites it
    op.adjoint(True, ma, torch.from_numpy(data).cuda())
    assert rel(ma.cpu().numpy(), 2 * got) <= 1e-6
    op.adjoint(False, ma, torch.from_numpy(data).cuda())
    assert rel(ma.cpu().numpy(), got) == 0.0


def test_reference_operator_window_from_float_origins(born, po, torch_cuda):
    """At 10.3 m spacing and 10 boundary cells the compute grid starts at
    -144.2 m, which the reference's image window truncates to sample -13,
    not -14; the operator windows the model there too."""
    torch = torch_cuda
    kw = setup_problem(seed=5, nbound=10, nt_data=40, nshots=1, d=10.3)
    L = po.port_lib()
    oc = float(np.float32(-10.3) * np.float32(14))
    assert L.oracle_window_offset(oc, 0.0, 10.3) == -13
    op = born.BornOperator(**kw)
    rng = np.random.default_rng(12)
    m = rng.standard_normal(op.model_shape).astype(np.float32)
    dd = torch.zeros(op.data_shape, device="cuda")
    op.forward(False, torch.from_numpy(m).cuda(), dd)
    want = oracle_operator(po, kw, model=m)
    assert rel(dd.cpu().numpy(), want) <= 1e-5
    data = rng.standard_normal(op.data_shape).astype(np.float32)
    ma = torch.zeros(op.model_shape, device="cuda")
    op.adjoint(False, ma, torch.from_numpy(data).cuda())
    want = oracle_operator(po, kw, data=data)
    assert rel(ma.cpu().numpy(), want) <= 1e-6


def test_exact_operator_dot_product(born, torch_cuda):
    torch = torch_cuda
    kw = setup_problem(seed=8, nshots=2)
    op = born.BornOperator(exact=True, ckpt_interval=13, **kw)
    g = torch.Generator(device="cuda").manual_seed(1004)
    m = torch.randn(op.model_shape, device="cuda", generator=g)
    d = torch.randn(op.data_shape, device="cuda", generator=g)
    lm = torch.zeros(op.data_shape, device="cuda")
    ltd = torch.zeros(op.model_shape, device="cuda")
    op.forward(False, m, lm)
    op.adjoint(False, ltd, d)
    a = op.dot(lm, d)
    b = op.dot(m, ltd)
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b)), (a, b)
    # device FP64 dot agrees with a host FP64 dot
    host = float(np.dot(lm.cpu().numpy().astype(np.float64).ravel(),
                        d.cpu().numpy().astype(np.float64).ravel()))
    assert abs(a - host) <= 1e-10 * abs(host)


def test_cg_matches_fp64_restatement(born, torch_cuda):
    torch = torch_cuda
    kw = setup_problem(seed=9, nshots=1, nt_data=50)
    op = born.BornOperator(exact=True, ckpt_interval=16, **kw)
    rng = np.random.default_rng(1002)
    m_true = np.zeros(op.model_shape, np.float32)
    m_true[10:12] = rng.choice([-1.0, 1.0], size=m_true[10:12].shape) * 1e-3
    d_obs = torch.zeros(op.data_shape, device="cuda")
    op.forward(False, torch.from_numpy(m_true).cuda(), d_obs)
    niter = 4
    m_gpu = torch.zeros(op.model_shape, device="cuda")
    res = op.cg(d_obs, m_gpu, niter)
    assert all(res[i + 1] < res[i] for i in range(niter)), res

    # FP64 numpy cgstep (cgstep.cc:11-54) with the same operator
    def L(x):
        out = torch.zeros(op.data_shape, device="cuda")
        op.forward(False, torch.from_numpy(x.astype(np.float32)).cuda(), out)
        return out.cpu().numpy().astype(np.float64)

    def Lt(y):
        out = torch.zeros(op.model_shape, device="cuda")
        op.adjoint(False, out, torch.from_numpy(y.astype(np.float32)).cuda())
        return out.cpu().numpy().astype(np.float64)

    d = d_obs.cpu().numpy().astype(np.float64)
    m = np.zeros(op.model_shape)
    rr = -d
    s = np.zeros_like(m)
    ss = np.zeros_like(rr)
    for it in range(niter):
        g = Lt(rr)
        gg = L(g)
        if it == 0:
            alfa, beta = -np.vdot(gg, rr) / np.vdot(gg, gg), 0.0
        else:
            ggg, sss, ggs = np.vdot(gg, gg), np.vdot(ss, ss), np.vdot(gg, ss)
            det = ggg * sss * (1.0 - ggs / ggg * ggs / sss)
            ggr, ssr = -np.vdot(gg, rr), -np.vdot(ss, rr)
            alfa = (sss * ggr - ggs * ssr) / det
            beta = (-ggs * ggr + ggg * ssr) / det
        s = beta * s + alfa * g
        ss = beta * ss + alfa * gg
        m += s
        rr += ss
    assert rel(m_gpu.cpu().numpy(), m) <= 1e-3
    assert abs(res[-1] - np.vdot(rr, rr)) <= 1e-3 * res[-1]


def test_operator_orders_after_torch_stream(born, torch_cuda):
    """The operator's work runs on the handle's own stream; tensors that
    torch is still producing on its current stream must be complete before
    the operator reads them, and the operator's output must be complete for
    the torch work queued after it.  The input here is written behind a
    long device sleep on torch's stream, and the output is cloned on that
    stream right after the call."""
    torch = torch_cuda
    kw = setup_problem(seed=6, nshots=1, nt_data=40)
    op = born.BornOperator(exact=True, ckpt_interval=10, **kw)
    g = torch.Generator(device="cuda").manual_seed(77)
    m_src = torch.randn(op.model_shape, device="cuda", generator=g)
    d_src = torch.randn(op.data_shape, device="cuda", generator=g)
    want_d = torch.zeros(op.data_shape, device="cuda")
    want_m = torch.zeros(op.model_shape, device="cuda")
    op.forward(False, m_src, want_d)
    op.adjoint(False, want_m, d_src)
    want_dot = op.dot(m_src, want_m)
    torch.cuda.synchronize()
    for _ in range(2):
        m = torch.zeros(op.model_shape, device="cuda")
        d = torch.zeros(op.data_shape, device="cuda")
        torch.cuda._sleep(200_000_000)  # ~0.1 s of device time
        m.copy_(m_src)                  # still queued when forward starts
        d.copy_(d_src)
        out_d = torch.zeros(op.data_shape, device="cuda")
        op.forward(False, m, out_d)
        got_d = out_d.clone()           # torch's stream, right after
        torch.cuda._sleep(200_000_000)
        m2 = m_src * 1.0
        got_dot = op.dot(m2, want_m)
        out_m = torch.zeros(op.model_shape, device="cuda")
        op.adjoint(False, out_m, d)
        got_m = out_m.clone()
        torch.cuda.synchronize()
        assert torch.equal(got_d, want_d)
        assert torch.equal(got_m, want_m)
        assert got_dot == want_dot


def test_exact_operator_keeps_shot_checkpoints(born, torch_cuda):
    """Exact mode keeps every shot's background checkpoints across operator
    applications: after a linearised forward of all shots, the adjoint of
    each shot skips its checkpoint sweep, and gives the same model as an
    operator whose adjoint had to sweep."""
    torch = torch_cuda
    kw = setup_problem(seed=12, nshots=3)
    g = torch.Generator(device="cuda").manual_seed(1006)
    d = torch.randn(born.BornOperator(exact=True, ckpt_interval=13,
                                      **kw).data_shape,
                    device="cuda", generator=g)
    fresh = born.BornOperator(exact=True, ckpt_interval=13, **kw)
    want = torch.zeros(fresh.model_shape, device="cuda")
    fresh.adjoint(False, want, d)   # every shot sweeps
    assert fresh.checkpoints_reused == 0
    op = born.BornOperator(exact=True, ckpt_interval=13, **kw)
    m = torch.randn(op.model_shape, device="cuda", generator=g)
    out = torch.zeros(op.data_shape, device="cuda")
    op.forward(False, m, out)
    assert op.checkpoint_shots == 3
    got = torch.zeros(op.model_shape, device="cuda")
    op.adjoint(False, got, d)
    assert op.checkpoints_reused == 3
    assert torch.equal(got, want)
    op.adjoint(False, got, d)   # and again, without a forward in between
    assert op.checkpoints_reused == 6
    assert torch.equal(got, want)
