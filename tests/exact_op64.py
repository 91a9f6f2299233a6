"""FP64 restatement of the Born operator's exact mode (born_op with exact = 1)
for least-squares checks -- test infrastructure.

Per shot (rtm_zero_op_3d.cc:101-299 in order, the propagation replaced by
the exact linearised pair):
  forward:  m -> window (image_rtm_3d.cc:53-95) -> laplac (laplac_3d.cc:51-105)
               -> oracle_lin_forwardd -> map_data (map_data_3d.cc:57-75)
               -> deriv (deriv_3d.cc:31-56) -> data
  adjoint:  the transpose of every stage, oracle_lin_adjointd for the pair.
The geometry (compute grid, FD step, sinc table, source and receiver cells,
wavelet derivative, v^2 dt^2) comes from the oracle's restatement of the
reference's helpers, as tests/test_operator.py's oracle chain makes it; the
arrays are promoted to double and every operation below is FP64.
"""
from __future__ import annotations

import ctypes as C

import numpy as np


class ExactOperator64:
    def __init__(self, po, kw):
        L = po.port_lib()
        vel = np.ascontiguousarray(kw["velocity"], np.float32)
        self.model_shape = vel.shape
        n3, n2, n1 = vel.shape
        d = kw["d"][0]
        nb = kw["nbound"]
        nt_c = C.c_int()
        dt = L.oracle_calc_stability(float(vel.max()), d, kw["dt_data"],
                                     kw["nt_data"], C.byref(nt_c))
        self.nt = nt_c.value
        self.jt = int(np.float32(kw["dt_data"]) / np.float32(dt))
        nc = [L.oracle_compute_size(m, nb, 4) for m in (n1, n2, n3)]
        self.shape_c = (nc[2], nc[1], nc[0])
        f = nb + 4
        oc = float(np.float32(0) + np.float32(-d) * np.float32(f))
        self.w = L.oracle_window_offset(oc, 0.0, d)
        tab = po.sinc_table(self.jt)
        wav = np.ascontiguousarray(kw["wavelet"], np.float32)
        wd = np.zeros_like(wav)
        L.oracle_wavelet_deriv(po.fptr(wav), wav.size, kw["dt_wavelet"],
                               po.fptr(wd))
        self.rnx, self.rny = kw["rec_n"]
        locs_r = np.zeros(self.rnx * self.rny, np.int32)
        L.oracle_receiver_geometry(self.rnx, self.rny, kw["rec_o"][0],
                                   kw["rec_d"][0], kw["rec_o"][1],
                                   kw["rec_d"][1], kw["rec_depth"], oc, oc,
                                   oc, d, d, d, nc[0], nc[1],
                                   po.iptr(locs_r))
        self.nt_data, self.nt_big = kw["nt_data"], kw["nt_data"] + 8
        self.dt_data = np.float64(np.float32(kw["dt_data"]))
        self.data_shape = (len(kw["shots"]), self.rny, self.rnx, self.nt_data)
        self.props = []
        for sx, sy, sz in kw["shots"]:
            locs_s = np.zeros(9, np.int32)
            vals = np.zeros((9, self.nt_big), np.float32)
            L.oracle_source_geometry(float(sx), float(sy), float(sz), oc, oc,
                                     oc, d, d, d, nc[0], nc[1], po.fptr(wd),
                                     wd.size, self.nt_big, po.iptr(locs_s),
                                     po.fptr(vals))
            seed = int(locs_s[3] % 10000)
            vn = np.zeros(self.shape_c, np.float32)
            L.oracle_rand_subspace(po.fptr(vel), n1, n2, n3, 0., 0., 0., d, d,
                                   d, float(vel.max()), seed, 0, 0, 0, dt,
                                   nc[0], nc[1], nc[2], oc, oc, oc, d, d, d,
                                   po.fptr(vn))
            p = po.PortProp64()
            p.createSpace(d, d, d, 50, .0005, .0005, nc[0], nc[1], nc[2])
            p.transferSincTableS(8, self.jt, tab)
            p.transferSincTableD(8, self.jt, tab)
            p.transferSourceFunc(9, self.nt_big, locs_s, vals)
            p.transferVelFunc1(nc[0], nc[1], nc[2], vn)
            p.transferVelFunc2(nc[0], nc[1], nc[2], vn)
            rec = np.zeros((self.rnx * self.rny, self.nt_big))
            p.transferReceiverFunc(self.rnx, self.rny, self.nt_big, locs_r,
                                   rec)
            self.props.append(p)

    # ---- glue, FP64 ----
    def _window(self, m):
        """model grid -> compute grid, first compute cell at model sample w"""
        out = np.zeros(self.shape_c)
        sl_c, sl_m = [], []
        for nm, ncell in zip(self.model_shape, self.shape_c):
            lo = max(0, self.w)
            hi = min(nm, self.w + ncell)
            sl_m.append(slice(lo, hi))
            sl_c.append(slice(lo - self.w, hi - self.w))
        out[tuple(sl_c)] = m[tuple(sl_m)]
        return out, tuple(sl_c), tuple(sl_m)

    def _window_adj(self, x):
        out = np.zeros(self.model_shape)
        _, sl_c, sl_m = self._window(out)
        out[sl_m] = x[sl_c]
        return out

    @staticmethod
    def _laplac(m):
        d = np.zeros_like(m)
        d[1:] += m[:-1]
        d[:-1] -= m[:-1]
        return d

    @staticmethod
    def _laplac_adj(d):
        m = np.zeros_like(d)
        m[:-1] = d[1:] - d[:-1]
        return m

    def _deriv(self, tr):
        """deriv_3d.cc:31-56 on traces [rny][rnx][nt], with the reference's
        repeated first-sample term (twice on the first trace of each row)"""
        q = tr / self.dt_data
        out = np.zeros_like(tr)
        out[..., :-1] -= q[..., :-1]
        out[..., 1:] += q[..., :-1]
        heads = np.ones(tr.shape[:-1])
        heads[:, 0] = 2.0
        out[..., 1] += heads * q[..., 0]
        out[..., 0] -= heads * q[..., 0]
        return out

    def _deriv_adj(self, d):
        out = np.zeros_like(d)
        diff = (d[..., 1:] - d[..., :-1]) / self.dt_data
        out[..., :-1] += diff
        heads = np.ones(d.shape[:-1])
        heads[:, 0] = 2.0
        out[..., 0] += heads * diff[..., 0]
        return out

    def forward(self, m):
        m = np.asarray(m, np.float64)
        lap = self._laplac(self._window(m)[0])
        data = np.zeros(self.data_shape)
        for s, p in enumerate(self.props):
            rec = np.zeros((self.rnx * self.rny, self.nt_big))
            p.transferReceiverFunc(self.rnx, self.rny, self.nt_big,
                                   p._keep["lr"], rec)
            p.lin_forward(self.jt, lap, rec, self.nt)
            tr = rec[:, 4:4 + self.nt_data].reshape(self.rny, self.rnx,
                                                    self.nt_data)
            data[s] = self._deriv(tr)
        return data

    def adjoint(self, data):
        data = np.asarray(data, np.float64)
        img = np.zeros(self.shape_c)
        for s, p in enumerate(self.props):
            tr = self._deriv_adj(data[s]).reshape(self.rnx * self.rny,
                                                  self.nt_data)
            rec = np.zeros((self.rnx * self.rny, self.nt_big))
            rec[:, 4:4 + self.nt_data] = tr
            img += p.lin_adjoint(self.jt, rec, self.nt)
        return self._window_adj(self._laplac_adj(img))


def cgstep_solve(op_fwd, op_adj, data, niter, m0=None):
    """Claerbout's CG (lin_solver.cc:104-132, cgstep.cc:11-54) in FP64:
    returns the model and rr.rr before and after every iteration."""
    m = np.zeros_like(op_adj(np.zeros_like(data))) if m0 is None else m0.copy()
    rr = -np.asarray(data, np.float64) + (op_fwd(m) if m0 is not None else 0)
    s = np.zeros_like(m)
    ss = np.zeros_like(rr)
    res = [float(np.vdot(rr, rr))]
    for it in range(niter):
        g = op_adj(rr)
        gg = op_fwd(g)
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
        res.append(float(np.vdot(rr, rr)))
    return m, res
