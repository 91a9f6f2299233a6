"""Study (test infrastructure, not part of the library): 16-bit level
storage forms on the random-boundary RTM (source propagation + adjoint,
cpu_prop.cc:56-129), emulated on the oracle's float primitives, with the
image error against the FP64 oracle.  Forms per field: f32; p16 (each stored
level rounded to FP16 with a power-of-two scale, as BORN_STORE_F16 stores
it); pq16 and qp16 (the level and its difference to the current level,
each 16-bit with its own scale, the previous level rebuilt as P - Q; pq16
takes the difference from the rounded new level, qp16 from the new level
before rounding).  With f32 for both fields the emulation reproduces the
oracle's image bit for bit.  STUDY_FORMS="s/r,..." (e.g. "f32/qp16")
limits the runs to some (source field, receiver field) forms.

    python tests/storage_forms_study.py <model n> <data samples> [born]

"born" migrates the shot's own Born traces (band-limited) instead of the
seeded white-noise traces of the benchmark cases."""
import ctypes as C
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import importlib.util  # noqa: E402

import pyoracle as po  # noqa: E402

spec = importlib.util.spec_from_file_location(
    "wl", os.path.join(ROOT, "sc17-born_gb300", "workload.py"))
wl = importlib.util.module_from_spec(spec)
spec.loader.exec_module(wl)

L = po.port_lib()
P = C.POINTER(po._PropF)
fp = C.POINTER(C.c_float)
L.oracle_inject_sourcef.argtypes = [P, C.c_int, C.c_int, fp]
L.oracle_inject_receiversf.argtypes = [P, C.c_int, C.c_int, fp]
f = lambda a: a.ctypes.data_as(fp)  # noqa: E731


def q16(x):
    m = float(np.max(np.abs(x)))
    if m == 0.0 or not np.isfinite(m):
        return x.copy()
    e = int(np.ceil(np.log2(m))) - 15
    S = np.float32(2.0 ** e)
    return (x / S).astype(np.float16).astype(np.float32) * S


class Field:
    """Two time levels of one field under a storage form."""

    def __init__(self, n, form):
        self.form = form
        self.p0 = np.zeros(n, np.float32)  # old (to be overwritten by new)
        self.p1 = np.zeros(n, np.float32)  # cur
        self.Q = np.zeros(n, np.float32)   # stored difference (pq16)

    def before_step(self):
        # the levels the step reads: cur = p1 as stored, old = p0 or P - Q
        if self.form in ("pq16", "qp16"):
            self.p0[:] = self.p1 - self.Q

    def after_step(self):
        # p0 holds the new level (FP32, after taper and injection), p1 the
        # current level as the step left it (tapered in place where the
        # reference tapers it)
        if self.form == "p16":
            self.p0[:] = q16(self.p0)
        elif self.form == "pq16":
            # the difference of the stored levels (the previous level is
            # rebuilt exactly as P - Q up to Q's rounding)
            newP = q16(self.p0)
            self.Q = q16(newP - self.p1)
            self.p0[:] = newP
        elif self.form == "qp16":
            # the difference of the new level before rounding and the stored
            # current one (the time derivative keeps no level rounding)
            self.Q = q16(self.p0 - self.p1)
            self.p0[:] = q16(self.p0)
        self.p0, self.p1 = self.p1, self.p0


def run(case, form_s, form_r):
    nz, ny, nx = case["shape"]
    n = nx * ny * nz
    pr = po.PortProp()
    pr.createSpace(case["d"], case["d"], case["d"], 50, .0005, .0005, nx, ny, nz)
    pr.transferSincTableS(8, case["jts"], case["table_s"])
    pr.transferSincTableD(8, case["jtd"], case["table_d"])
    pr.transferSourceFunc(9, case["nt_big"], case["locs_s"], case["src"])
    v1 = np.ascontiguousarray(case["vel1"], np.float32).reshape(-1)
    v2 = np.ascontiguousarray(case["vel2"], np.float32).reshape(-1)
    pr.transferVelFunc1(nx, ny, nz, v1)
    pr.transferVelFunc2(nx, ny, nz, v2)
    rec = np.ascontiguousarray(case["rec_in"], np.float32)
    pr.transferReceiverFunc(case["rec_nx"], case["rec_ny"], case["nt_big"],
                            case["locs_r"], rec)
    s = pr.s
    nt = case["nt"]
    # sourceProp (cpu_prop.cc:106-129)
    S = Field(n, form_s)
    s.jt = case["jts"]
    s.dir = 1
    for it in range(nt + 1):
        idd, ii = it // s.jt_s, it % s.jt_s
        S.before_step()
        L.oracle_prop_stepf(C.byref(s), f(S.p0), f(S.p1), f(v1))
        L.oracle_inject_sourcef(C.byref(s), idd, ii, f(S.p0))
        S.after_step()
    if nt % 2 == 1:
        # cpu_prop.cc:123-128: memcpy(p1, p0) after the last swap, so both
        # levels hold the level before the last
        S.p1[:] = S.p0
        if form_s in ("pq16", "qp16"):
            S.Q[:] = 0.0
    # rtmAdjoint (cpu_prop.cc:56-96) with rtm_zero_op's argument order:
    # src_p0 (the buffer a step overwrites) = the level before the last,
    # src_p1 = the last level; the first step (it = nt - 1) does not
    # propagate s, the swap after it makes the last level "old" and the one
    # before it "current": time runs backwards
    Sa = Field(n, form_s)
    Sa.p0 = S.p0.copy()
    Sa.p1 = S.p1.copy()
    R = Field(n, form_r)
    img = np.zeros(n, np.float32)
    s.dir = -1
    for it in range(nt - 1, -1, -1):
        id_s, i_s = (it + 1) // s.jt_s, (it + 1) % s.jt_s
        idd, ii = it // s.jt_d, it % s.jt_d
        R.before_step()
        if it > 0:
            L.oracle_prop_stepf(C.byref(s), f(R.p0), f(R.p1), f(v2))
        if it < nt - 1:
            Sa.before_step()
            L.oracle_prop_stepf(C.byref(s), f(Sa.p0), f(Sa.p1), f(v1))
            L.oracle_inject_sourcef(C.byref(s), id_s, i_s, f(Sa.p1))
        L.oracle_dampf(C.byref(s), f(R.p0), f(R.p1))
        L.oracle_inject_receiversf(C.byref(s), idd, ii, f(R.p0))
        L.oracle_image_conditionf(C.byref(s), f(R.p0), f(Sa.p0), f(img))
        R.after_step()
        if it < nt - 1:
            Sa.after_step()
        else:
            Sa.p0, Sa.p1 = Sa.p1, Sa.p0
            if form_s in ("pq16", "qp16"):
                Sa.Q = q16(Sa.p1 - Sa.p0)
    return img


if __name__ == "__main__":
    n_model = int(sys.argv[1]) if len(sys.argv) > 1 else 48
    nt = int(sys.argv[2]) if len(sys.argv) > 2 else 600
    po.set_threads(os.cpu_count() or 1)
    case = wl.prepare_shot(po.Geometry(), "c3", nt=nt, n=n_model)
    print("grid", case["shape"], "nt", case["nt"], "jt", case["jts"],
          flush=True)
    if len(sys.argv) > 3 and sys.argv[3] == "born":
        # band-limited data: the shot's own Born traces (FP32 oracle)
        tr = po.run_case(po.PortProp(), case, which="forward")["traces"]
        case["rec_in"] = np.ascontiguousarray(tr, np.float32)
        print("data: Born traces of the shot", flush=True)
    else:
        print("data: seeded white noise (the bench's synthetic traces)",
              flush=True)
    ref = po.run_case(po.PortProp64(), case, which="adjoint")["image"]
    ref32 = po.run_case(po.PortProp(), case, which="adjoint")["image"]
    nrm = np.linalg.norm(ref)
    print("oracle f32 vs f64", np.linalg.norm(ref32 - ref) / nrm, flush=True)
    forms = (("f32", "f32"), ("p16", "p16"), ("f32", "p16"),
             ("f32", "pq16"), ("pq16", "pq16"), ("f32", "qp16"),
             ("qp16", "qp16"), ("qp16", "f32"))
    if os.environ.get("STUDY_FORMS"):
        forms = [tuple(x.split("/")) for x in
                 os.environ["STUDY_FORMS"].split(",")]
    for fs, fr in forms:
        t0 = time.time()
        img = run(case, fs, fr).reshape(ref.shape)
        print(f"s {fs:5s} r {fr:5s}: image rel L2 vs f64 "
              f"{np.linalg.norm(img - ref) / nrm:.3e}  "
              f"({time.time() - t0:.0f} s)", flush=True)
