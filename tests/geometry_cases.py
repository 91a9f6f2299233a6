"""Seeded inputs for the geometry and glue helpers of the Born / RTM path,
and one runner that applies either the reference's own compiled code
(oracle/_ref/libref_geom.so: fd_prop::calc_stability,
source_func::set_compute_size, the wavelet reader and source points,
vel_fd_3d::rand_subspace, data_rtm_3d::get_source_func + map_data receiver
cells, image_rtm_3d's window, map_data, laplac, deriv) or the oracle's restatement to them, so that
the two can be compared bit for bit (tests/test_oracle_golden.py) and the
reference's outputs stored as fixtures (tests/golden/make_golden.py)."""
import ctypes as C

import numpy as np

# fixed geometry of the cases
SRC_GRID = dict(n=(48, 40, 36), o=(-120.0, -80.0, -90.0), d=(10.0, 10.0, 10.0),
                nts=96, dt_wav=0.001)
VEL_AXES = dict(o=(0.0, 0.0, 0.0), d=(10.0, 10.0, 10.0))
RAND_GRID = dict(n=(36, 30, 26), o=(-90.0, -80.0, -70.0), d=(10.0, 10.0, 10.0),
                 dt=0.001, irand=1234)
REC_GRID = dict(n=(64, 56, 40), o=(-60.0, -60.0, -60.0), d=(10.0, 10.0, 10.0),
                nt=50)
OP_SHAPE = (9, 7, 11)             # n3, n2, n1 for laplac / deriv
MAP_SHAPE = dict(nt=20, ntb=28, n2=5, n3=3)
DERIV_D1 = 0.002
WIN_WHOLE = (12, 10, 9)          # n1, n2, n3 of the whole image


def window_cases():
    """(whole origins, whole spacings, window sizes, window origins): a
    window around the image, inside it, over its far edge, and three on
    origins that are not multiples of the spacing (float truncation toward
    zero, on both sides)."""
    f32 = np.float32
    wo, wd = (0.0, 0.0, 0.0), (10.0, 10.0, 10.0)
    oo = tuple(f32(x) for x in (13.7, -2.3, 0.1))
    od = tuple(f32(x) for x in (7.3, 6.1, 9.7))
    return [
        (wo, wd, (16, 14, 13), (-20.0, -20.0, -20.0)),
        (wo, wd, (5, 4, 3), (30.0, 20.0, 10.0)),
        (wo, wd, (6, 5, 4), (90.0, 70.0, 60.0)),
        (oo, od, (14, 12, 11), tuple(o - f32(2) * d for o, d in zip(oo, od))),
        (oo, od, (5, 4, 3), tuple(o + f32(3.5) * d for o, d in zip(oo, od))),
        (oo, od, (6, 5, 5), tuple(o - f32(3.5) * d for o, d in zip(oo, od))),
    ]


def make_inputs(seed: int = 0) -> dict:
    rng = np.random.default_rng(seed)
    return {
        "cs": np.array([(n, b, fa) for n in (17, 64, 100, 128, 255, 256, 512)
                        for b in (0, 6, 20, 50) for fa in (0, 4)], np.int32),
        "wav_raw": rng.standard_normal(80).astype(np.float32),
        "src_pos": np.array([(253.3, 141.7, 20.0), (100.0, 100.0, 35.5),
                             (0.0, 0.0, 10.0),
                             tuple(rng.uniform(0, 300, 3))], np.float32),
        "vel": (1500 + 2000 * rng.random((26, 28, 30))).astype(np.float32),
        "op_m": rng.standard_normal(OP_SHAPE).astype(np.float32),
        "op_d": rng.standard_normal(OP_SHAPE).astype(np.float32),
        "map_m": rng.standard_normal(
            (MAP_SHAPE["n3"], MAP_SHAPE["n2"], MAP_SHAPE["ntb"])).astype(
                np.float32),
        "map_d": rng.standard_normal(
            (MAP_SHAPE["n3"], MAP_SHAPE["n2"], MAP_SHAPE["nt"])).astype(
                np.float32),
        "win_whole": rng.standard_normal(WIN_WHOLE[::-1]).astype(np.float32),
        "win_sub": [rng.standard_normal(c[2][::-1]).astype(np.float32)
                    for c in window_cases()],
        "rec_cfg": np.array([(16, 12, 40.0, 20.0, 30.0, 20.0, 10.0),
                             (7, 9, 13.7, 7.3, 21.1, 11.9, 14.2)], np.float32),
        "stab_cfg": np.array([(4500.0, 10.0, 0.001, 2000),
                              (4500.0, 8.0, 0.001, 1500),
                              (3000.0, 5.0, 0.002, 700),
                              (4120.0, 10.0, 0.001, 1000)], np.float64),
    }


def run(inp: dict, po, ref: bool) -> dict:
    """Outputs of the reference's compiled code (ref=True) or of the
    oracle's restatement on the inputs of make_inputs()."""
    R = po.ref_geom_lib() if ref else None
    L = po.port_lib()
    f, i = po.fptr, po.iptr
    out = {}
    out["compute_size"] = np.array(
        [(R.ref_geom_compute_size if ref else L.oracle_compute_size)(*map(
            int, row)) for row in inp["cs"]], np.int32)

    # wavelet derivative and source points of each shot
    raw = np.ascontiguousarray(inp["wav_raw"])
    g = SRC_GRID
    wd = np.zeros_like(raw)
    L.oracle_wavelet_deriv(f(raw), raw.size, g["dt_wav"], f(wd))
    locs, vals = [], []
    for sx, sy, sz in inp["src_pos"].astype(float):
        lo = np.zeros(9, np.int32)
        va = np.zeros(9 * g["nts"], np.float32)
        if ref:
            R.ref_geom_source(f(raw), raw.size, g["dt_wav"], sx, sy, sz,
                              *g["o"], *g["d"], *g["n"], g["nts"], i(lo),
                              f(va))
        else:
            L.oracle_source_geometry(sx, sy, sz, *g["o"], *g["d"], g["n"][0],
                                     g["n"][1], f(wd), raw.size, g["nts"],
                                     i(lo), f(va))
        locs.append(lo)
        vals.append(va)
    out["src_locs"], out["src_vals"] = np.stack(locs), np.stack(vals)

    # random boundary (and without one) of the velocity on a compute grid
    vel = np.ascontiguousarray(inp["vel"])
    vn3, vn2, vn1 = vel.shape
    r = RAND_GRID
    for tag, nr in (("rand_band", 8), ("rand_none", 0)):
        o = np.zeros(r["n"][::-1], np.float32)
        va = (vn1, vn2, vn3, *VEL_AXES["o"], *VEL_AXES["d"])
        if ref:
            R.ref_geom_rand_subspace(f(vel), *va, r["irand"], nr, nr, nr,
                                     r["dt"], *r["n"], *r["o"], *r["d"], f(o))
        else:
            L.oracle_rand_subspace(f(vel), *va, float(vel.max()), r["irand"],
                                   nr, nr, nr, r["dt"], *r["n"], *r["o"],
                                   *r["d"], f(o))
        out[tag] = o

    # receiver cells
    rg = REC_GRID
    for k, row in enumerate(inp["rec_cfg"]):
        rnx, rny = int(row[0]), int(row[1])
        rest = [float(x) for x in row[2:]]
        lo = np.zeros(rnx * rny, np.int32)
        if ref:
            R.ref_geom_receivers(rnx, rny, *rest, *rg["o"], *rg["d"],
                                 *rg["n"], rg["nt"], i(lo))
        else:
            L.oracle_receiver_geometry(rnx, rny, *rest, *rg["o"], *rg["d"],
                                       rg["n"][0], rg["n"][1], i(lo))
        out[f"rec_locs_{k}"] = lo

    # FD time step and step count
    stab = []
    for vmax, dv, dtd, ntd in inp["stab_cfg"]:
        if ref:
            v = np.full((6, 5, 4), 1500.0, np.float32)
            v[2, 2, 2] = vmax
            dt = np.zeros(1, np.float32)
            nt = np.zeros(1, np.int32)
            R.ref_geom_calc_stability(f(v), 4, 5, 6, dv, dv, dv, dtd,
                                      int(ntd), f(dt), i(nt))
            stab.append((float(dt[0]), int(nt[0])))
        else:
            nt = C.c_int()
            dt = L.oracle_calc_stability(float(vmax), float(dv), float(dtd),
                                         int(ntd), C.byref(nt))
            stab.append((float(np.float32(dt)), nt.value))
    out["stability"] = np.array(stab, np.float64)

    # image window: extract_sub and add_image with offsets from the axes
    w1, w2, w3 = WIN_WHOLE
    for k, (wo, wd, sn, so) in enumerate(window_cases()):
        wo, wd, so = ([float(x) for x in t] for t in (wo, wd, so))
        for extract in (1, 0):
            whole = inp["win_whole"].copy()
            sub = (np.zeros(sn[::-1], np.float32) if extract
                   else inp["win_sub"][k].copy())
            if ref:
                R.ref_geom_image_window(extract, f(whole), w1, w2, w3, *wo,
                                        *wd, f(sub), *sn, *so, *wd)
            else:
                off = [L.oracle_window_offset(so[a], wo[a], wd[a])
                       for a in range(3)]
                if extract:
                    L.oracle_extract_sub(f(whole), w1, w2, w3, f(sub), *sn,
                                         *off)
                else:
                    L.oracle_add_image(f(whole), w1, w2, w3, f(sub), *sn,
                                       *off)
            out[f"win_{'ext' if extract else 'add'}_{k}"] = \
                sub if extract else whole

    # the linear glue: laplac, deriv, map_data (forward and adjoint, with and
    # without accumulation)
    n3, n2, n1 = OP_SHAPE
    ms = MAP_SHAPE
    for name in ("laplac", "deriv", "map"):
        for adj in (0, 1):
            for add in (0, 1):
                if name == "map":
                    m = inp["map_m"].copy()
                    d = inp["map_d"].copy()
                else:
                    m = inp["op_m"].copy()
                    d = inp["op_d"].copy()
                if ref:
                    if name == "laplac":
                        R.ref_geom_laplac(adj, add, f(m), f(d), n1, n2, n3)
                    elif name == "deriv":
                        R.ref_geom_deriv(adj, add, f(m), f(d), n1, n2, n3,
                                         DERIV_D1)
                    else:
                        R.ref_geom_map_data(adj, add, f(m), f(d), ms["nt"],
                                            ms["n2"], ms["n3"], ms["ntb"])
                else:
                    if name == "laplac":
                        fn = L.oracle_laplac_adjoint if adj else \
                            L.oracle_laplac_forward
                        fn(add, f(m), f(d), n1, n2, n3)
                    elif name == "deriv":
                        fn = L.oracle_deriv_adjoint if adj else \
                            L.oracle_deriv_forward
                        fn(add, f(m), f(d), n1, n2, n3, DERIV_D1)
                    else:
                        fn = L.oracle_map_data_adjoint if adj else \
                            L.oracle_map_data_forward
                        fn(add, f(m), f(d), ms["nt"], ms["n2"], ms["n3"],
                           ms["ntb"])
                out[f"{name}_{'adj' if adj else 'fwd'}_{add}"] = \
                    m if adj else d
    return out
