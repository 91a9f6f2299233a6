"""Seeded synthetic shots for the benchmark and the larger tests.

The reference names no public dataset; these generators stand in with the
shapes, sizes and value ranges of the benchmark configurations:

* ``c1``: 128^3 model at 10 m, 20-cell boundary -> 176^3 compute grid,
  nt = 1000, 15 Hz Ricker, 6 flat layers 1500..4000 m/s with a seeded
  +-3 % smooth perturbation, 64 x 64 receivers at 20 m, 10 m deep.
* ``c2``: 256^3 model at 10 m, 50-cell boundary -> 368^3, nt = 2000,
  12 Hz Ricker, layered 1500..4500 m/s with a dipping interface and a
  Gaussian salt-like blob at 4500 m/s, 128 x 128 receivers at 20 m.

``prepare_shot`` turns a model into the propagator inputs exactly as the
reference's operator does per shot (rtm_zero_op_3d.cc:139-185 and
:243-273): compute grid and origin, sinc tables, 9-point source with the
wavelet's time derivative, receiver cells, random-boundary and plain v^2 dt^2
models, and the reflectivity after the z first difference.  The geometry
comes from ``geo``, any object with the host-geometry functions of this
package (``calc_stability``, ``compute_size``, ``sinc_table``,
``wavelet_deriv``, ``source_geometry``, ``receiver_geometry``,
``rand_subspace``, ``extract_sub``, ``laplac_forward``): the package itself,
or a CPU restatement with the same functions, which gives bit-identical
arrays.  This module itself is plain numpy.
"""
from __future__ import annotations

import numpy as np

SEEDS = dict(velocity=1001, reflectivity=1002, data=1004, jitter=1006,
             aperture=1007)


def ricker(nt: int, dt: float, f: float, t0: float = 0.064) -> np.ndarray:
    """util/Wavelet.cc:23-29."""
    t = -t0 + np.arange(nt) * dt
    a = (np.pi * f * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def _smooth3(a, sigma_cells):
    # separable Gaussian via FFT along each axis
    out = a
    for ax in range(3):
        n = out.shape[ax]
        k = np.fft.rfftfreq(n)
        g = np.exp(-0.5 * (2 * np.pi * k * sigma_cells) ** 2)
        shape = [1, 1, 1]
        shape[ax] = g.size
        out = np.fft.irfft(np.fft.rfft(out, axis=ax) * g.reshape(shape), n=n,
                           axis=ax)
    return out


def model_c1(n=128, seed=SEEDS["velocity"]):
    rng = np.random.default_rng(seed)
    z = np.arange(n)
    layer = np.minimum(z * 6 // n, 5)
    v = (1500.0 + 500.0 * layer)[:, None, None] * np.ones((n, n, n))
    dv = _smooth3(rng.standard_normal((n, n, n)), 4.0)
    v *= 1 + 0.03 * dv / np.abs(dv).max()
    return v.astype(np.float32)


def model_c2(n=256, seed=SEEDS["velocity"]):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n),
                          indexing="ij")
    v = 1500.0 + 2500.0 * z / (n - 1)
    dip = np.tan(np.deg2rad(rng.uniform(5, 15)))
    v = np.where(z > 0.55 * n + dip * (x - n / 2), v + 400.0, v)
    c = np.array([0.6, 0.5, 0.45]) * n
    r2 = ((z - c[0]) ** 2 + (y - c[1]) ** 2 + (x - c[2]) ** 2) / (0.1 * n) ** 2
    blob = np.exp(-r2)
    v = v * (1 - blob) + 4500.0 * blob
    return np.clip(v, 1500.0, 4500.0).astype(np.float32)


def reflectivity(v, seed=SEEDS["reflectivity"]):
    """dv/dz normalised to 1, plus seeded sparse +-0.05 spikes."""
    rng = np.random.default_rng(seed)
    r = np.zeros_like(v)
    r[1:] = v[1:] - v[:-1]
    r /= max(np.abs(r).max(), 1e-30)
    mask = rng.random(v.shape) < 1e-3
    r[mask] += rng.choice([-0.05, 0.05], size=int(mask.sum()))
    return r.astype(np.float32)


CONFIGS = {
    "c1": dict(n=128, d=10.0, nbound=20, nt=1000, f=15.0, model=model_c1,
               rec=(64, 20.0), src_depth=20.0, rec_depth=10.0),
    "c2": dict(n=256, d=10.0, nbound=50, nt=2000, f=12.0, model=model_c2,
               rec=(128, 20.0), src_depth=20.0, rec_depth=10.0),
    # 512^3 at 8 m: FD dt 0.5 ms against data dt 1 ms (jt = 2), so 1500
    # data samples make 2999 FD steps
    "c3": dict(n=512, d=8.0, nbound=50, nt=1500, f=20.0, model=model_c2,
               rec=(128, 16.0), src_depth=16.0, rec_depth=8.0),
}


def prepare_shot(geo, name: str = "c2", nt: int | None = None,
                 n: int | None = None, nbound: int | None = None,
                 shot: int = 0) -> dict:
    """Propagator inputs for shot ``shot`` of configuration ``name`` (shot 0
    at the model centre, others offset along x on a 20 m lattice); ``geo``
    provides the host geometry (see the module docstring)."""
    cfg = dict(CONFIGS[name])
    if n is not None:
        cfg["n"] = n
    if nbound is not None:
        cfg["nbound"] = nbound
    n, d, nb = cfg["n"], cfg["d"], cfg["nbound"]
    vel = cfg["model"](n)
    dt_data = 0.001
    nt_data = nt if nt is not None else cfg["nt"]
    dt, nt_fd = geo.calc_stability(float(vel.max()), d, dt_data, nt_data)
    jt = int(round(dt_data / dt))
    fat = 4
    nc = geo.compute_size(n, nb, fat)
    o_c = -d * (nb + fat)
    o = (o_c, o_c, o_c)
    dd = (d, d, d)
    table = geo.sinc_table(jt, 8)
    nt_big = nt_data + 8
    wav = geo.wavelet_deriv(ricker(nt_data, dt_data, cfg["f"]), dt_data)
    mid = (n // 2) * d
    sx = mid + 20.0 * (((shot * 7) % 11) - 5 if shot else 0)
    locs_s, src = geo.source_geometry(sx, mid, cfg["src_depth"], o, dd, nc,
                                      nc, wav, nt_big)
    seed = int(locs_s[3] % 10000)
    shape = (nc, nc, nc)
    vrand = geo.rand_subspace(vel, (0., 0., 0.), dd, float(vel.max()), seed,
                              (nb, nb, nb), dt, shape, o, dd)
    vnone = geo.rand_subspace(vel, (0., 0., 0.), dd, float(vel.max()), seed,
                              (0, 0, 0), dt, shape, o, dd)
    nr, dr = cfg["rec"]
    r0 = mid - dr * (nr // 2)
    locs_r = geo.receiver_geometry(nr, nr, r0, dr, r0, dr, cfg["rec_depth"],
                                   o, dd, nc, nc)
    rng = np.random.default_rng(SEEDS["data"])
    rec = np.zeros((nr * nr, nt_big), np.float32)
    rec[:, 4:4 + nt_data] = 1e-3 * rng.standard_normal((nr * nr, nt_data))
    # model-grid reflectivity -> compute-grid window -> z first difference
    sub = geo.extract_sub(reflectivity(vel), shape, (-(nb + fat),) * 3)
    refl = geo.laplac_forward(sub)
    return dict(shape=shape, d=d, nt=nt_fd, jts=jt, jtd=jt, nt_big=nt_big,
                table_s=table, table_d=table, locs_s=locs_s, src=src,
                vel1=vrand, vel2=vnone, locs_r=locs_r, rec_nx=nr, rec_ny=nr,
                rec_in=rec, refl=refl, name=name, model_n=n, nbound=nb)


def interior_cells(shape) -> int:
    nz, ny, nx = shape
    return (nx - 8) * (ny - 8) * (nz - 8)


# ---------------------------------------------------------------------------
# c4: batched multi-shot RTM on a large model with uneven shot apertures

def model_c4(nx=800, ny=800, nz=400, seed=SEEDS["velocity"]):
    """Layered 1500..4500 m/s with a dipping interface and a Gaussian blob,
    built by broadcasting (no full-size index grids)."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz, dtype=np.float32)[:, None, None]
    y = np.arange(ny, dtype=np.float32)[None, :, None]
    x = np.arange(nx, dtype=np.float32)[None, None, :]
    dip = np.float32(np.tan(np.deg2rad(rng.uniform(5, 15))))
    v = np.empty((nz, ny, nx), np.float32)
    v[...] = 1500.0 + 2500.0 * z / (nz - 1)
    v += np.where(z > 0.55 * nz + dip * (x - nx / 2), np.float32(400.0),
                  np.float32(0.0))
    r2 = ((z - 0.6 * nz) ** 2 / (0.1 * nz) ** 2 +
          ((y - 0.5 * ny) ** 2 + (x - 0.45 * nx) ** 2) / (0.08 * nx) ** 2)
    blob = np.exp(-r2).astype(np.float32)
    v = v * (1 - blob) + 4500.0 * blob
    np.clip(v, 1500.0, 4500.0, out=v)
    return v


def c4_shots(nx=800, ny=800, d=10.0, gx=8, gy=6):
    """Jittered 8 x 6 surface grid (+-25 % of the spacing) and per-shot
    aperture sizes uniform in 192..320 (x, y) and 256..400 (z) cells,
    rounded to 16."""
    rj = np.random.default_rng(SEEDS["jitter"])
    ra = np.random.default_rng(SEEDS["aperture"])
    sx, sy = nx * d / gx, ny * d / gy
    shots = []
    for j in range(gy):
        for i in range(gx):
            x = (i + 0.5) * sx + rj.uniform(-0.25, 0.25) * sx
            y = (j + 0.5) * sy + rj.uniform(-0.25, 0.25) * sy
            ax = int(ra.integers(192, 321)) // 16 * 16
            ay = int(ra.integers(192, 321)) // 16 * 16
            az = int(ra.integers(256, 401)) // 16 * 16
            shots.append((x, y, ax, ay, az))
    return shots


def prepare_batch_c4(born, nshots=48, nt=2500, nbound=40, f=15.0,
                     model=None, device=0):
    """Set-up shot handles for c4: each shot's compute grid is its aperture
    centred on the source, velocities made on the device (random boundary
    from counter-based draws), receivers every 25 m inside the aperture, data
    traces seeded noise.  Returns (handles, common dict)."""
    d = 10.0
    vel = model_c4() if model is None else model
    nz_m, ny_m, nx_m = vel.shape
    vmax = float(vel.max())
    dt_data = 0.001
    dt, nt_fd = born.calc_stability(vmax, d, dt_data, nt)
    jt = int(round(dt_data / dt))
    table = born.sinc_table(jt, 8)
    nt_big = nt + 8
    wav = born.wavelet_deriv(ricker(nt, dt_data, f), dt_data)
    rng = np.random.default_rng(SEEDS["data"])
    handles = []
    for k, (sx, sy, ax, ay, az) in enumerate(c4_shots()[:nshots]):
        n1, n2, n3 = ax, ay, az
        o = (sx - d * (n1 // 2), sy - d * (n2 // 2), -d * (nbound + 4))
        h = born.Gb300Prop(device)
        h.createSpace(d, d, d, 50.0, 0.0005, 0.0005, n1, n2, n3)
        h.transferSincTableS(8, jt, table)
        h.transferSincTableD(8, jt, table)
        locs_s, src = born.source_geometry(sx, sy, 20.0, o, (d, d, d), n1, n2,
                                           wav, nt_big)
        h.transferSourceFunc(9, nt_big, locs_s, src)
        # the model window the aperture covers (indices clamped as the
        # reference's resampling does)
        i0 = int(np.clip(np.floor(o[0] / d), 0, nx_m - 1))
        j0 = int(np.clip(np.floor(o[1] / d), 0, ny_m - 1))
        sub = vel[:, j0:min(ny_m, j0 + n2), i0:min(nx_m, i0 + n1)]
        sub = np.ascontiguousarray(sub)
        vo = (i0 * d, j0 * d, 0.0)
        seed = int(locs_s[3] % 10000)
        h.make_velocity(1, sub, vo, (d, d, d), vmax, seed,
                        (nbound, nbound, nbound), dt, o, (d, d, d))
        h.make_velocity(2, sub, vo, (d, d, d), vmax, seed, (0, 0, 0), dt, o,
                        (d, d, d))
        margin = (nbound + 4) * d
        nrx = int((n1 * d - 2 * margin) // 25.0)
        nry = int((n2 * d - 2 * margin) // 25.0)
        locs_r = born.receiver_geometry(nrx, nry, o[0] + margin, 25.0,
                                        o[1] + margin, 25.0, 10.0, o,
                                        (d, d, d), n1, n2)
        rec = np.zeros((nrx * nry, nt_big), np.float32)
        rec[:, 4:4 + nt] = 1e-3 * rng.standard_normal((nrx * nry, nt),
                                                      dtype=np.float32)
        h.transferReceiverFunc(nrx, nry, nt_big, locs_r, rec)
        handles.append(h)
    return handles, dict(nt=nt_fd, jt=jt, nbound=nbound)


# ---------------------------------------------------------------------------
# c5: least-squares RTM by CG over several shots

def c5_problem(model_n=128, nshots=16, nt_data=400, nbound=40, d=10.0,
               f=15.0, dt_data=0.001, seed=1005):
    """The c5 inversion problem: model_n x model_n x max(32, 2 model_n / 3)
    cells at d, layered 1500..4000 m/s with a dipping +300 m/s step,
    sqrt(nshots) x sqrt(nshots) sources 2 d deep, receivers over the model
    surface, a Ricker wavelet, and the true reflectivity: six seeded
    z-planes of +-1e-3.  Returns (keyword arguments of BornOperator,
    m_true)."""
    n1 = n2 = model_n
    n3 = max(32, (2 * n1) // 3)
    rng = np.random.default_rng(seed)
    z = np.arange(n3, dtype=np.float32)[:, None, None]
    x = np.arange(n1, dtype=np.float32)[None, None, :]
    vel = 1500.0 + 2500.0 * z / (n3 - 1) + 0 * x
    vel = np.where(z > 0.5 * n3 + 0.1 * (x - n1 / 2), vel + 300.0, vel)
    vel = np.broadcast_to(vel, (n3, n2, n1)).astype(np.float32)
    m_true = np.zeros((n3, n2, n1), np.float32)
    for zl in rng.choice(np.arange(n3 // 4, n3 - 8), size=6, replace=False):
        m_true[zl] = rng.choice([-1.0, 1.0]) * 1e-3
    ns = int(round(np.sqrt(nshots)))
    sx = (np.arange(ns) + 0.5) * (n1 * d / ns)
    shots = np.array([[a, b, 2 * d] for b in sx for a in sx], np.float32)
    t = -1.2 / f + np.arange(nt_data) * dt_data
    a = (np.pi * f * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    nr = max(8, n1 // 2)
    rd = d * (n1 - 2) / nr  # receivers spread over the model surface
    kw = dict(velocity=vel, o=(0., 0., 0.), d=(d, d, d), shots=shots,
              wavelet=wav, dt_wavelet=dt_data, nt_data=nt_data,
              dt_data=dt_data, rec_n=(nr, nr), rec_o=(d, d), rec_d=(rd, rd),
              rec_depth=d, nbound=nbound)
    return kw, m_true
