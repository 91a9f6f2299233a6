"""Seeded propagator inputs for parity tests.

A *case* holds exactly what the reference hands its propagator for one shot
(``rtm_zero_op_3d.cc:147-185`` forward, ``:249-273`` adjoint): velocity in
v^2 dt^2 form for the random-boundary (vel1) and plain (vel2) models, the
source and data sinc tables, 9 source points with their traces, a receiver
grid with its traces, and a reflectivity image.  Traces carry the 4-sample
lead of the reference (``source_func_3d.cc:104``, ``map_data_3d.cc:184``).
"""
from __future__ import annotations

import numpy as np


def _smooth(a: np.ndarray, passes: int = 2) -> np.ndarray:
    for _ in range(passes):
        for ax in range(a.ndim):
            a = (np.roll(a, 1, ax) + 2 * a + np.roll(a, -1, ax)) / 4
    return a


def ricker(nt: int, dt: float, f: float, t0: float = 0.064) -> np.ndarray:
    """util/Wavelet.cc:23-29: (1 - 2 pi^2 f^2 t^2) exp(-pi^2 f^2 t^2)."""
    t = -t0 + np.arange(nt) * dt
    a = (np.pi * f * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def make_case(seed: int, shape=(24, 28, 32), nt: int = 40, jt: int = 1,
              d: float = 10.0, dt: float = 0.001, rec_step: int = 2,
              dup_receivers: int = 0, sinc=None) -> dict:
    """Small seeded case on an (nz, ny, nx) compute grid.

    ``sinc(ntab)`` returns the jt x 8 table; tests pass the oracle's table
    so that every checker sees identical inputs."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    # layered velocity with a smooth perturbation; FD dt = dt/jt
    dtf = dt / jt
    z = np.arange(nz)[:, None, None]
    v = 1800.0 + 1200.0 * (z / max(nz - 1, 1)) + np.zeros(shape)
    v = v * (1 + 0.03 * _smooth(rng.standard_normal(shape)))
    vnone = (v * v * dtf * dtf).astype(np.float32)
    # random-boundary stand-in: perturb within 6 cells of each face
    edge = np.minimum.reduce(np.meshgrid(
        np.minimum(np.arange(nz), nz - 1 - np.arange(nz)),
        np.minimum(np.arange(ny), ny - 1 - np.arange(ny)),
        np.minimum(np.arange(nx), nx - 1 - np.arange(nx)), indexing="ij"))
    pert = 1 + 0.2 * rng.uniform(-1, 1, shape) * (edge < 6)
    vrand = (vnone * pert * pert).astype(np.float32)

    nt_data = (nt - 1) // jt + 1
    nt_big = nt_data + 8
    table = sinc(jt) if sinc is not None else np.eye(jt, 8, 3, np.float32)
    table = np.ascontiguousarray(table, np.float32).reshape(jt, 8)

    # 9 source points on the plane iz-1 (source_func_3d.cc:95-101)
    iz, iy, ix = nz // 3, ny // 2, nx // 2
    locs_s, w = [], []
    for i2 in (iy - 1, iy, iy + 1):
        for i1 in (ix - 1, ix, ix + 1):
            locs_s.append(i1 + i2 * nx + (iz - 1) * nx * ny)
            w.append(np.exp(-((i1 - ix) ** 2 + (i2 - iy) ** 2) * 0.3))
    wav = ricker(nt_data, dt, 25.0, 0.02)
    wav = np.append((wav[1:] - wav[:-1]) / dt, 0).astype(np.float32)
    src = np.zeros((9, nt_big), np.float32)
    for i in range(9):
        src[i, 4:4 + nt_data] = w[i] * wav

    # receiver grid on the plane 5 (+4 pad) (map_data_3d.cc:17-31)
    rz = 5
    rys = np.arange(5, ny - 5, rec_step)
    rxs = np.arange(5, nx - 5, rec_step)
    locs_r = np.array([x + y * nx + rz * nx * ny for y in rys for x in rxs],
                      np.int32)
    if dup_receivers:
        locs_r[-dup_receivers:] = locs_r[:dup_receivers]
    rec_nx, rec_ny = len(rxs), len(rys)
    rec_in = np.zeros((rec_ny * rec_nx, nt_big), np.float32)
    rec_in[:, 4:4 + nt_data] = 1e-3 * _smooth(
        rng.standard_normal((rec_ny * rec_nx, nt_data)), 1)

    refl = np.zeros(shape, np.float32)
    refl[nz // 2:, :, :] = 1.0
    refl += 0.05 * rng.standard_normal(shape).astype(np.float32)
    refl = np.ascontiguousarray(refl, np.float32)

    return dict(shape=shape, d=d, nt=nt, jts=jt, jtd=jt, nt_big=nt_big,
                table_s=table, table_d=table, locs_s=np.array(locs_s, np.int32),
                src=src, vel1=vrand, vel2=vnone, locs_r=locs_r, rec_nx=rec_nx,
                rec_ny=rec_ny, rec_in=rec_in, refl=refl)
