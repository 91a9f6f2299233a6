"""Random-boundary velocity made on the device (vel_fd_3d::rand_subspace
with counter-based draws): the plain model and every cell outside the random
bands equal the host restatement bit for bit; band cells respect the
reference's acceptance bound; the field is deterministic per seed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_velocity(born):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(3)
    vel = (2000 + 500 * rng.random((14, 16, 18))).astype(np.float32)
    vmax = float(vel.max())
    shape = (32, 36, 40)
    o, d = (-80.0, -80.0, -80.0), (10.0, 10.0, 10.0)
    vo, vd = (0.0, 0.0, 0.0), (10.0, 10.0, 10.0)
    g = born.Gb300Prop()
    g.createSpace(10., 10., 10., 50, .0005, .0005, shape[2], shape[1],
                  shape[0])
    host0 = born.rand_subspace(vel, vo, vd, vmax, 5, (0, 0, 0), 0.001, shape,
                               o, d)
    g.make_velocity(2, vel, vo, vd, vmax, 5, (0, 0, 0), 0.001, o, d)
    assert np.array_equal(g.get_velocity(2), host0)
    nr = 8
    g.make_velocity(1, vel, vo, vd, vmax, 77, (nr, nr, nr), 0.001, o, d)
    a = g.get_velocity(1)
    g.make_velocity(1, vel, vo, vd, vmax, 77, (nr, nr, nr), 0.001, o, d)
    assert np.array_equal(a, g.get_velocity(1))           # deterministic
    g.make_velocity(1, vel, vo, vd, vmax, 78, (nr, nr, nr), 0.001, o, d)
    b = g.get_velocity(1)
    inner = (slice(nr, -nr),) * 3
    assert np.array_equal(a[inner], host0[inner])         # outside the bands
    assert not np.array_equal(a, b)                       # seed matters
    v = np.sqrt(a.astype(np.float64)) / 0.001
    assert v.min() > 0.0001 and v.max() <= vmax * 1.03 * 1.0000001


def _band2(n, nr):
    """Squared normalised distance into the bands of one axis, in float32 as
    vel_fd_3d.cc:60-99 forms it."""
    i = np.arange(n)
    k = np.where(i < nr, nr - i, np.where(i >= n - nr, i - (n - nr - 1), 0))
    return (np.float32(1) * (k * k).astype(np.float32) /
            np.float32(nr * nr)).astype(np.float32)


def test_device_velocity_tapered_bound(born):
    """Every band cell obeys the reference's per-cell acceptance bound
    |v| < vmax * 1.03 * (1 - 0.4 min(1, dist)) (vel_fd_3d.cc:115-122), and
    the accepted draws have the reference's form
    v = val (1 + 1.3 dist (u - 0.5 - 0.49 dist)) with u in [0, 1), u
    spread uniformly where the bound does not bite."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(4)
    vm = (1500 + 2500 * rng.random((20, 22, 24))).astype(np.float32)
    vmax = float(vm.max())
    n3, n2, n1 = shape = (48, 52, 56)
    nr, dt = 12, 0.001
    o, d = (-120.0, -120.0, -120.0), (10.0, 10.0, 10.0)
    g = born.Gb300Prop()
    g.createSpace(10., 10., 10., 50, .0005, .0005, n1, n2, n3)
    g.make_velocity(1, vm, (0., 0., 0.), d, vmax, 31, (nr, nr, nr), dt, o, d)
    a = g.get_velocity(1).astype(np.float64)
    v = np.sqrt(a) / dt
    # nearest model index, clamped: (-120 + 10 i) / 10 is exact here
    idx = [np.clip(np.arange(m) - 12, 0, vn - 1)
           for m, vn in ((n3, 20), (n2, 22), (n1, 24))]
    val = vm[np.ix_(idx[0], idx[1], idx[2])].astype(np.float64)
    bz, by, bx = _band2(n3, nr), _band2(n2, nr), _band2(n1, nr)
    s = (bx[None, None, :] + by[None, :, None]).astype(np.float32)
    dist = np.sqrt((s + bz[:, None, None]).astype(np.float32)).astype(
        np.float64)
    band = dist >= 1e-4
    assert band.sum() > 0.5 * band.size
    bound = vmax * 1.03 * (1.0 - np.minimum(1.0, dist) * 0.4)
    assert np.all(v[band] <= bound[band] * (1 + 1e-6)), \
        float((v[band] / bound[band]).max())
    assert np.all(v > 0)
    # outside the bands: the plain model
    assert np.allclose(v[~band], val[~band], rtol=1e-6)
    # cells that found no accepted draw in 64 keep 0.999 of the bound
    # (val >= bound) or their value (val < bound); few do
    fallback = band & (np.isclose(v, 0.999 * bound, rtol=1e-6) |
                       np.isclose(v, val, rtol=1e-7))
    assert fallback.sum() < 0.01 * band.sum()
    acc = band & ~fallback
    u = (v[acc] / val[acc] - 1.0) / (1.3 * dist[acc]) + 0.5 + 0.49 * dist[acc]
    assert u.min() > -1e-4 and u.max() < 1 + 1e-4, (u.min(), u.max())
    # where the bound cannot reject a draw (small dist, low val), u is
    # uniform on [0, 1)
    free = acc & (val * (1 + 1.3 * dist * 0.5) < bound) & (dist < 0.5)
    uf = ((v[free] / val[free] - 1.0) / (1.3 * dist[free]) + 0.5 +
          0.49 * dist[free])
    assert uf.size > 2000
    assert abs(uf.mean() - 0.5) < 0.02, uf.mean()
    assert abs(uf.std() - 12 ** -0.5) < 0.02, uf.std()
    hist = np.histogram(uf, bins=10, range=(0, 1))[0] / uf.size
    assert np.all(np.abs(hist - 0.1) < 0.03), hist
