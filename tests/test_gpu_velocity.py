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
