"""The multi-rank path of bench.py on CPU ranks (gloo, world size 2): shots
are sharded one per rank with no data-path collective, and the reported
time is the maximum over ranks, so the whole-job rate counts every rank's
cells against the slowest rank."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import importlib.util
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    t_ms = 100.0 + 50.0 * r  # rank 1 is slower
    t_max = bench.barrier_max(t_ms, w)
    rate = bench.aggregate_rate(1e9, 2, t_max, w)
    out[r] = (bench.shot_of_rank(r, 48), t_max, rate)
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_shots_and_take_max_time():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == 0 and res[1][0] == 1          # one shot per rank
    assert res[0][1] == res[1][1] == 150.0             # max over ranks
    assert abs(res[0][2] - 2 * 1e9 * 2 / 0.150 / 1e9) < 1e-9  # weak scaling


def _stack_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import importlib.util
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkg = os.path.join(root, "sc17-born_gb300")
    spec = importlib.util.spec_from_file_location(
        "born_gb300", os.path.join(pkg, "__init__.py"),
        submodule_search_locations=[pkg])
    born = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(born)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # each rank's "image" of its own shot; the stack is their sum
    img = torch.arange(24, dtype=torch.float32).reshape(2, 3, 4) * (rank + 1)
    born.stack_tensor(img)
    out[rank] = img.numpy().tolist()
    dist.destroy_process_group()


def test_image_stack_sums_the_ranks_shots():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_stack_worker, args=(world, port, out), nprocs=world,
                 join=True)
        res = dict(out)
    want = (torch.arange(24, dtype=torch.float32).reshape(2, 3, 4) * 3)
    for r in range(world):
        assert torch.equal(torch.tensor(res[r]), want)


def _rtm_worker(rank, world, port, out):
    """One rank: its own shot (bench.shot_of_rank) propagated by the oracle
    port on the CPU (sourceProp + rtmAdjoint in rtm_zero_op's order), then
    the images stacked over the ranks with stack_tensor (gloo)."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import importlib.util
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "tests"))
    import cases
    import pyoracle as po
    pkg = os.path.join(root, "sc17-born_gb300")
    spec = importlib.util.spec_from_file_location(
        "born_gb300", os.path.join(pkg, "__init__.py"),
        submodule_search_locations=[pkg])
    born = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(born)
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    po.set_threads(1)
    shot = bench.shot_of_rank(rank, 2)
    c = cases.make_case(60 + shot, shape=(20, 24, 28), nt=30, jt=1,
                        sinc=po.sinc_table)
    img = po.run_case(po.PortProp(), c, which="adjoint")["image"]
    t = torch.from_numpy(img.copy())
    born.stack_tensor(t)
    out[rank] = (shot, t.numpy().tobytes())
    dist.destroy_process_group()


def test_two_gloo_ranks_stack_propagated_images():
    """Sharding on real propagation outputs: two ranks migrate one shot
    each with the oracle port and the stacked image equals the sum of the
    two shots' images computed in one process.  The CPU stand-in for the
    GPU ranks; the multi-GPU stack itself is unmeasured on hardware (every
    GPU run of this build has one GPU)."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "tests"))
    import numpy as np

    import cases
    import pyoracle as po
    po.build_port()
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rtm_worker, args=(world, port, out), nprocs=world,
                 join=True)
        res = dict(out)
    assert sorted(res[r][0] for r in range(world)) == [0, 1]
    want = None
    for shot in range(world):
        c = cases.make_case(60 + shot, shape=(20, 24, 28), nt=30, jt=1,
                            sinc=po.sinc_table)
        img = po.run_case(po.PortProp(), c, which="adjoint")["image"]
        assert np.linalg.norm(img) > 0
        want = img if want is None else want + img
    for r in range(world):
        got = np.frombuffer(res[r][1], np.float32).reshape(want.shape)
        assert np.array_equal(got, want), r
