"""Batched shots: one launch per time step over shots with different grids
(and optionally one CUDA graph per time loop) must give every shot exactly
the results of running it alone."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

SHAPES = [(24, 28, 32), (28, 32, 48), (20, 24, 40)]  # nx % 8 == 0 for f16


def setup_shot(born, po, seed, shape, nt=40, jt=1, storage="f32"):
    c = cases.make_case(seed, shape=shape, nt=nt, jt=jt, sinc=po.sinc_table)
    p = born.Gb300Prop()
    nz, ny, nx = shape
    p.createSpace(c["d"], c["d"], c["d"], 50, .0005, .0005, nx, ny, nz)
    p.transferSincTableS(8, jt, c["table_s"])
    p.transferSincTableD(8, jt, c["table_d"])
    p.transferSourceFunc(9, c["nt_big"], c["locs_s"], c["src"])
    p.transferVelFunc1(nx, ny, nz, c["vel1"])
    p.transferVelFunc2(nx, ny, nz, c["vel2"])
    p.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"], c["locs_r"],
                           np.ascontiguousarray(c["rec_in"]))
    p.check(p.lib.born_set_reflectivity(p.h, born.fptr(c["refl"])))
    p.set_storage(storage)
    return p, c


def single(p, c):
    jt, nt = c["jts"], c["nt"]
    p.source_prop_device(jt, nt)
    p.rtm_adjoint_device(jt, nt, swap=1)
    img = p.get_image()
    p.zero_traces()
    p.rtm_forward_device(jt, nt)
    return img, p.get_traces(c["rec_in"])


@pytest.mark.parametrize("storage", ["f32", "f16", "f32fma"])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("jt", [1, 2])
def test_batch_matches_single_shots(born, po, graph, jt, storage):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    want = []
    for k, sh in enumerate(SHAPES):
        p, c = setup_shot(born, po, 90 + k, sh, nt=41 if jt == 2 else 40,
                          jt=jt, storage=storage)
        want.append(single(p, c))
    shots = [setup_shot(born, po, 90 + k, sh, nt=41 if jt == 2 else 40,
                        jt=jt, storage=storage)
             for k, sh in enumerate(SHAPES)]
    batch = born.Batch([p for p, _ in shots], graph=graph)
    c0 = shots[0][1]
    for rep in range(2):  # the second pass replays the recorded graphs
        # the forward loop overwrote the receiver traces: same receivers, new
        # values, so the recorded graphs stay valid
        for p, c in shots:
            p.set_traces(c["rec_in"])
        batch.source_prop(c0["jts"], c0["nt"])
        batch.rtm_adjoint(c0["jts"], c0["nt"])
        for p, _ in shots:
            p.zero_traces()
        batch.rtm_forward(c0["jts"], c0["nt"])
        batch.synchronize()
        for (p, c), (img, tr) in zip(shots, want):
            assert np.array_equal(p.get_image(), img)
            assert np.array_equal(p.get_traces(c["rec_in"]), tr)
    # the step kernels of both passes, launched or replayed; with graphs
    # every time loop is one graph launch (recorded once, replayed twice)
    steps = 2 * (3 * c0["nt"] + 1)
    if storage == "f32":
        assert batch.launches == steps
    assert batch.launches >= steps
    assert batch.graph_launches == (6 if graph else 0)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_tiling_refinement_keeps_results(born, po, graph):
    """Loops of 200 steps or more refine the batch's (tile, z-segment depth)
    on their first run, uncaptured; later runs record and replay the chosen
    tiling.  Every run gives every shot its single-shot results."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    nt = 200
    want = []
    for k, sh in enumerate(SHAPES):
        p, c = setup_shot(born, po, 190 + k, sh, nt=nt)
        want.append(single(p, c))
    shots = [setup_shot(born, po, 190 + k, sh, nt=nt)
             for k, sh in enumerate(SHAPES)]
    batch = born.Batch([p for p, _ in shots], graph=graph)
    c0 = shots[0][1]
    for rep in range(3):  # tuning run, recording run, replay
        for p, c in shots:
            p.set_traces(c["rec_in"])
        batch.source_prop(c0["jts"], c0["nt"])
        batch.rtm_adjoint(c0["jts"], c0["nt"])
        for p, _ in shots:
            p.zero_traces()
        batch.rtm_forward(c0["jts"], c0["nt"])
        batch.synchronize()
        for (p, c), (img, tr) in zip(shots, want):
            assert np.array_equal(p.get_image(), img), rep
            assert np.array_equal(p.get_traces(c["rec_in"]), tr), rep
        if rep == 0:
            # the first run of every loop timed the candidates instead of
            # recording a graph
            assert batch.graph_launches == 0
    assert batch.graph_launches == (6 if graph else 0)
    assert batch.launches == 3 * (3 * nt + 1)
