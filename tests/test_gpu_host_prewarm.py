"""Closing host copies warmed during the time loops (born_set_host_prewarm).

With page-locked destinations of 8 MiB or more and loops of 100 steps or
more, source_prop's levels, rtm_adjoint's image and rtm_forward's traces
are first copied into on a side stream while the loop runs, then
overwritten by the closing copy.  The results must equal those of the
unwarmed calls bit for bit, also for the image, which rtm_adjoint reads
from the caller's array before it accumulates into it (cpu_prop.cc:101):
the warming copy has to come after that upload."""
import ctypes as C

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(born):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return born


def run(born, c, warm, pinned):
    import torch
    nz, ny, nx = c["shape"]
    prop = born.Gb300Prop(0)
    prop.createSpace(c["d"], c["d"], c["d"], 50.0, .0005, .0005, nx, ny, nz)
    prop.transferSincTableS(8, c["jts"], c["table_s"])
    prop.transferSincTableD(8, c["jtd"], c["table_d"])
    prop.transferSourceFunc(9, c["nt_big"], c["locs_s"], c["src"])
    prop.transferVelFunc1(nx, ny, nz, c["vel1"])
    prop.transferVelFunc2(nx, ny, nz, c["vel2"])
    rec = np.ascontiguousarray(c["rec_in"])
    prop.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"],
                              c["locs_r"], rec)
    prop.check(prop.lib.born_set_reflectivity(prop.h, born.fptr(c["refl"])))
    prop.check(prop.lib.born_set_host_prewarm(prop.h, int(warm)))

    def buf(shape, fill=0.0):
        t = torch.full(shape, fill, dtype=torch.float32, pin_memory=pinned)
        return t, C.cast(t.data_ptr(), born._fp)

    (p0, f0), (p1, f1) = buf(c["shape"]), buf(c["shape"])
    img, fi = buf(c["shape"], 0.25)  # accumulated into by rtm_adjoint
    tr, ft = buf(c["rec_in"].shape)
    L, h, nt = prop.lib, prop.h, c["nt"]
    prop.check(L.born_source_prop(h, c["jts"], nt, f0, f1))
    prop.check(L.born_rtm_adjoint(h, c["jtd"], nt, 1, fi))
    prop.check(L.born_rtm_forward(h, c["jts"], nt, ft))
    out = [a.numpy().copy() for a in (p0, p1, img, tr)]
    return out, int(L.born_host_prewarm_count(h))


def test_warmed_closing_copies_are_bit_identical(gpu):
    # 144^3 fields (11.9 MB) and 17,956 receivers x 136 samples (9.3 MB)
    c = cases.make_case(31, shape=(144, 144, 144), nt=128, rec_step=1)
    assert c["rec_in"].nbytes >= 8 << 20
    cold, n_cold = run(gpu, c, False, True)
    warm, n_warm = run(gpu, c, True, True)
    assert n_cold == 0 and n_warm == 4  # p0, p1, image, traces
    for a, b, name in zip(cold, warm, ("p0", "p1", "image", "traces")):
        assert np.array_equal(a, b), name
    assert np.abs(cold[2]).max() > 0.25 and np.abs(cold[3]).max() > 0


def test_pageable_and_short_loops_are_not_warmed(gpu):
    c = cases.make_case(32, shape=(144, 144, 144), nt=64, rec_step=1)
    _, n_short = run(gpu, c, True, True)      # 64 steps < 100
    c = cases.make_case(33, shape=(144, 144, 144), nt=128, rec_step=1)
    _, n_pageable = run(gpu, c, True, False)  # pageable host arrays
    assert n_short == 0 and n_pageable == 0
