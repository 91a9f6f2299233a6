"""born_dot_f64_noalloc: the FP64 dot product for callers that cannot
allocate device memory (applications whose GPU memory is all held by their
own pool, code that cannot take the device-wide synchronisation of
cudaMalloc/cudaFree).  It must agree with the allocating entry point
born_dot_f64 within the FP64 tolerance used by the other dot tests, on two
calls in a row (the second call reuses the shared scratch array without any
clearing), and reject vectors longer than its fixed scratch allows.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test; it also runs alone in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

from test_operator import setup_problem

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative, FP64 accumulations of the same float products


def test_noalloc_dot_matches_allocating_entry_point(born):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = born.lib()
    op = born.BornOperator(exact=True, **setup_problem(seed=5, nshots=1))
    g = torch.Generator(device="cuda").manual_seed(123)
    for n in (1_000_003, 4097):
        a = torch.randn(n, device="cuda", generator=g)
        b = torch.randn(n, device="cuda", generator=g)
        want = op.dot(a, b)  # born_dot_f64 (scratch allocated by the op)
        for _ in range(2):  # two calls in a row share the scratch array
            out = C.c_double(0.0)
            rc = L.born_dot_f64_noalloc(C.c_void_p(a.data_ptr()),
                                        C.c_void_p(b.data_ptr()), n,
                                        C.byref(out), None)
            assert rc == 0
            assert abs(out.value - want) <= TOL * abs(want), (out.value, want)
    # beyond the scratch capacity: rejected before any device work
    out = C.c_double(0.0)
    rc = L.born_dot_f64_noalloc(C.c_void_p(a.data_ptr()),
                                C.c_void_p(b.data_ptr()),
                                268435456 + 1, C.byref(out), None)
    assert rc == -1
