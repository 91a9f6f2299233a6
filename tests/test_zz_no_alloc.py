"""born_dot_f64_noalloc: the FP64 dot product for callers that cannot
allocate device memory (applications whose GPU memory is all held by their
own pool, code that cannot take the device-wide synchronisation of
cudaMalloc/cudaFree).  It must agree with the allocating entry point
born_dot_f64 within the FP64 tolerance used by the other dot tests, on two
calls in a row (the second call reuses the shared scratch array without any
clearing), for an empty vector, for the longest vector its fixed scratch
allows, and on a caller's own stream; and it must reject longer vectors.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.  The last test repeats the check
in a fresh Python process, where the call is the first one on the device
(the call that looks up the scratch array's address)."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from test_operator import setup_problem

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative, FP64 accumulations of the same float products
MAX_N = 268435456  # BORN_DOT_NOALLOC_MAX


def noalloc_dot(L, a, b, n, stream=None):
    out = C.c_double(0.0)
    rc = L.born_dot_f64_noalloc(C.c_void_p(a.data_ptr()),
                                C.c_void_p(b.data_ptr()), n, C.byref(out),
                                None if stream is None
                                else C.c_void_p(stream))
    return rc, out.value


@pytest.fixture(scope="module")
def torch_cuda(born):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def test_noalloc_dot_matches_allocating_entry_point(born, torch_cuda):
    torch = torch_cuda
    L = born.lib()
    op = born.BornOperator(exact=True, **setup_problem(seed=5, nshots=1))
    g = torch.Generator(device="cuda").manual_seed(123)
    for n in (1_000_003, 4097):
        a = torch.randn(n, device="cuda", generator=g)
        b = torch.randn(n, device="cuda", generator=g)
        want = op.dot(a, b)  # born_dot_f64 (scratch allocated by the op)
        for _ in range(2):  # two calls in a row share the scratch array
            rc, got = noalloc_dot(L, a, b, n)
            assert rc == 0
            assert abs(got - want) <= TOL * abs(want), (got, want)
    # an empty vector: only the final pass runs, over no partials
    rc, got = noalloc_dot(L, a, b, 0)
    assert rc == 0 and got == 0.0
    # beyond the scratch capacity: rejected before any device work
    rc, _ = noalloc_dot(L, a, b, MAX_N + 1)
    assert rc == -1


def test_noalloc_dot_longest_vector(born, torch_cuda):
    """n = BORN_DOT_NOALLOC_MAX fills every one of the 65,536 partial sums
    (two 1 GiB inputs)."""
    torch = torch_cuda
    L = born.lib()
    op = born.BornOperator(exact=True, **setup_problem(seed=5, nshots=1))
    g = torch.Generator(device="cuda").manual_seed(7)
    a = torch.randn(MAX_N, device="cuda", generator=g)
    b = torch.randn(MAX_N, device="cuda", generator=g)
    want = op.dot(a, b)
    for _ in range(2):
        rc, got = noalloc_dot(L, a, b, MAX_N)
        assert rc == 0
        assert abs(got - want) <= TOL * abs(want), (got, want)
    # the shorter call after the longest one reads only its own partials
    rc, got = noalloc_dot(L, a, b, 5000)
    assert rc == 0
    assert abs(got - op.dot(a[:5000], b[:5000])) <= TOL * abs(got)
    del a, b
    torch.cuda.empty_cache()


def test_noalloc_dot_on_caller_stream(born, torch_cuda):
    """The inputs are produced on a torch side stream and the call is made
    on that stream: it is ordered after their production."""
    torch = torch_cuda
    L = born.lib()
    op = born.BornOperator(exact=True, **setup_problem(seed=5, nshots=1))
    g = torch.Generator(device="cuda").manual_seed(99)
    n = 3_000_017
    a0 = torch.randn(n, device="cuda", generator=g)
    b0 = torch.randn(n, device="cuda", generator=g)
    want = op.dot(a0, b0)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        torch.cuda._sleep(100_000_000)
        a = a0 * 1.0
        b = b0 * 1.0
        rc, got = noalloc_dot(L, a, b, n, stream=side.cuda_stream)
    assert rc == 0
    assert abs(got - want) <= TOL * abs(want), (got, want)


def test_noalloc_dot_fresh_process(born, torch_cuda):
    """The first call in a new process (which sets up the scratch address
    on the device) against born_dot_f64, two calls in a row."""
    here = os.path.dirname(os.path.abspath(__file__))
    test = os.path.basename(__file__) + \
        "::test_noalloc_dot_matches_allocating_entry_point"
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m",
                        "gpu", "-p", "no:cacheprovider", test], cwd=here,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "1 passed" in r.stdout
