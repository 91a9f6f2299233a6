"""The exact Born coupling (csrc/born_couple.h, storage BORN_STORE_F32_EXACT)
against the reference's double expression of cpuProp::imageAdd
(base/cpu_prop.cc:216-223), on the CPU: the same float operations the
kernel performs, compiled without fused multiply-adds, must give the
double expression's float bit for bit on wavefield-like, full-range,
near-tie, underflow and signed-zero inputs (tests/cpp/couple_check.cc)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "sc17-born_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("couple") / "couple_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-fno-fast-math",
                    "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "cpp", "couple_check.cc"), "-o", exe],
                   check=True)
    return exe


def test_couple_exact_matches_double_expression(checker):
    out = subprocess.run([checker, "1000000"], capture_output=True, text=True)
    rows = {}
    for line in out.stdout.splitlines():
        name, n, bad, fb = line.split()
        rows[name] = (int(n), int(bad), int(fb))
    print(out.stdout, out.stderr)
    assert set(rows) == {"field", "wide", "neartie", "tiny", "edge", "zeros"}
    for name, (n, bad, fb) in rows.items():
        assert n > 0 and bad == 0, (name, n, bad, out.stderr)
    # the near-tie class exercises both outcomes of the boundary test
    n, _, fb = rows["neartie"]
    assert 0 < fb < n
    assert out.returncode == 0
