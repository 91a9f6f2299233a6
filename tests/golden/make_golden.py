"""Generate the golden fixtures for the Born / RTM hot path.

Runs the reference's own CPU propagator (base/cpu_prop.cc and
base/sinc_bob.cc, compiled from source by ``oracle/Makefile ref``) on small
seeded cases and stores inputs and outputs in ``tests/golden/*.npz``.  Needs
the reference sources (present only where the fixtures are made); the
fixtures themselves travel with the repository.

    python tests/golden/make_golden.py           # every fixture
    python tests/golden/make_golden.py solver    # solver_ref.npz only
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import pyoracle as po  # noqa: E402
import cases  # noqa: E402

# (name, seed, shape (nz, ny, nx), nt, jt, duplicated receivers)
CASES = [
    ("g1_jt1_even", 11, (20, 24, 28), 40, 1, 0),
    ("g2_jt2_odd", 12, (20, 24, 28), 41, 2, 0),
    ("g3_jt1_dup", 13, (20, 24, 32), 30, 1, 3),
]


def main():
    if po.ref_lib() is None:
        sys.exit("reference sources not available: cannot make fixtures")
    tabs = {f"sinc_{n}": po.sinc_table(n, 8, ref=True) for n in (1, 2, 3, 4, 8)}
    np.savez_compressed(os.path.join(HERE, "sinc_tables.npz"), **tabs)
    for name, seed, shape, nt, jt, dup in CASES:
        c = cases.make_case(seed, shape=shape, nt=nt, jt=jt,
                            dup_receivers=dup,
                            sinc=lambda n: po.sinc_table(n, 8, ref=True))
        out = po.run_case(po.RefProp(), c)
        arrays = {k: v for k, v in c.items() if isinstance(v, np.ndarray)}
        scalars = {k: np.array(v) for k, v in c.items()
                   if not isinstance(v, np.ndarray)}
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            **{f"in_{k}": v for k, v in arrays.items()},
            **{f"par_{k}": v for k, v in scalars.items()},
            **{f"out_{k}": v for k, v in out.items()})
        print(name, {k: float(np.linalg.norm(v)) for k, v in out.items()})
    make_geometry()


def make_geometry():
    """Outputs of the reference's geometry and glue code (compiled from its
    own sources into oracle/_ref/libref_geom.so) on the seeded inputs of
    tests/geometry_cases.py; the inputs are regenerated from the seed."""
    import geometry_cases as gc
    if po.ref_geom_lib() is None:
        sys.exit("reference sources not available: cannot make fixtures")
    out = gc.run(gc.make_inputs(GEOMETRY_SEED), po, ref=True)
    np.savez_compressed(os.path.join(HERE, "geometry.npz"),
                        seed=np.array(GEOMETRY_SEED), **out)
    print("geometry", sorted(out))


GEOMETRY_SEED = 0


def make_solver():
    """Outputs of the reference's own least-squares classes (lin_solver,
    cgstep; compiled from its sources into oracle/_ref by oracle/Makefile):
    the CG loop on a host problem (tests/cpp/pin_solver.cc) and the operator
    adapter under those classes over a host stand-in of the C ABI
    (tests/cpp/drive_solver.cc + fake_born.cc) on the problem
    tests/test_solver_adapter.py uses."""
    import subprocess
    import tempfile
    import pathlib
    import test_solver_adapter as tsa
    pin = po.ref_program("pin_solver_ref")
    drive = po.ref_program("drive_solver_ref_fake")
    if pin is None or drive is None:
        sys.exit("reference sources not available: cannot make fixtures")
    pin_out = subprocess.run([pin, "10"], capture_output=True, text=True,
                             check=True).stdout
    kw, m_true = tsa.fake_problem()
    with tempfile.TemporaryDirectory() as d:
        d = pathlib.Path(d)
        tsa.write_problem(d, kw, m_true)
        drive_out = subprocess.run([drive, str(d), "6", "1"],
                                   capture_output=True, text=True,
                                   check=True).stdout
        model = np.fromfile(d / "model_solver.f32", np.float32)
    np.savez_compressed(os.path.join(HERE, "solver_ref.npz"),
                        pin_stdout=np.array(pin_out),
                        adapter_stdout=np.array(drive_out),
                        adapter_model=model)
    print(pin_out)
    print(drive_out)


if __name__ == "__main__":
    if sys.argv[1:] == ["solver"]:
        make_solver()
    else:
        main()
        make_solver()
