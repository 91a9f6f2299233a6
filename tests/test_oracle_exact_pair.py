"""The oracle's exact linearised pair and the FP64 restatement of the
exact Born operator (test infrastructure) are transposes of each other:
<L m, d> = <m, L' d> to FP64 rounding."""
import numpy as np

import cases
from exact_op64 import ExactOperator64


def test_oracle_lin_pair_is_a_transpose_pair(po):
    for jt in (1, 2):
        c = cases.make_case(81 + jt, shape=(28, 32, 36), nt=60, jt=jt,
                            sinc=po.sinc_table)
        o = po.PortProp64()
        po.run_case(o, c, which="none")
        rng = np.random.default_rng(1)
        m = rng.standard_normal(c["shape"])
        d = rng.standard_normal(c["rec_in"].shape)
        rec = np.zeros(c["rec_in"].shape)
        o.transferReceiverFunc(c["rec_nx"], c["rec_ny"], c["nt_big"],
                               c["locs_r"], rec)
        o.lin_forward(c["jts"], m, rec, c["nt"])
        a = np.vdot(rec, d)
        b = np.vdot(m, o.lin_adjoint(c["jts"], d, c["nt"]))
        assert abs(a - b) <= 1e-11 * abs(a), (jt, a, b)


def test_fp64_exact_operator_is_a_transpose_pair(po):
    from test_operator import setup_problem
    op = ExactOperator64(po, setup_problem(seed=9, nshots=2, nt_data=40))
    rng = np.random.default_rng(3)
    m = rng.standard_normal(op.model_shape)
    d = rng.standard_normal(op.data_shape)
    a = np.vdot(op.forward(m), d)
    b = np.vdot(m, op.adjoint(d))
    assert abs(a - b) <= 1e-11 * abs(a), (a, b)
