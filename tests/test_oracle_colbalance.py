"""CPU checks of the oracle's restatement of balance_check!'s column checks: the cases of
test_balance_check.jl with the stop decisions it asserts, and the report's maxima and
first indices on seeded columns against numpy."""
import numpy as np

import colbalance_cases as B
from clmgb import abi, colbalance
from oracle import oracle as O


def test_balance_check_reference_cases():
    g = B.load()
    assert len(g["cases"]) == 9
    for case in g["cases"]:
        cb = B.build(case)
        rep = O.balance_check_columns(cb, case["dtime"])
        B.check(case, cb, rep)


def test_balance_report_matches_numpy():
    cb = colbalance.random_state(3000, seed=2)
    cb["endwb"][:] = np.where(np.isnan(cb["endwb"]), cb["begwb"], cb["endwb"])     # all finite here
    rep = O.balance_check_columns(cb, 1800.0)
    a = np.abs(cb["errh2o"])
    assert rep.errh2o_max == a.max() and rep.errh2o_index == int(np.argmax(a)) + 1
    assert rep.errh2o_nonfinite == 0
    s = np.where(cb["col_active"] != 0, np.abs(cb["errsoi"]), 0.0)
    assert rep.errsoi_max == s.max() and rep.errsoi_index == int(np.argmax(s)) + 1
    assert bool(rep.flags & abi.BAL_SOI_WARN) == (s.max() > 1e-5)
    assert np.all(cb["errh2o"][cb["col_active"] == 0] == 0.0)


def test_skip_steps_follow_balance_check_init():
    assert colbalance.skip_steps(1800.0) == 3
    assert colbalance.skip_steps(3600.0) == 3
    assert colbalance.skip_steps(600.0) == 7
