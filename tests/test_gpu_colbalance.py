"""GPU tests of balance_check!'s column checks (clmgb_balance_check_columns): the cases of
test_balance_check.jl, and bit-for-bit parity of errh2o and of the device-reduced report
with the oracle on seeded columns (with non-finite storages and ties)."""
import numpy as np
import pytest

import colbalance_cases as B
from clmgb import abi, api, colbalance, synth
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_balance_check_reference_cases():
    g = B.load()
    h = api.Handle(synth.clm5_varpar())
    try:
        for case in g["cases"]:
            host = B.build(case)
            ref = host.copy()
            rref = O.balance_check_columns(ref, case["dtime"])
            d = host.to_device()
            rep = colbalance.balance_check_columns(h, d, case["dtime"])
            out = d.to_host()
            B.check(case, out, rep)
            assert np.array_equal(out["errh2o"], ref["errh2o"], equal_nan=True), case["name"]
            B.same_report(rep, rref)
    finally:
        h.close()


@pytest.mark.parametrize("seed,nc,with_errsoi", [(1, 100000, True), (2, 7, True), (3, 5000, False)])
def test_balance_check_matches_oracle_bits(seed, nc, with_errsoi):
    h = api.Handle(synth.clm5_varpar())
    try:
        host = colbalance.random_state(nc, seed=seed)
        host["errsoi"][: nc // 3] = 0.0                       # ties among the maxima of inactive/zero
        ref = host.copy()
        rref = O.balance_check_columns(ref, 1800.0)
        d = host.to_device()
        rep = colbalance.balance_check_columns(h, d, 1800.0, with_errsoi=with_errsoi)
        out = d.to_host()
        assert np.array_equal(out["errh2o"], ref["errh2o"], equal_nan=True)
        if with_errsoi:
            B.same_report(rep, rref)
        else:
            assert rep.errsoi_max == 0.0 and rep.errsoi_index == 0
            assert (rep.errh2o_index, rep.errh2o_nonfinite) == (rref.errh2o_index, rref.errh2o_nonfinite)
            assert np.array_equal(np.float64(rep.errh2o_max), np.float64(rref.errh2o_max), equal_nan=True)
            assert rep.flags == rref.flags & (abi.BAL_H2O_WARN | abi.BAL_H2O_ERROR | abi.BAL_H2O_NONFINITE)
    finally:
        h.close()
