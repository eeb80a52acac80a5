"""The FP64 work model of the Richards solve (clmgb/flops_model.py): FP64-pipe work in
DFMA-equivalents from the kernel-counted level attempts and refreshes, with the
divisions counted as integer-pipe work, and the roofline entry the bench reports."""
import pytest

from clmgb import flops_model as fm


def test_divisions_are_not_fp64_pipe_work():
    w = {"div": 7.5, "pow": 42.5}
    # one level attempt: 15 add/mul/fma; one level refresh: 27 + 2 pow
    assert fm.dfma_equivalents(1, 0, w) == pytest.approx(15.0)
    assert fm.dfma_equivalents(0, 1, w) == pytest.approx(27.0 + 2 * 42.5)
    assert fm.integer_divisions(1, 0) == 3
    assert fm.integer_divisions(0, 1) == 10
    assert fm.integer_divisions(18_080_370, 14_075_378) == 18_080_370 * 3 + 14_075_378 * 10


def test_roofline_entry_is_consistent():
    # rates in the ratios the probe measures on GB300: DFMA, division, pow, log10, integer division
    probe = (5.28e11, 7.02e10, 1.24e10, 1.72e10, 1.42e11)
    att, ref, launches, ms = 18.08e6 * 3, 14.08e6 * 3, 3, 10.43
    r = fm.fp64_roofline(att, ref, launches, ms, probe)
    w = fm.weights(probe)
    work = fm.dfma_equivalents(att, ref, w) / launches
    assert r["dfma_equivalents_per_launch"] == pytest.approx(work)
    assert r["frac"] == pytest.approx(work / (ms / 1e3) / probe[0])
    assert r["achieved"] == pytest.approx(2 * work / (ms / 1e3) / 1e12)
    assert r["peak"] == pytest.approx(2 * probe[0] / 1e12)
    assert r["integer_pipe_divisions_per_launch"] == pytest.approx(fm.integer_divisions(att, ref) / launches)
    assert r["probe_rates_per_s"]["integer_div"] == probe[4]
    assert 0.0 < r["frac"] < 1.0
    # a probe from before the integer-division rate was measured still gives an entry
    assert fm.fp64_roofline(att, ref, launches, ms, probe[:4])["probe_rates_per_s"]["integer_div"] is None
