"""The CPU restatement of the Newton-iteration and time-step control
(oracle/nrctl.py) against the reference's own values, recorded by the dump
harness after every Newton iteration and time step of the golden fixtures.
Everything is bit-exact: the maxima select values, the decisions compare."""
import pytest

import parity as P
from oracle import nrctl

FIXTURES = ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4", "comp4_field_6x5x3", "bo_field_10x10x3"]


def _f(rec, k):
    return float(rec[k].ravel()[0])


def _i(rec, k):
    return int(rec[k].ravel()[0])


@pytest.mark.parametrize("name", FIXTURES)
def test_max_change_nr(name):
    fx = P.load_fixture(name)
    cases = P.nr_cases(fx)
    assert cases
    for it, last, now, rec in cases:
        _, nc, np_ = P.state_dims(now)
        got = nrctl.max_change_nr(now, last, nc, np_)
        for k, ref in (("dP", "nr_dPBmax"), ("dT", "nr_dTmax"), ("dN", "nr_dNmax"), ("dS", "nr_dSmax"),
                       ("eV", "nr_eVmax")):
            assert got[k] == _f(rec, ref), (it, k, got[k], _f(rec, ref))


# fixtures that hold finished time steps (the FIELD ones stop inside their first)
STEP_FIXTURES = ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4"]


@pytest.mark.parametrize("name", STEP_FIXTURES)
def test_max_change_time(name):
    fx = P.load_fixture(name)
    cases = P.ts_cases(fx)
    assert cases
    for it, start, now, rec in cases:
        _, nc, np_ = P.state_dims(now)
        got = nrctl.max_change_time(now, start, nc, np_)
        for k, ref in (("dP", "ts_dPBmax"), ("dT", "ts_dTmax"), ("dN", "ts_dNmax"), ("dS", "ts_dSmax"),
                       ("eV", "ts_eVmax")):
            assert got[k] == _f(rec, ref), (it, k, got[k], _f(rec, ref))


@pytest.mark.parametrize("name", FIXTURES)
def test_check_converge(name):
    fx = P.load_fixture(name)
    states = []
    for it, _, _, rec in P.nr_cases(fx):
        st = nrctl.check_converge(_f(rec, "nr_maxRelRes_V"), _f(rec, "nr_maxRelRes0_V"), _f(rec, "nr_maxRelRes_N"),
                                  _f(rec, "nr_maxWellRelRes_mol"), _f(rec, "nr_dPBmax"), _f(rec, "nr_dSmax"),
                                  _i(rec, "nr_iter"), _f(rec, "nr_tol"), _f(rec, "nr_dPmin"), _f(rec, "nr_dSmin"),
                                  _i(rec, "nr_maxIter"))
        assert st == _i(rec, "nr_state"), it
        states.append(st)
    if name == "bo_10x10x3":
        assert 0 in states and 1 in states  # both outcomes are exercised


@pytest.mark.parametrize("name", FIXTURES)
def test_next_time_step(name):
    fx = P.load_fixture(name)
    for it, _, _, rec in P.ts_cases(fx):
        dt, pdt = nrctl.next_time_step(_f(rec, "ts_last_dt"), _f(rec, "ts_time_before"), _f(rec, "ts_dPBmax"),
                                       _f(rec, "ts_dPWmax"), _f(rec, "ts_dSmax"), _i(rec, "ts_iter"),
                                       _f(rec, "ts_maxIncreFac"), _f(rec, "ts_minChopFac"), _f(rec, "ts_dPlim"),
                                       _f(rec, "ts_dSlim"), _f(rec, "ts_timeMax"), _f(rec, "ts_timeMin"),
                                       _f(rec, "ts_end_time"))
        assert dt == _f(rec, "ts_next_dt") and pdt == _f(rec, "ts_predict_dt"), (it, dt, pdt)
