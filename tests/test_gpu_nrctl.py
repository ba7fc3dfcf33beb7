"""Newton-iteration and time-step control on the device (ocpx_nr_*,
ocpx_step_max_change, ocpx_next_time_step) against the reference's own values
recorded in the golden fixtures, bit-exact, and against the CPU restatement
(oracle/nrctl.py) where the device's own residual norms are used."""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim
from oracle import nrctl

pytestmark = pytest.mark.gpu

FIXTURES = ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4"]


def _f(rec, k):
    return float(rec[k].ravel()[0])


def _i(rec, k):
    return int(rec[k].ravel()[0])


def _ctx(fx):
    model, grid = fim.model_and_grid_from_dump(fx)
    return fim.FimContext(model, grid)


def _nr_control(rec, **kw):
    c = fim.NRControl.make(maxIter=_i(rec, "nr_maxIter"), tol=_f(rec, "nr_tol"), dPmin=_f(rec, "nr_dPmin"),
                           dSmin=_f(rec, "nr_dSmin"), iterNR=_i(rec, "nr_iter"),
                           maxWellRelRes_mol=_f(rec, "nr_maxWellRelRes_mol"), res_from_host=1,
                           maxRelRes_V=_f(rec, "nr_maxRelRes_V"), maxRelRes0_V=_f(rec, "nr_maxRelRes0_V"),
                           maxRelRes_N=_f(rec, "nr_maxRelRes_N"))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("name", FIXTURES)
def test_nr_max_change_and_converge(gpu_lib, name):
    fx = P.load_fixture(name)
    cases = P.nr_cases(fx)
    assert cases
    with _ctx(fx) as ctx:
        for it, last, now, rec in cases:
            dt = float(P.jac_state(fx, it)["dt"].ravel()[0])
            ctx.load_state(last)
            n0 = ctx.cal_res(dt)
            ctx.update_last_time_step()
            ctx.nr_init_step()
            ctx.load_state(now)
            got = ctx.nr_max_change()
            for k, ref in (("dP", "nr_dPBmax"), ("dT", "nr_dTmax"), ("dN", "nr_dNmax"), ("dS", "nr_dSmax"),
                           ("eV", "nr_eVmax")):
                assert got[k] == _f(rec, ref), (it, k, got[k], _f(rec, ref))
            # the reference's residual norms (with the wells' perforation terms)
            assert ctx.nr_check_converge(_nr_control(rec)) == _i(rec, "nr_state"), it
            # the device's own (bulk) norms, against the restatement
            n1 = ctx.cal_res(dt)
            c = _nr_control(rec, res_from_host=0)
            ref = nrctl.check_converge(n1.maxRelRes_V, n0.maxRelRes_V, n1.maxRelRes_N, c.maxWellRelRes_mol,
                                       got["dP"], got["dS"], c.iterNR, c.tol, c.dPmin, c.dSmin, c.maxIter)
            assert ctx.nr_check_converge(c) == ref, it
            # a second call compares with the state the first one recorded
            assert ctx.nr_max_change() == dict(dP=0.0, dT=0.0, dN=0.0, dS=0.0, eV=got["eV"]), it


@pytest.mark.parametrize("name", FIXTURES)
def test_step_max_change_and_next_dt(gpu_lib, name):
    fx = P.load_fixture(name)
    cases = P.ts_cases(fx)
    assert cases
    with _ctx(fx) as ctx:
        for it, start, now, rec in cases:
            ctx.load_state(start)
            ctx.update_last_time_step()
            ctx.load_state(now)
            got = ctx.step_max_change()
            for k, ref in (("dP", "ts_dPBmax"), ("dT", "ts_dTmax"), ("dN", "ts_dNmax"), ("dS", "ts_dSmax"),
                           ("eV", "ts_eVmax")):
                assert got[k] == _f(rec, ref), (it, k, got[k], _f(rec, ref))
            c = fim.NRControl.make(maxIncreFac=_f(rec, "ts_maxIncreFac"), minChopFac=_f(rec, "ts_minChopFac"),
                                   dPlim=_f(rec, "ts_dPlim"), dSlim=_f(rec, "ts_dSlim"),
                                   timeMax=_f(rec, "ts_timeMax"), timeMin=_f(rec, "ts_timeMin"),
                                   end_time=_f(rec, "ts_end_time"), current_dt=_f(rec, "ts_last_dt"),
                                   current_time=_f(rec, "ts_time_before"), iterNR=_i(rec, "ts_iter"),
                                   dPWmaxT=_f(rec, "ts_dPWmax"))
            dt, pdt = ctx.next_time_step(c)
            assert dt == _f(rec, "ts_next_dt") and pdt == _f(rec, "ts_predict_dt"), (it, dt, pdt)


def test_max_change_tie_rule_and_zeros(gpu_lib):
    """Planted changes at 300,000 cells (several reduction blocks): equal
    magnitudes of both signs keep the first cell in order; all-zero changes
    give +0; the device agrees with the restatement."""
    from opencaeporox_gb300 import synthetic
    nb, ncomp = 300_000, 4
    model = synthetic.comp_model(ncomp, 3)
    grid = synthetic.flash_grid(nb)
    rng = np.random.default_rng(5)
    P0 = rng.uniform(100, 300, nb)
    Ni0 = rng.uniform(1, 2, (nb, ncomp + 1))
    st = synthetic.flash_state(P0, Ni0, 80.0)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(st)
        ctx.update_property()
        base = {k: ctx.get(k) for k in ("P", "NI", "S", "VF", "ROCKVP", "T")}
        ctx.update_last_time_step()
        ctx.nr_init_step()
        zero = ctx.nr_max_change()
        assert zero["dP"] == 0.0 and zero["dS"] == 0.0 and zero["dN"] == 0.0
        assert np.copysign(1.0, zero["dP"]) == 1.0
        P1 = base["P"].copy()
        P1[[7, 123_456, 299_999]] += [-2.5, 2.5, -2.5]  # same magnitude: cell 7 wins, sign kept
        ctx.set("P", P1)
        got = ctx.nr_max_change()
        assert got["dP"] == -2.5
        now = dict(P=P1, T=base["T"], Ni=base["NI"], S=base["S"], vf=base["VF"], rockVp=base["ROCKVP"])
        last = dict(P=base["P"], T=base["T"], Ni=base["NI"], S=base["S"])
        assert got == nrctl.max_change_nr(now, last, ncomp + 1)
