"""The oracle's restatement of the wells' part of the FIM residual against
the reference's own values (the wells_* golden fixtures): perforation
pressures, phase transmissibilities, perforation and well mole rates, and
the full residual rebuilt from the bulk residual, all bit-identical."""
import os

import numpy as np
import pytest

from oracle import wells as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["wells_bo_10x10x3", "wells_comp6_8x8x3"]


def iterations(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    its = sorted({k.split("/")[0] for k in z.files if k.startswith("it")})
    return [(it, {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(it + "/")}) for it in its]


@pytest.mark.parametrize("name", CASES)
def test_fixture_has_both_controls_and_types(name):
    its = iterations(name)
    assert its
    fx = its[0][1]
    assert set(fx["well_type"].tolist()) == {0, 1}
    assert len(fx["res_full"]) > len(fx["res_bulk"])


@pytest.mark.parametrize("name", CASES)
def test_perforations_and_rates(name):
    for it, fx in iterations(name):
        wells, nc, np_ = W.split_wells(fx)
        p0 = 0
        for w in wells:
            fl = W.perf_flux(w, fx, nc, np_)
            n = len(w["loc"])
            assert np.array_equal(fl["P"], fx["perf_P"][p0:p0 + n]), it
            assert np.array_equal(np.ravel(fl["transj"]), fx["perf_transj"][p0 * np_:(p0 + n) * np_]), it
            if w["type"] == 0:
                assert np.array_equal(fl["trans_inj"], fx["perf_trans_inj"][p0:p0 + n]), it
            assert np.array_equal(np.ravel(fl["perf_qi"]), fx["perf_qi"][p0 * nc:(p0 + n) * nc]), it
            p0 += n
        assert np.array_equal(np.ravel([W.perf_flux(w, fx, nc, np_)["qi"] for w in wells]), fx["well_qi"]), it


@pytest.mark.parametrize("name", CASES)
def test_residual_with_wells(name):
    for it, fx in iterations(name):
        wells, nc, np_ = W.split_wells(fx)
        res, max_rel = W.residual_with_wells(fx["res_bulk"], wells, fx, float(fx["dt"][0]), nc, np_)
        assert np.array_equal(res, fx["res_full"]), it
        assert max_rel == float(fx["maxWellRelRes_mol"][0]), it


def test_a_planted_error_is_caught():
    """A wrong sign in the restated producer flux must fail the comparison."""
    it, fx = iterations("wells_bo_10x10x3")[0]
    wells, nc, np_ = W.split_wells(fx)
    bad = dict(fx, Pj=2 * np.asarray(fx["perf_P"]).max() - np.asarray(fx["Pj"]))
    res, _ = W.residual_with_wells(fx["res_bulk"], wells, bad, float(fx["dt"][0]), nc, np_)
    assert not np.array_equal(res, fx["res_full"])
