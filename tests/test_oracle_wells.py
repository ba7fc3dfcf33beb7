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


def _blocks(rowptr, col, val, ncol):
    bs = ncol * ncol
    out = {}
    for r in range(len(rowptr) - 1):
        for e in range(int(rowptr[r]), int(rowptr[r + 1])):
            out[(r, int(col[e]))] = np.asarray(val[e * bs:(e + 1) * bs]).reshape(ncol, ncol)
    return out


def _close(a, b, tol=1e-13):
    return np.linalg.norm(a - b) <= tol * max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_well_jacobian_blocks(name):
    """The blocks the wells' assembly adds to the system: bulk-to-well and the
    wells' diagonal blocks exact; the blocks that carry dQ/dXs times
    dSec_dPri (a BLAS product in the reference) within 1e-13 normwise; every
    other block of the system untouched."""
    checked = 0
    for it, fx in iterations(name):
        jac = {k.split("/", 1)[1]: v for k, v in fx.items() if k.startswith("jac/")}
        if not jac:
            continue
        wells, nc, np_ = W.split_wells(jac)
        ncol = nc + 1
        nb = len(jac["jac_rowptr"]) - 1
        before = _blocks(jac["jac_rowptr"], jac["jac_col"], jac["jac_val"], ncol)
        after = _blocks(jac["jacw_rowptr"], jac["jacw_col"], jac["jacw_val"], ncol)
        got = W.well_jacobian(wells, jac, float(jac["dt"][0]), nb, nc, np_)
        expect_new = set(got["bulk_well"]) | {(w, w) for w in got["well_diag"]} | set(got["well_bulk"])
        assert set(after) == set(before) | expect_new, it
        for key, blk in after.items():
            r, c = key
            if key in got["bulk_well"]:
                assert np.array_equal(blk, got["bulk_well"][key]), (it, key)
            elif r >= nb and r == c:
                assert np.array_equal(blk, got["well_diag"][r]), (it, key)
            elif key in got["well_bulk"]:
                assert _close(blk, got["well_bulk"][key]) or (
                    not np.any(blk) and not np.any(got["well_bulk"][key])), (it, key)
            elif r == c and r in got["bulk_add"]:
                assert _close(blk, before[key] + got["bulk_add"][r]), (it, key)
            else:
                assert np.array_equal(blk, before[key]), (it, key)
        checked += 1
    assert checked > 0


@pytest.mark.parametrize("name", CASES)
def test_well_index(name):
    """Peaceman's WI and the derived kh of every perforation, from the cell
    and the well radius and skin, bit-identical (the decks give no WI or kh)."""
    for it, fx in iterations(name):
        conv = float(fx["conv_darcy"][0])
        for p in range(len(fx["perf_loc"])):
            wi, kh = W.well_index(int(fx["perf_dir"][p]), *(float(fx["perf_cell_" + k][p]) for k in
                                                            ("dx", "dy", "dz", "ntg", "kx", "ky", "kz")),
                                  float(fx["perf_radius"][p]), float(fx["perf_skin"][p]), conv)
            assert kh == float(fx["perf_kh"][p]), (it, p)
            assert wi == float(fx["perf_WI"][p]), (it, p)
