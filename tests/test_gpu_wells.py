"""Peaceman wells on the device (ocpx_wells_eval) against the oracle and the
reference: the residual with the wells and maxWellRelRes_mol against the
oracle's on the device's own bulk residual (rows without a perforation
bit-identical, the others within 1e-12 of the row's scale: the library's host
code sums them uncontracted, as the oracle does, and the margin covers a host
compiler that would fuse a*b + c, which moves a row by up to 5e-13 here); the blocks the
wells add to the system against the reference's system before and after its
wells' assembly (bit-identical cell-to-well blocks and well diagonals, the
blocks that carry dQ/dXs * dSec_dPri within 1e-13 normwise)."""
import os

import numpy as np
import pytest

import parity as P
from oracle import wells as W
from opencaeporox_gb300 import fim

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [("wells_bo_10x10x3", "bo_10x10x3"), ("wells_comp6_8x8x3", "comp6_8x8x3")]


def _iterations(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    its = sorted({k.split("/")[0] for k in z.files if k.startswith("it")})
    return [(it, {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(it + "/")}) for it in its]


def _api_wells(wells):
    return [dict(type=w["type"], mode=w["mode"], bhp=w["bhp"], tar_bhp=w["tar_bhp"], tar_rate=w["tar_rate"],
                 cell=w["loc"], WI=np.asarray(w["WI"]) * np.asarray(w["mult"]), dG=w["dG"], xi_inj=w["xi_inj"],
                 inj_zi=w["inj_zi"], factor=w["factor"]) for w in wells]


def _blocks(rowptr, col, val, ncol):
    bs = ncol * ncol
    return {(r, int(col[e])): np.asarray(val[e * bs:(e + 1) * bs]).reshape(ncol, ncol)
            for r in range(len(rowptr) - 1) for e in range(int(rowptr[r]), int(rowptr[r + 1]))}


def _close(a, b, tol=1e-13):
    return np.linalg.norm(a - b) <= tol * max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_residual(gpu_lib, wname, fname):
    fx = P.load_fixture(fname)
    model, grid = fim.model_and_grid_from_dump(fx)
    checked = 0
    with fim.FimContext(model, grid) as ctx:
        for it, fw in _iterations(wname):
            post = P.group(fx, it + "/post")
            if "P" not in post:
                continue
            ctx.load_state(post)
            dt = float(fw["dt"][0])
            ctx.cal_res(dt)
            wells, nc, np_ = W.split_wells(fw)
            res, _, _, mrel = ctx.wells_eval(_api_wells(wells), dt)
            ref, ref_mrel = W.residual_with_wells(ctx.get("RES"), wells, fw, dt, nc, np_)
            ncol = nc + 1
            rows_res, rows_ref = res.reshape(-1, ncol), ref.reshape(-1, ncol)
            touched = set(int(c) for w in wells for c in np.asarray(w["loc"]).tolist())
            touched |= set(range(grid.nb, grid.nb + len(wells)))
            for r in range(len(rows_ref)):
                if r in touched:
                    assert np.linalg.norm(rows_res[r] - rows_ref[r]) <= 1e-12 * max(
                        np.linalg.norm(rows_ref[r]), 1e-300), (it, r)
                else:
                    assert np.array_equal(rows_res[r], rows_ref[r]), (it, r)
            assert abs(mrel - ref_mrel) <= 1e-12 * max(abs(ref_mrel), 1e-300), it
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_jacobian_blocks(gpu_lib, wname, fname):
    fx = P.load_fixture(fname)
    model, grid = fim.model_and_grid_from_dump(fx)
    checked = 0
    with fim.FimContext(model, grid) as ctx:
        for it, fw in _iterations(wname):
            jac = {k.split("/", 1)[1]: v for k, v in fw.items() if k.startswith("jac/")}
            if not jac:
                continue
            ctx.load_state(jac)
            wells, nc, np_ = W.split_wells(jac)
            ncol = nc + 1
            nb = len(jac["jac_rowptr"]) - 1
            _, pb, wd, _ = ctx.wells_eval(_api_wells(wells), float(jac["dt"][0]), residual=False)
            before = _blocks(jac["jac_rowptr"], jac["jac_col"], jac["jac_val"], ncol)
            after = _blocks(jac["jacw_rowptr"], jac["jacw_col"], jac["jacw_val"], ncol)
            q = 0
            diag = {}   # a cell's diagonal gets every perforation's addition, in well then perforation order
            for wi, w in enumerate(wells):
                for n in np.asarray(w["loc"]).tolist():
                    diag[n] = diag.get(n, before[(n, n)]) + pb[q, 0]
                    assert np.array_equal(after[(n, nb + wi)], pb[q, 1]), (it, n)
                    blk = after[(nb + wi, n)]
                    assert _close(blk, pb[q, 2]) or (not np.any(blk) and not np.any(pb[q, 2])), (it, n)
                    q += 1
                assert np.array_equal(after[(nb + wi, nb + wi)], wd[wi]), (it, wi)
            for n, d in diag.items():
                assert _close(after[(n, n)], d), (it, n)
            checked += 1
    assert checked > 0


def test_wells_refuse_bad_input(gpu_lib):
    fx = P.load_fixture("bo_10x10x3")
    model, grid = fim.model_and_grid_from_dump(fx)
    with fim.FimContext(model, grid) as ctx:
        w = dict(type=1, mode=0, bhp=100.0, tar_bhp=100.0, tar_rate=0.0, cell=[grid.nb], WI=[1.0], dG=[0.0])
        with pytest.raises(fim.OcpxError, match="out of range"):
            ctx.wells_eval([w], 1.0)
        w = dict(type=1, mode=1, bhp=100.0, tar_bhp=100.0, tar_rate=0.0, cell=[0], WI=[1.0], dG=[0.0])
        with pytest.raises(fim.OcpxError, match="rate data"):
            ctx.wells_eval([w], 1.0)
