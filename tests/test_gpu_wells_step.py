"""Peaceman wells inside the device Newton step (ocpx_set_wells) against the
reference's own system and the oracle.

The golden wells_* fixtures hold, per Newton iteration, the reference's wells
(type, control, bhp, perforations, WI, dG, injected fluid, rate factors), its
full residual with the wells' rows (res_full) and its linear system before
and after AssembleMatWells (jac_*, jacw_*).  Here the wells are set once on a
context and every residual and Jacobian the device computes includes them:

* residual: the rows bit-identical to the oracle's wells added in the
  reference's order to the device's own bulk residual, and within the parity
  tolerance of the reference's res_full; the norms recomputed for the
  perforated rows; maxWellRelRes_mol;
* Jacobian: the reference's block-CSR pattern with the wells' rows and
  columns exactly (block order included); bulk rows normwise within 1e-10
  (the reference multiplies dF/dXs by dSec_dPri with BLAS dgemm), the wells'
  rows within 1e-13 per block, the bulk-to-well blocks bit-identical;
* the batched form's replayed graph bit-identical to the eager plain path;
  the Newton update of the wells' bhp and its checkpoint; the device linear
  solve of the full system against a direct solve; J^T lambda with the
  wells' rows against the transposed matrix;
* a cell perforated more than once.
"""
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


def _device_norms(res, rockVp, Nt, nb, ncol):
    r = np.abs(res.reshape(-1, ncol)[:nb])
    return float(np.max(r / rockVp[:, None])), float(np.max(r[:, 1:] / Nt[:, None]))


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_in_step_residual(gpu_lib, wname, fname):
    fx = P.load_fixture(fname)
    model, grid = fim.model_and_grid_from_dump(fx)
    checked = 0
    with fim.FimContext(model, grid) as bulk, fim.FimContext(model, grid) as ctx:
        for it, fw in _iterations(wname):
            post = P.group(fx, it + "/post")
            if "P" not in post:
                continue
            dt = float(fw["dt"][0])
            wells, nc, np_ = W.split_wells(fw)
            ncol = nc + 1
            bulk.load_state(post)
            bulk.cal_res(dt)
            ref, ref_mrel = W.residual_with_wells(bulk.get("RES"), wells, fw, dt, nc, np_)
            ctx.load_state(post)
            ctx.set_wells(_api_wells(wells))
            norms = ctx.cal_res(dt)
            res = ctx.get("RES")
            assert res.size == (grid.nb + len(wells)) * ncol
            bad = np.nonzero(np.any(res.reshape(-1, ncol) != ref.reshape(-1, ncol), axis=1))[0]
            assert bad.size == 0, f"{it}: rows {bad}"
            bhp, mrel = ctx.get_wells()
            assert mrel == ref_mrel, it
            assert np.array_equal(bhp, [w["bhp"] for w in wells])
            # the norms, with the perforated rows recomputed
            rockVp, Nt = ctx.get("ROCKVP"), ctx.get("NT")
            assert (norms.maxRelRes_V, norms.maxRelRes_N) == _device_norms(res, rockVp, Nt, grid.nb, ncol), it
            # and the reference's own residual with its wells
            rf = np.asarray(fw["res_full"], np.float64)
            assert P.res_err(res[:grid.nb * ncol], rf[:grid.nb * ncol], post["rockVp"], post["Nt"], nc) <= P.REL_TOL
            wr, wf = res[grid.nb * ncol:], rf[grid.nb * ncol:]
            assert np.all(np.abs(wr - wf) <= P.REL_TOL * np.abs(wf)), it
            assert abs(mrel - float(fw["maxWellRelRes_mol"][0])) <= P.REL_TOL * max(abs(mrel), 1e-300), it
            checked += 1
    assert checked > 0


def _blocks(rowptr, col, val, ncol):
    bs = ncol * ncol
    return [(r, int(col[e]), np.asarray(val[e * bs:(e + 1) * bs]).reshape(ncol, ncol))
            for r in range(len(rowptr) - 1) for e in range(int(rowptr[r]), int(rowptr[r + 1]))]


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_in_step_jacobian(gpu_lib, wname, fname):
    fx = P.load_fixture(fname)
    model, grid = fim.model_and_grid_from_dump(fx)
    checked = 0
    with fim.FimContext(model, grid) as ctx:
        for it, fw in _iterations(wname):
            jac = {k.split("/", 1)[1]: v for k, v in fw.items() if k.startswith("jac/")}
            if not jac:
                continue
            wells, nc, np_ = W.split_wells(jac)
            ncol, nb = nc + 1, grid.nb
            dt = float(jac["dt"][0])
            ctx.load_state(P.jac_state(fx, it))
            ctx.load_state(jac)
            ctx.set_wells(_api_wells(wells))
            ctx.cal_res(dt)
            ctx.assemble_mat(dt)
            rp, col, val = ctx.jacobian()
            assert np.array_equal(rp, jac["jacw_rowptr"]) and np.array_equal(col, jac["jacw_col"]), it
            got = _blocks(rp, col, val, ncol)
            ref = _blocks(jac["jacw_rowptr"], jac["jacw_col"], jac["jacw_val"], ncol)
            bs = ncol * ncol
            for r in range(nb):     # bulk rows: normwise (dgemm in the reference)
                a = val[rp[r] * bs:rp[r + 1] * bs]
                b = jac["jacw_val"][rp[r] * bs:rp[r + 1] * bs]
                assert np.linalg.norm(a - b) <= P.REL_TOL * np.linalg.norm(b), (it, r)
            for (r, c, a), (_, _, b) in zip(got, ref):
                if r < nb and c >= nb:
                    assert np.array_equal(a, b), (it, r, c)          # bulk-to-well: dt * dQ/dP_well
                elif r >= nb:
                    assert np.linalg.norm(a - b) <= 1e-13 * max(np.linalg.norm(b), 1e-300) or \
                        (not np.any(a) and not np.any(b)), (it, r, c)
            checked += 1
    assert checked > 0


def _case(wname, fname):
    fx = P.load_fixture(fname)
    model, grid = fim.model_and_grid_from_dump(fx)
    it, fw = _iterations(wname)[0]
    wells, nc, _ = W.split_wells(fw)
    return fx, model, grid, it, fw, _api_wells(wells), nc


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_in_graph_step_and_update(gpu_lib, wname, fname):
    """The batched form's replayed step with the wells equals the eager plain
    path, replay after replay; the Newton update moves each well's bhp by its
    row of u and a checkpoint restores it."""
    fx, model, grid, it, fw, wells, nc = _case(wname, fname)
    post = P.group(fx, it + "/post")
    dt = float(fw["dt"][0])
    ncol = nc + 1
    outs = []
    for variant in (0, 1):
        with fim.FimContext(model, grid, variant=variant) as ctx:
            ctx.load_state(post)
            ctx.set_wells(wells)
            ctx.checkpoint(0)
            got = []
            for rep in range(2):
                ctx.checkpoint(0, restore=True)
                ctx.enqueue_step(dt)
                ctx.step_report()
                got.append((ctx.get("RES"), ctx.jacobian()[2]))
            assert all(np.array_equal(g[0], got[0][0]) and np.array_equal(g[1], got[0][1]) for g in got)
            # Newton update with the wells' rows
            u = np.zeros(ctx.nv)
            du = np.arange(1, len(wells) + 1, dtype=np.float64) * 0.5
            u[grid.nb * ncol::ncol] = du
            bhp0 = ctx.get_wells()[0]
            ctx.get_solution(u, 0.2)
            assert np.array_equal(ctx.get_wells()[0], bhp0 + du)
            ctx.checkpoint(0, restore=True)
            assert np.array_equal(ctx.get_wells()[0], bhp0)
            outs.append(got[0])
    bad = np.nonzero(outs[0][0] != outs[1][0])[0]
    assert bad.size == 0, f"residual entries {bad[:20]} (rows {np.unique(bad // ncol)[:20]}) of {outs[0][0].size}: " \
                          f"{outs[0][0][bad[:5]]} vs {outs[1][0][bad[:5]]}"
    assert np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("wname,fname", CASES)
def test_wells_linsolve_and_adjoint(gpu_lib, wname, fname):
    """The device solve covers the wells' rows (against a direct solve of the
    assembled system); J^T lambda covers their rows and columns (against the
    transposed matrix)."""
    from scipy.sparse import bsr_matrix
    from scipy.sparse.linalg import spsolve
    fx, model, grid, it, fw, wells, nc = _case(wname, fname)
    dt = float(fw["dt"][0])
    dim = nc + 1
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(P.group(fx, it + "/post"))
        ctx.set_wells(wells)
        ctx.cal_res(dt)
        ctx.assemble_mat(dt)
        rp, col, val = ctx.jacobian()
        n = ctx.nv
        J = bsr_matrix((val.reshape(-1, dim, dim), col, rp), shape=(n, n)).tocsr()
        rhs = ctx.get("RES")
        ref = spsolve(J, rhs)
        u, rep = ctx.linsolve(tol=1e-12, maxit=4000)
        assert rep["converged"], rep
        assert np.linalg.norm(J @ u - rhs) <= 1e-9 * np.linalg.norm(rhs)
        assert np.linalg.norm(u - ref) <= 1e-6 * np.linalg.norm(ref)
        lam = np.random.default_rng(3).normal(size=n)
        jt, _, _ = ctx.adjoint(lam, trans=False, poro=False)
        assert np.linalg.norm(jt - J.T @ lam) <= 1e-13 * np.linalg.norm(J.T @ lam)


def test_wells_in_step_refusals(gpu_lib):
    fx, model, grid, it, fw, wells, nc = _case(*CASES[0])
    dt = float(fw["dt"][0])
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(P.group(fx, it + "/post"))
        bad = dict(wells[0], cell=[grid.nb])
        with pytest.raises(fim.OcpxError, match="out of range"):
            ctx.set_wells([bad])
        ctx.set_wells(wells)
        ctx.cal_res(dt)
        with pytest.raises(fim.OcpxError, match="holds wells"):
            ctx.wells_eval(wells, dt)
        # the same perforations: data only; none: the bulk system again
        ctx.set_wells([dict(w, bhp=w["bhp"] + 1.0) for w in wells])
        assert np.array_equal(ctx.get_wells()[0], [w["bhp"] + 1.0 for w in wells])
        ctx.set_wells([])
        ctx.cal_res(dt)
        assert ctx.get("RES").size == grid.nb * (nc + 1)
        with pytest.raises(fim.OcpxError, match="INVALID_ARG"):
            ctx.get_wells()


def test_cell_perforated_more_than_once(gpu_lib):
    """A cell perforated twice by one well and once more by another: its
    residual rows get the three perforations' rates in well then perforation
    order (bit-identical to the oracle's), its diagonal block the three
    additions in that order, and its row one bulk-to-well block per
    perforation (against the per-perforation blocks of ocpx_wells_eval)."""
    fx, model, grid, it, fw, wells, nc = _case(*CASES[1])
    post = P.group(fx, it + "/post")
    dt = float(fw["dt"][0])
    ncol, nb = nc + 1, grid.nb
    w0, w1 = wells
    c = int(np.ravel(w0["cell"])[0])

    def plus(w, scale):
        r = lambda k: np.ravel(w[k])
        return dict(w, cell=np.r_[r("cell"), c], WI=np.r_[r("WI"), scale * r("WI")[0]], dG=np.r_[r("dG"), r("dG")[0]],
                    xi_inj=np.r_[r("xi_inj"), r("xi_inj")[0]])

    twice = [plus(w0, 0.7), plus(w1, 1.3)]
    with fim.FimContext(model, grid) as bulk, fim.FimContext(model, grid) as ctx:
        bulk.load_state(post)
        bulk.cal_res(dt)
        ow = [dict(type=w["type"], mode=w["mode"], bhp=w["bhp"], tar_bhp=w["tar_bhp"], tar_rate=w["tar_rate"],
                   factor=w["factor"], inj_zi=w["inj_zi"], loc=np.ravel(w["cell"]), WI=np.ravel(w["WI"]),
                   mult=np.ones(np.ravel(w["cell"]).size), dG=np.ravel(w["dG"]), xi_inj=np.ravel(w["xi_inj"]))
              for w in twice]
        ref, _ = W.residual_with_wells(bulk.get("RES"), ow, fw, dt, nc, 3)
        bulk.assemble_mat(dt)
        rp_b, col_b, val_b = bulk.jacobian()
        _, pb, _, _ = bulk.wells_eval(twice, dt, residual=False)
        ctx.load_state(post)
        ctx.set_wells(twice)
        ctx.cal_res(dt)
        assert np.array_equal(ctx.get("RES"), ref)
        ctx.assemble_mat(dt)
        rp, col, val = ctx.jacobian()
        bs = ncol * ncol
        perfs = [q for q, cell in enumerate(np.r_[np.ravel(twice[0]["cell"]), np.ravel(twice[1]["cell"])])
                 if cell == c]
        assert len(perfs) == 3
        diag = val_b[rp_b[c] * bs:(rp_b[c] + 1) * bs].copy()
        for q in perfs:
            diag = diag + pb[q, 0].ravel()
        assert np.linalg.norm(val[rp[c] * bs:(rp[c] + 1) * bs] - diag) <= 1e-13 * np.linalg.norm(diag)
        n_conn = int(rp_b[c + 1] - rp_b[c] - 1)
        assert rp[c + 1] - rp[c] == 1 + n_conn + 3
        assert np.array_equal(col[rp[c] + 1 + n_conn:rp[c + 1]], [nb, nb, nb + 1])
        for k, q in enumerate(perfs):
            e = rp[c] + 1 + n_conn + k
            assert np.array_equal(val[e * bs:(e + 1) * bs].reshape(ncol, ncol), pb[q, 1])
