"""The 200,000-cell compositional case (100 x 100 x 20, 8 seeded components,
layered lognormal permeability: median 200 mD, sigma_ln 1.5, correlation
length 10 cells) on the GPU, through properties that do not need the
reference at this size:

* the batched form is bit-identical to the plain form (flash outputs,
  residual, Jacobian values);
* the flash of a 2,000-cell window and the residual and Jacobian of the whole
  grid agree with the oracle (the CPU restatement pinned to the reference) on
  the same inputs, within the parity tolerances;
* the adjoint (dR/dT)^T lambda matches central differences on 256 seeded
  connections, and J^T lambda matches the transpose of the assembled Jacobian.

and, with eight vertical Peaceman wells (two under a rate target) set on the
device, the replayed graph of the batched form bit-identical to the plain
path, the residual with the wells bit-identical to the oracle's wells added
to the device's own bulk residual, and the Newton update of the wells' bhp.
"""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim, synthetic

pytestmark = pytest.mark.gpu

NX, NY, NZ, NCOMP, SEED = 100, 100, 20, 8, 4
DT, DSMAX = 0.1, 0.2
FLASH_OUT = ("PHASE_EXIST", "S", "XIJ", "RHO", "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "VF", "VFP",
             "VFI", "NT", "DSEC_DPRI", "FTYPE", "FLASH_ITERS", "STATUS", "SKIP_FLAG", "SKIP_MINEIG")
STATE_FIELDS = [f for f in fim.FIELDS if f not in ("STATUS", "FTYPE", "FLASH_ITERS", "UPBLOCK", "CONN_DP", "FLUX_VJ",
                                                   "FLUX_NI", "RES", "RES_REL_V", "RES_REL_N", "TRANS", "PORO_INIT")]


@pytest.fixture(scope="module")
def case(gpu_lib):
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid_lognormal(NX, NY, NZ, median=200.0, sigma_ln=1.5, corr_cells=10, seed=SEED)
    out = {}
    for variant in (0, 1):
        ctx = fim.FimContext(model, grid, variant=variant)
        synthetic.ptn_workload(ctx, grid, NCOMP, SEED, dt=DT, dsmax=DSMAX)
        ctx.checkpoint(0)
        inputs = {f: ctx.get(f) for f in STATE_FIELDS}
        ctx.update_property()
        ctx.cal_res(DT)
        ctx.assemble_mat(DT)
        res = {k: ctx.get(k) for k in FLASH_OUT}
        res["RES"] = ctx.get("RES")
        res["JAC"] = ctx.jacobian()[2]
        out[variant] = dict(ctx=ctx, inputs=inputs, res=res)
    yield model, grid, out
    for v in out.values():
        v["ctx"].close()


def test_large_batched_matches_plain(case):
    _, _, out = case
    a, b = out[0]["res"], out[1]["res"]
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("params", [dict(fused_blocks=0, flash_budget=8, rounds=3, round_growth=4, cell_blocks=152,
                                         pre_blocks=38),
                                    dict(fused_blocks=0),
                                    dict(fused_blocks=152, flash_budget=8, coop_cells=0),
                                    dict(fused_blocks=608, flash_budget=24),
                                    dict(fused_blocks=152, fused_coop_blocks=38, flash_budget=24),
                                    dict(fused_blocks=152, fused_coop_blocks=57, fused_excl=0, post_block=32)],
                         ids=["rounds+persistent+exclusive", "two-stream", "fused-exclusive", "fused-shared",
                              "fused-roles", "fused-roles-l1"])
def test_large_batched_launch_forms_match_plain(case, params):
    """Re-budgeting rounds, the persistent per-cell kernel, SM-exclusive
    pre-deferral blocks and the fused kernel at 200,000 cells: the flash
    stays bit-identical."""
    _, _, out = case
    ctx = out[1]["ctx"]
    keep = {k: ctx.get_param(k) for k in ("flash_budget", "rounds", "round_growth", "cell_blocks", "pre_blocks",
                                          "fused_blocks", "coop_cells", "fused_coop_blocks", "fused_excl", "post_block")}
    try:
        for k, v in params.items():
            ctx.set_param(k, v)
        ctx.checkpoint(0, restore=True)
        ctx.update_property()
        assert ctx.get_param("deferred") > 0
        for k in FLASH_OUT:
            assert np.array_equal(out[0]["res"][k], ctx.get(k), equal_nan=True), k
    finally:
        for k, v in keep.items():
            ctx.set_param(k, v)


def fim_to_ref(field):
    """Field name of the library -> BulkVarSet name (the oracle's)."""
    inv = {v: k for k, v in fim.REF_NAMES.items()}
    return inv.get(field)


def _oracle_with(model, grid, fields):
    from oracle.pyoracle import OracleBulk
    ob = OracleBulk(model, grid)
    ob.load({fim_to_ref(k): v for k, v in fields.items() if fim_to_ref(k)})
    return ob


def test_large_flash_window_against_oracle(case):
    """A 2,000-cell window flashed by the oracle from the GPU's own inputs;
    tolerances from the one-ulp sensitivity of the oracle on the same window."""
    from oracle.pyoracle import OracleBulk
    model, grid, out = case
    n0, n1 = 50000, 52000
    keys = ("phaseExist", "S", "xij", "rho", "xi", "mu", "rhoP", "xiP", "muP", "rhox", "xix", "mux", "vf", "vfP",
            "vfi", "Nt", "dSec_dPri")
    got = {fim_to_ref(k): v for k, v in out[0]["res"].items() if fim_to_ref(k)}
    cut = lambda a: np.asarray(a).reshape(grid.nb, -1)[n0:n1].ravel()
    mine = {k: cut(got[k]) for k in keys}

    def oracle_window(variant="exact", seed=None):
        ob = OracleBulk(model, grid, variant=variant)
        if seed is not None:
            ob.set_nudge_seed(seed)
        ob.load({fim_to_ref(k): v for k, v in out[0]["inputs"].items() if fim_to_ref(k)})
        ob.flash(n0, n1)
        return {k: cut(ob.a[k]) for k in keys}

    ref = oracle_window()
    assert np.array_equal(mine["phaseExist"].astype(np.uint32), ref["phaseExist"])
    errs = P.state_errors(mine, ref, model.nc, n1 - n0)
    sens = {}
    for seed in P.NUDGE_SEEDS:
        nudged = oracle_window("ulp", seed)
        if not np.array_equal(nudged["phaseExist"], ref["phaseExist"]):
            continue
        for k, v in P.state_errors(nudged, ref, model.nc, n1 - n0).items():
            sens[k] = max(sens.get(k, 0.0), v)
    bad = {k: (v, P.tolerance(k, sens)) for k, v in errs.items() if v > P.tolerance(k, sens)}
    assert not bad, bad


def test_large_residual_and_jacobian_against_oracle(case):
    model, grid, out = case
    ctx = out[0]["ctx"]
    # the oracle assembles from the GPU's own post-flash state: this isolates flux, residual and Jacobian
    post = {f: ctx.get(f) for f in STATE_FIELDS}
    ob = _oracle_with(model, grid, post)
    ob.cal_res(DT)
    rp, col, val = ob.assemble(DT)
    assert np.array_equal(ctx.get("UPBLOCK"), ob.conn["upblock"])
    assert P.res_err(ctx.get("RES"), ob.res, post["ROCKVP"], post["NT"], model.nc) <= P.REL_TOL
    g_rp, g_col, g_val = ctx.jacobian()
    assert np.array_equal(g_rp, rp) and np.array_equal(g_col, col)
    bs = (model.nc + 1) ** 2
    a = g_val.reshape(-1, bs)
    b = val.reshape(-1, bs)
    # normwise per block row
    num = np.sqrt(np.add.reduceat(np.sum((a - b) ** 2, axis=1), rp[:-1]))
    den = np.sqrt(np.add.reduceat(np.sum(b ** 2, axis=1), rp[:-1]))
    assert np.max(num / np.maximum(den, 1e-300)) <= P.REL_TOL


def test_large_adjoint(case):
    from scipy.sparse import bsr_matrix
    model, grid, out = case
    ctx = out[0]["ctx"]
    dim = model.nc + 1
    rng = np.random.default_rng(21)
    lam = rng.normal(size=grid.nb * dim)
    jt, g, _ = ctx.adjoint(lam, poro=False)
    rp, col, val = ctx.jacobian()
    J = bsr_matrix((val.reshape(-1, dim, dim), col, rp), shape=(grid.nb * dim, grid.nb * dim))
    ref = J.T @ lam
    assert np.linalg.norm(jt - ref) <= 1e-12 * np.linalg.norm(ref)
    T0 = ctx.get("TRANS").copy()
    errs = []
    for c in rng.choice(grid.nconn, size=256, replace=False):
        h = 1e-6 * T0[c]
        rr = []
        for sgn in (1, -1):
            T = T0.copy()
            T[c] = T0[c] + sgn * h
            ctx.set("TRANS", T)
            ctx.cal_res(DT)
            rr.append(ctx.get("RES"))
        fd = lam @ (rr[0] - rr[1]) / (2 * h)
        errs.append(abs(fd - g[c]) / max(abs(g[c]), abs(fd), 1e-9 * np.max(np.abs(g))))
    ctx.set("TRANS", T0)
    assert max(errs) <= 1e-6, max(errs)


def test_large_wells_in_step(gpu_lib):
    from oracle import wells as W
    from opencaeporox_gb300 import wells as WL
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid_lognormal(NX, NY, NZ, median=200.0, sigma_ln=1.5, corr_cells=10, seed=SEED)
    k = np.full(grid.nb, 200.0)
    wl = WL.vertical_wells(NX, NY, NZ, 4, 4, 20.0, 5.0, k, 0.1 * k, grid.depth, NCOMP, SEED, n_rate=2)
    nb, nc = grid.nb, model.nc
    out = {}
    for variant in (0, 1):
        with fim.FimContext(model, grid, variant=variant) as ctx:
            synthetic.ptn_workload(ctx, grid, NCOMP, SEED, dt=DT, dsmax=DSMAX)
            ctx.set_wells(wl)
            ctx.checkpoint(0)
            for rep in range(2):  # a replay from the checkpoint repeats the first
                ctx.checkpoint(0, restore=True)
                ctx.enqueue_step(DT)
                ctx.step_report()
                got = dict(RES=ctx.get("RES"), JAC=ctx.jacobian()[2], WELLS=ctx.get_wells())
                if rep:
                    assert np.array_equal(got["RES"], first["RES"]) and np.array_equal(got["JAC"], first["JAC"])
                first = got
            state = {name: ctx.get(f) for name, f in (("P", "P"), ("Pj", "PJ"), ("kr", "KR"), ("mu", "MU"),
                                                      ("xi", "XI"), ("xij", "XIJ"), ("phaseExist", "PHASE_EXIST"))}
            u = np.zeros(ctx.nv)
            u[nb * (nc + 1)::nc + 1] = np.arange(1, len(wl) + 1) * 0.25
            bhp0 = got["WELLS"][0]
            ctx.get_solution(u, DSMAX)
            assert np.array_equal(ctx.get_wells()[0], bhp0 + np.arange(1, len(wl) + 1) * 0.25)
            out[variant] = (got, state)
    (a, _), (b, state) = out[0], out[1]
    assert np.array_equal(a["RES"], b["RES"]) and np.array_equal(a["JAC"], b["JAC"])
    assert np.array_equal(a["WELLS"][0], b["WELLS"][0]) and a["WELLS"][1] == b["WELLS"][1]
    # the bulk residual of the same post-flash state without wells, plus the
    # oracle's wells in the reference's order
    with fim.FimContext(model, grid, variant=0) as bulk:
        synthetic.ptn_workload(bulk, grid, NCOMP, SEED, dt=DT, dsmax=DSMAX)
        bulk.update_property()
        bulk.cal_res(DT)
        res_bulk = bulk.get("RES")
    wells_o = [dict(type=w["type"], mode=w["mode"], bhp=w["bhp"], tar_bhp=w["tar_bhp"], tar_rate=w["tar_rate"],
                    factor=np.asarray(w["factor"]), inj_zi=np.asarray(w["inj_zi"]), loc=np.asarray(w["cell"]),
                    WI=np.asarray(w["WI"]), mult=np.ones(len(w["cell"])), dG=np.asarray(w["dG"]),
                    xi_inj=np.asarray(w["xi_inj"])) for w in wl]
    ref, ref_mrel = W.residual_with_wells(res_bulk, wells_o, state, DT, nc, 3)
    bad = np.nonzero(b["RES"] != np.asarray(ref))[0]
    assert bad.size == 0, f"residual entries {bad[:10]}"
    assert b["WELLS"][1] == ref_mrel
