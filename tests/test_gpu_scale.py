"""The two largest workloads at full size on the GPU.

* The 4,000,000-cell corner-point Newton step (200 x 200 x 100, 9 components,
  20 wells, adjoint products in every step) that the bench times: the
  batched form's replayed graph bit-identical to the plain form (flash
  outputs, residual with the wells' rows, upwind choices, Jacobian rows,
  adjoint products), and the bench's own parity window (two layers with their
  ghost layers) against the oracle.
* The 1,048,576-cell batched-flash stress set (10 components, 20 % of the
  cells within 5 % of saturation): batched bit-identical to plain on every
  cell, and a 2,000-cell window against the oracle, phase labels exact except
  where the oracle itself changes them under one-ulp perturbations of its
  transcendentals.
"""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim, synthetic

pytestmark = pytest.mark.gpu

CELL_OUT = ("PHASE_EXIST", "S", "XI", "MU", "NT", "VF", "FTYPE", "FLASH_ITERS", "SKIP_FLAG", "KR", "PJ")
ROW_WINDOWS = ((0, 20000), (1990000, 2010000), (3980000, 4000000))


class _Args:
    large_dims = (200, 200, 100)
    cpu_layers = 5


def _step_outputs(ctx):
    out = {k: ctx.get(k) for k in CELL_OUT}
    out["RES"] = ctx.get("RES")
    out["UPBLOCK"] = ctx.get("UPBLOCK")
    for r0, r1 in ROW_WINDOWS:
        out[f"JAC{r0}"] = ctx.jacobian_rows(r0, r1)
        out[f"XIJ{r0}"] = ctx.get_range("XIJ", r0, r1 - r0)
        out[f"DSEC{r0}"] = ctx.get_range("DSEC_DPRI", r0, r1 - r0)
    out["ADJ"] = ctx.get_adjoint()
    out["WELLS"] = ctx.get_wells()
    return out


def test_large_step_batched_matches_plain_and_oracle(gpu_lib):
    import bench
    wl = bench.LargeWorkload(_Args())
    model, grid = wl.model(), wl.grid()
    outs = []
    for variant in (0, 1):
        ctx, _ = bench.prepare(wl, model, grid, variant, 0)
        try:
            ctx.checkpoint(0, restore=True)
            ctx.enqueue_step(bench.DT)
            ctx.step_report()
            outs.append(_step_outputs(ctx))
            if variant == 1:
                par = bench.parity(ctx, wl, model, grid)
        finally:
            ctx.close()
    a, b = outs
    for k in a:
        if k in ("ADJ", "WELLS") or k.startswith("JAC"):
            for x, y in zip(a[k], b[k]):
                assert np.array_equal(x, y), k
        else:
            assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert par["pass"], par
    assert par["residual_and_jacobian_rows_compared"] > 70000


FS_CELLS, FS_NCOMP, FS_SEED = 1 << 20, 10, 3


def test_flash_stress_batched_matches_plain_and_oracle(gpu_lib):
    from oracle.pyoracle import OracleBulk
    model = synthetic.comp_model(FS_NCOMP, FS_SEED)
    P_, Ni = synthetic.flash_stress_cells(lambda g: fim.FimContext(model, g, variant=1), FS_CELLS, FS_NCOMP,
                                          FS_SEED)
    grid = synthetic.flash_grid(FS_CELLS)
    st = synthetic.flash_state(P_, Ni, 71.85)
    keys = ("PHASE_EXIST", "S", "XIJ", "RHO", "XI", "MU", "RHOX", "XIX", "MUX", "VF", "VFP", "VFI", "NT",
            "DSEC_DPRI", "FTYPE", "FLASH_ITERS", "STATUS")
    outs = []
    for variant in (0, 1):
        with fim.FimContext(model, grid, variant=variant) as ctx:
            ctx.load_state(st)
            ctx.update_property()
            outs.append({k: ctx.get(k) for k in keys})
    for k in keys:
        assert np.array_equal(outs[0][k], outs[1][k], equal_nan=True), k
    # a window of cells, half of them from the near-saturation set
    n0, n1 = 500000, 502000
    win = slice(n0, n1)
    nc = model.nc
    sub_st = {k: np.asarray(v).reshape(FS_CELLS, -1)[win].ravel() for k, v in st.items()}
    sub_grid = synthetic.flash_grid(n1 - n0)

    def oracle(variant="exact", seed=None):
        ob = OracleBulk(model, sub_grid, variant=variant)
        if seed is not None:
            ob.set_nudge_seed(seed)
        ob.load(sub_st)
        ob.flash()
        return ob

    ob = oracle()
    pe_o = ob.a["phaseExist"].reshape(-1, 3).astype(bool)
    pe_g = outs[0]["PHASE_EXIST"].reshape(-1, 3)[win].astype(bool)
    nudged, sensitive = [], np.zeros(n1 - n0, bool)
    for seed in P.NUDGE_SEEDS:
        nz = oracle("ulp", seed)
        sensitive |= np.any(nz.a["phaseExist"].reshape(-1, 3).astype(bool) != pe_o, axis=1)
        nudged.append(nz)
    mismatch = np.any(pe_o != pe_g, axis=1)
    assert not np.any(mismatch & ~sensitive), np.nonzero(mismatch & ~sensitive)[0]
    keep = ~(mismatch | sensitive)
    names = {"S": "S", "XIJ": "xij", "RHO": "rho", "XI": "xi", "MU": "mu", "VF": "vf", "NT": "Nt",
             "RHOX": "rhox", "XIX": "xix", "MUX": "mux", "VFI": "vfi", "VFP": "vfP", "DSEC_DPRI": "dSec_dPri"}
    cut = lambda a: np.asarray(a).reshape(n1 - n0, -1)[keep]
    got = {names[k]: cut(np.asarray(outs[0][k]).reshape(FS_CELLS, -1)[win]) for k in names}
    got["phaseExist"] = cut(pe_g)
    ref = {v: cut(ob.a[v]) for v in names.values()}
    ref["phaseExist"] = cut(pe_o)
    nk = int(keep.sum())
    errs = P.state_errors(got, ref, nc, nk)
    sens = {}
    for nz in nudged:
        alt = {v: cut(nz.a[v]) for v in names.values()}
        alt["phaseExist"] = ref["phaseExist"]
        for k, v in P.state_errors(alt, ref, nc, nk).items():
            sens[k] = max(sens.get(k, 0.0), v)
    bad = {k: (v, P.tolerance(k, sens)) for k, v in errs.items() if v > P.tolerance(k, sens)}
    assert not bad, bad
