"""The timed path of the Newton step, checked for parity.

The bench times ``ocpx_enqueue_step`` of the batched form: the whole Newton
iteration (properties, residual, Jacobian) captured once into a CUDA graph and
replayed, with the launch parameters the autotuner picks.  Its end-to-end
figure times ``ocpx_step``: a host Newton update in, the host residual and
Jacobian values out.  Both replace the reference's IsoT_FIM::UpdateProperty +
CalRes + AssembleMat (src/IsoThermalMethod.cpp:742-752, 811-836); this file
checks that what they compute is what the eager plain path computes, bit for
bit, and what the reference computed, at the parity tolerances:

* graph replays from a device checkpoint, several in a row, after a launch
  parameter change (which forces a new capture) and after a dt change;
* the cooperative fused launch and the two-stream form inside a graph;
* ocpx_step with host buffers, in both forms;
* the 36,000-cell bench state with autotuned parameters against the plain
  eager step and against the oracle run from the same inputs.
"""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim, synthetic

pytestmark = pytest.mark.gpu

FIXTURES = ["comp6_8x8x3", "comp8_6x6x4"]
STEP_OUT = ("PHASE_EXIST", "S", "XIJ", "RHO", "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "DSEC_DPRI",
            "VF", "VFP", "VFI", "NT", "FTYPE", "FLASH_ITERS", "STATUS", "SKIP_FLAG", "SKIP_MINEIG", "SKIP_P",
            "SKIP_ZI", "KR", "PC", "PJ", "DKRDS", "DPCDS", "PORO", "POROP", "ROCKVP", "UPBLOCK", "CONN_DP",
            "FLUX_VJ", "FLUX_NI", "RES", "RES_REL_V", "RES_REL_N")
FORMS = {
    "defaults": {},
    "fused-roles": dict(fused_blocks=3, fused_coop_blocks=1, flash_budget=3, coop_cells=0, predefer=1),
    "two-stream": dict(fused_blocks=0, flash_budget=3, coop_cells=0, predefer=1),
    "split-refill": dict(split_refill=1),
    "split-refill-predefer": dict(split_refill=1, flash_budget=3, coop_cells=0, predefer=1),
}


def first_it(fx):
    return [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")][0]


def outputs(ctx):
    out = {k: ctx.get(k) for k in STEP_OUT}
    out["JAC"] = ctx.jacobian()[2]
    return out


def same(a, b, what):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), f"{what}: {k} differs"


def eager_step(model, grid, state, dt):
    """The plain per-kernel path, one call per reference loop."""
    with fim.FimContext(model, grid, variant=0) as ctx:
        for s in state:
            ctx.load_state(s)
        ctx.update_property()
        ctx.cal_res(dt)
        ctx.assemble_mat(dt)
        return outputs(ctx)


def graph_step(ctx, dt):
    ctx.enqueue_step(dt)
    ctx.step_report()
    return outputs(ctx)


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("form", list(FORMS))
def test_graph_replay_matches_eager_and_reference(gpu_lib, name, form):
    fx = P.load_fixture(name)
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    pre, post = P.group(fx, it + "/pre"), P.group(fx, it + "/post")
    dt = float(pre["dt"][0])
    state = [P.jac_state(fx, it), pre]
    ref = eager_step(model, grid, state, dt)
    ref_half = eager_step(model, grid, state, 0.5 * dt)
    with fim.FimContext(model, grid, variant=1) as ctx:
        for k, v in FORMS[form].items():
            ctx.set_param(k, v)
        for s in state:
            ctx.load_state(s)
        ctx.checkpoint(0)
        got = graph_step(ctx, dt)                       # capture, then one replay
        same(got, ref, "first graph step")
        per_step = None
        for rep in range(3):                            # replays of the same graph
            ctx.checkpoint(0, restore=True)
            n0 = ctx.launch_count
            same(graph_step(ctx, dt), ref, f"replay {rep}")
            n = ctx.launch_count - n0
            assert per_step is None or n == per_step    # the same graph each time
            per_step = n
        ctx.set_param("flash_budget", ctx.get_param("flash_budget") + 5)  # a new capture
        ctx.checkpoint(0, restore=True)
        same(graph_step(ctx, dt), ref, "after a parameter change")
        ctx.checkpoint(0, restore=True)
        same(graph_step(ctx, 0.5 * dt), ref_half, "after a dt change")
        ctx.checkpoint(0, restore=True)
        same(graph_step(ctx, dt), ref, "back to the first dt")
    # the replayed step against the reference's own iteration
    nb = grid.nb
    assert np.array_equal(got["PHASE_EXIST"], post["phaseExist"].astype(np.uint8))
    assert np.array_equal(got["UPBLOCK"], post["upblock"])
    assert P.res_err(got["RES"], post["res_bulk"], post["rockVp"], post["Nt"], model.nc) <= P.REL_TOL
    names = {"S": "S", "XIJ": "xij", "RHO": "rho", "XI": "xi", "MU": "mu", "VF": "vf", "NT": "Nt",
             "PHASE_EXIST": "phaseExist", "DSEC_DPRI": "dSec_dPri", "VFI": "vfi", "VFP": "vfP"}
    errs = P.state_errors({names[k]: got[k] for k in names}, post, model.nc, nb)
    sens = P.libm_sensitivity(dict(fx, __name__=name), it, model, grid)
    bad = {k: (v, P.tolerance(k, sens)) for k, v in errs.items() if v > P.tolerance(k, sens)}
    assert not bad, bad


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("variant", [0, 1])
def test_step_with_host_buffers(gpu_lib, name, variant):
    """ocpx_step: the Newton update u from a host buffer, then properties,
    residual and Jacobian, with the residual and Jacobian values copied to
    host buffers: equal to the eager calls, twice in a row from a checkpoint,
    and to the reference's iteration (its Jacobian is checked against the
    reference's in test_gpu_parity.test_jacobian)."""
    fx = P.load_fixture(name)
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    js, pre, post = P.jac_state(fx, it), P.group(fx, it + "/pre"), P.group(fx, it + "/post")
    dt, dsmax, u = float(pre["dt"][0]), float(pre["dSmax"][0]), np.ascontiguousarray(pre["u"], np.float64)
    with fim.FimContext(model, grid, variant=0) as e:
        e.load_state(js)
        e.get_solution(u, dsmax)
        e.update_property()
        e.cal_res(dt)
        e.assemble_mat(dt)
        ref = outputs(e)
    with fim.FimContext(model, grid, variant=variant) as ctx:
        ctx.load_state(js)
        ctx.checkpoint(1)
        bs = (model.nc + 1) ** 2
        for rep in range(2):
            ctx.checkpoint(1, restore=True)
            res = np.full(grid.nb * (model.nc + 1), np.nan)
            jac = np.full(ref["JAC"].size, np.nan)
            ctx.step(u=u, dSmax=dsmax, dt=dt, res_out=res, jac_out=jac)
            assert np.array_equal(res, ref["RES"]), f"step {rep}: residual"
            assert np.array_equal(jac, ref["JAC"]), f"step {rep}: Jacobian"
            same({k: ctx.get(k) for k in STEP_OUT}, {k: ref[k] for k in STEP_OUT}, f"step {rep}")
    assert np.array_equal(ref["PHASE_EXIST"], post["phaseExist"].astype(np.uint8))
    assert P.res_err(res, post["res_bulk"], post["rockVp"], post["Nt"], model.nc) <= P.REL_TOL


# ------------------------------------------------------ the bench state ---
NX, NY, NZ, NCOMP, SEED = 60, 60, 10, 6, 2
DT, DSMAX = 0.1, 0.2
ORACLE_FIELDS = [f for f in fim.FIELDS if f in fim.REF_NAMES.values()]


@pytest.fixture(scope="module")
def bench_state(gpu_lib):
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid(NX, NY, NZ)
    ctxs = {}
    for variant in (0, 1):
        ctx = fim.FimContext(model, grid, variant=variant)
        synthetic.ptn_workload(ctx, grid, NCOMP, SEED, dt=DT, dsmax=DSMAX)
        ctx.checkpoint(0)
        ctxs[variant] = ctx
    yield model, grid, ctxs
    for c in ctxs.values():
        c.close()


def test_bench_state_autotuned_graph_matches_plain_and_oracle(bench_state):
    from opencaeporox_gb300 import autotune
    from oracle.pyoracle import OracleBulk
    model, grid, ctxs = bench_state
    plain, batched = ctxs[0], ctxs[1]
    inputs = {f: plain.get(f) for f in ORACLE_FIELDS}
    plain.update_property()
    plain.cal_res(DT)
    plain.assemble_mat(DT)
    ref = outputs(plain)
    space = {"fused_blocks": ("sms", 1, 2), "fused_coop_blocks": ("sms/8", 0, 4), "flash_budget": (24, 48),
             "predefer": (96, 192), "coop_cells": (1216,), "coop_blocks": (608,), "block_cell": (128,),
             "pre_blocks": (0,)}
    tuned = autotune.tune(batched, DT, slot=0, space=space, rounds=1, reps=1)
    assert np.isfinite(tuned["step_ms"])
    for rep in range(2):
        batched.checkpoint(0, restore=True)
        same(graph_step(batched, DT), ref, f"tuned graph, replay {rep}")
    # the oracle, from the same inputs: labels and upwind choices exact, values
    # at the parity tolerances (flash outputs on a window, with the window's
    # one-ulp sensitivity)
    ob = OracleBulk(model, grid)
    inv = {v: k for k, v in fim.REF_NAMES.items()}
    ob.load({inv[f]: v for f, v in inputs.items()})
    ob.update_property()
    assert np.array_equal(ob.a["phaseExist"], ref["PHASE_EXIST"].astype(np.uint32))
    names = {"S": "S", "XIJ": "xij", "RHO": "rho", "XI": "xi", "MU": "mu", "VF": "vf", "NT": "Nt", "XIX": "xix",
             "RHOX": "rhox", "MUX": "mux", "RHOP": "rhoP", "XIP": "xiP", "MUP": "muP", "PHASE_EXIST": "phaseExist",
             "DSEC_DPRI": "dSec_dPri", "VFI": "vfi", "VFP": "vfP"}
    errs = P.state_errors({names[k]: ref[k] for k in names}, dict(ob.a), model.nc, grid.nb)
    sens = {}
    for seed in P.NUDGE_SEEDS:
        nb_ = OracleBulk(model, grid, variant="ulp")
        nb_.set_nudge_seed(seed)
        nb_.load({inv[f]: v for f, v in inputs.items()})
        nb_.update_property()
        if not np.array_equal(nb_.a["phaseExist"], ob.a["phaseExist"]):
            continue
        for k, v in P.state_errors(dict(nb_.a), dict(ob.a), model.nc, grid.nb).items():
            sens[k] = max(sens.get(k, 0.0), v)
    bad = {k: (v, P.tolerance(k, sens)) for k, v in errs.items() if v > P.tolerance(k, sens)}
    assert not bad, bad
    # residual and Jacobian of the oracle from the GPU's post-flash state
    post = {f: plain.get(f) for f in ORACLE_FIELDS}
    oc = OracleBulk(model, grid)
    oc.load({inv[f]: v for f, v in post.items()})
    oc.cal_res(DT)
    rp, col, val = oc.assemble(DT)
    assert np.array_equal(ref["UPBLOCK"], oc.conn["upblock"])
    assert P.res_err(ref["RES"], oc.res, post["ROCKVP"], post["NT"], model.nc) <= P.REL_TOL
    g_rp, g_col, _ = plain.jacobian()
    assert np.array_equal(g_rp, rp) and np.array_equal(g_col, col)
    bs = (model.nc + 1) ** 2
    a, b = ref["JAC"].reshape(-1, bs), val.reshape(-1, bs)
    num = np.sqrt(np.add.reduceat(np.sum((a - b) ** 2, axis=1), rp[:-1]))
    den = np.sqrt(np.add.reduceat(np.sum(b ** 2, axis=1), rp[:-1]))
    assert np.max(num / np.maximum(den, 1e-300)) <= P.REL_TOL


@pytest.mark.parametrize("variant", [0, 1])
def test_adjoint_inside_the_step(gpu_lib, variant):
    """With an adjoint seed, every step (the replayed graph in the batched
    form) also computes J^T lambda, (dR/dT)^T lambda and (dR/dporoInit)^T
    lambda; they equal ocpx_adjoint's at the same state, replay after replay,
    and go away with the seed."""
    fx = P.load_fixture("comp8_6x6x4")
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    pre = P.group(fx, it + "/pre")
    dt = float(pre["dt"][0])
    lam = np.random.default_rng(5).normal(size=grid.nb * (model.nc + 1))
    with fim.FimContext(model, grid, variant=variant) as ctx:
        ctx.load_state(P.jac_state(fx, it))
        ctx.load_state(pre)
        ctx.checkpoint(0)
        ctx.set_adjoint_seed(lam)
        got = []
        for rep in range(2):
            ctx.checkpoint(0, restore=True)
            ctx.enqueue_step(dt)
            ctx.step_report()
            got.append(ctx.get_adjoint())
        ref = ctx.adjoint(lam)
        for g in got:
            for a, b in zip(g, ref):
                assert np.array_equal(a, b)
        again = ctx.get_adjoint()                       # the explicit call left the seed alone
        for a, b in zip(again, ref):
            assert np.array_equal(a, b)
        ctx.set_adjoint_seed(None)
        with pytest.raises(fim.OcpxError, match="INVALID_ARG"):
            ctx.get_adjoint()


def test_field_ranges(gpu_lib):
    """Windows of fields in the reference layout equal the same slices of the
    whole field, in both directions; out-of-range windows are refused."""
    fx = P.load_fixture("comp6_8x8x3")
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(P.jac_state(fx, it))
        ctx.load_state(P.group(fx, it + "/pre"))
        ctx.update_property()
        ctx.cal_res(float(P.group(fx, it + "/pre")["dt"][0]))
        for name in ("P", "XIJ", "DSEC_DPRI", "PHASE_EXIST", "UPBLOCK", "FLUX_NI", "RES", "FLASH_ITERS"):
            full = ctx.get(name)
            w = ctx.field_width(name)
            n = full.size // w
            for first, cnt in ((0, n), (3, 17), (n - 5, 5), (n, 0)):
                assert np.array_equal(ctx.get_range(name, first, cnt), full[first * w:(first + cnt) * w]), name
            with pytest.raises(fim.OcpxError, match="INVALID_ARG"):
                ctx.get_range(name, n - 2, 3)
        xij = ctx.get("XIJ")
        w = ctx.field_width("XIJ")
        new = np.arange(7 * w, dtype=np.float64)
        ctx.set_range("XIJ", 11, new)
        ref = xij.copy()
        ref[11 * w:18 * w] = new
        assert np.array_equal(ctx.get("XIJ"), ref)
        with pytest.raises(fim.OcpxError, match="INVALID_ARG"):
            ctx.set_range("RES", 0, np.zeros(model.nc + 1))   # read-only field


def test_bench_state_split_refill_matches_plain(bench_state):
    """The split cells' first loop with lane refill (SPLIT_REFILL) on the
    36,000-cell state: the replayed graph bit-identical to the plain step."""
    model, grid, ctxs = bench_state
    plain, batched = ctxs[0], ctxs[1]
    plain.checkpoint(0, restore=True)
    plain.update_property()
    plain.cal_res(DT)
    plain.assemble_mat(DT)
    ref = outputs(plain)
    batched.set_param("split_refill", 1)
    try:
        for rep in range(2):
            batched.checkpoint(0, restore=True)
            same(graph_step(batched, DT), ref, f"split refill, replay {rep}")
    finally:
        batched.set_param("split_refill", 0)
