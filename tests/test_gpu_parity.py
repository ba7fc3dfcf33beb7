"""GPU parity of the FIM Newton-step kernels against the reference simulator.

The golden fixtures were produced by the reference's own C++ (see
tests/golden/gen_fixtures.py); every test here calls the CUDA library through
its C ABI and compares with them.

Tolerances (REL_TOL = 1e-10 from tests/parity.py):
  * exact: phase-existence labels, flash types, skip flags, upwind choices,
    Jacobian sparsity pattern and block order, Newton-update results;
  * elementwise <= REL_TOL: phase properties, saturations, kr/Pc, rock,
    residual, fluxes, residual norms; for the compositional flash outputs
    <= max(REL_TOL, 4 x the reference algorithm's own deviation under
    one-ulp perturbations of its transcendentals), measured per fixture
    iteration by the perturbed oracle (parity.libm_sensitivity);
  * per-cell normwise <= REL_TOL for the quantities obtained from the NC x NC
    derivative solve (vfi, vfP, dSec_dPri): the reference solves it with
    LAPACK dgesv from OpenBLAS, whose rounding differs from any other LU;
  * Jacobian values normwise per block row <= REL_TOL (dgemm rounding);
  * SkipPSA minimum eigenvalue <= 1e-4 relative: the reference computes it in
    single precision (ssyevd_).
"""
import json
import os

import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim

pytestmark = pytest.mark.gpu

FIXTURES = ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4", "fault_comp3_8x6x5"]
REPORT = {}


@pytest.fixture(scope="module", autouse=True)
def write_report():
    yield
    out = os.environ.get("OCPX_PARITY_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


def make_ctx(fx, variant=0):
    model, grid = fim.model_and_grid_from_dump(fx)
    return fim.FimContext(model, grid, variant=variant), model, grid


def check_update(ctx, fx, it, model, grid):
    pre = P.group(fx, it + "/pre")
    post = P.group(fx, it + "/post")
    js = P.jac_state(fx, it)
    ctx.load_state(js)
    ctx.load_state(pre)
    ctx.update_property()
    got = P.state_from_ctx(ctx)
    nb = grid.nb
    pe_g = got["phaseExist"].reshape(nb, 3)
    pe_r = post["phaseExist"].reshape(nb, 3)
    assert np.array_equal(pe_g, pe_r), f"{it}: phase labels differ in {np.sum(np.any(pe_g != pe_r, 1))} cells"
    errs = P.state_errors(got, post, model.nc, nb)
    if "flash_ftype" in post and model.compositional:
        assert np.array_equal(ctx.get("FTYPE"), post["flash_ftype"].astype(np.int8)), f"{it}: flash types differ"
        assert np.array_equal(ctx.get("SKIP_FLAG"), post["skip_flag"].astype(np.uint8)), f"{it}: skip flags differ"
        ref = post["skip_minEigen"]
        m = post["skip_flag"].astype(bool)
        assert P.rel_err(ctx.get("SKIP_MINEIG")[m], ref[m]) < 1e-4
    norms = ctx.cal_res(float(pre["dt"][0]))
    assert np.array_equal(ctx.get("UPBLOCK"), post["upblock"]), f"{it}: upwind choices differ"
    errs["res"] = P.res_err(ctx.get("RES"), post["res_bulk"], post["rockVp"], post["Nt"], model.nc)
    errs["flux_ni"] = P.rel_err(ctx.get("FLUX_NI"), post["flux_ni"])
    errs["dP"] = P.rel_err(ctx.get("CONN_DP"), post["dP"])
    errs["resRelV"] = float(np.max(np.abs(ctx.get("RES_REL_V") - post["resRelV"])))
    errs["resRelN"] = float(np.max(np.abs(ctx.get("RES_REL_N") - post["resRelN"])))
    errs["maxRelRes_V"] = abs(norms.maxRelRes_V - float(post["maxRelRes_V"][0]))
    assert norms.maxId_V == int(post["maxId_V"][0]) and norms.maxId_N == int(post["maxId_N"][0])
    REPORT.setdefault(fx["__name__"], {})[it] = errs
    sens = P.libm_sensitivity(fx, it, model, grid) if model.compositional else {}
    REPORT[fx["__name__"]][it + "/libm_sensitivity"] = sens
    # worst cells of the transcendental-heavy outputs, with their flash record
    st, iters = ctx.get("STATUS"), ctx.get("FLASH_ITERS").reshape(nb, 5)
    for k in ("mu", "xij"):
        w = np.asarray(got[k], np.float64).reshape(nb, -1)
        r = np.asarray(post[k], np.float64).reshape(nb, -1)
        m = pe_r.astype(bool) if k == "mu" else np.repeat(pe_r.astype(bool), model.nc, axis=1)
        e = np.where(m, np.abs(w - r) / np.maximum(np.abs(r), 1e-300), 0).max(axis=1)
        worst = np.argsort(e)[-3:][::-1]
        REPORT[fx["__name__"]][it + "/" + k + "_worst"] = [
            [int(c), float(e[c]), int(st[c]), iters[c].tolist(), pe_r[c].tolist()] for c in worst]
    bad = {k: (v, P.tolerance(k, sens)) for k, v in errs.items() if v > P.tolerance(k, sens)}
    assert not bad, f"{it}: {bad}"
    return errs


@pytest.mark.parametrize("name", FIXTURES)
def test_property_update_and_residual(gpu_lib, name):
    fx = P.load_fixture(name)
    fx["__name__"] = name
    its = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")]
    assert its
    ctx, model, grid = make_ctx(fx)
    with ctx:
        for it in its:
            check_update(ctx, fx, it, model, grid)


@pytest.mark.parametrize("name", FIXTURES)
def test_jacobian(gpu_lib, name):
    fx = P.load_fixture(name)
    ctx, model, grid = make_ctx(fx)
    bs = (model.nc + 1) ** 2
    with ctx:
        for it in P.iterations(fx):
            js = P.jac_state(fx, it)
            dt = float(js["dt"][0])
            ctx.load_state(js)
            ctx.cal_res(dt)
            assert np.array_equal(ctx.get("UPBLOCK"), js["upblock"])
            assert P.res_err(ctx.get("RES"), js["res_bulk"], js["rockVp"], js["Nt"], model.nc) <= P.REL_TOL
            ctx.assemble_mat(dt)
            rp, col, val = ctx.jacobian()
            assert np.array_equal(rp, js["jac_rowptr"]) and np.array_equal(col, js["jac_col"]), f"{it}: pattern"
            ref = js["jac_val"]
            # normwise per block row
            for r in range(grid.nb):
                a, b = val[rp[r] * bs: rp[r + 1] * bs], ref[rp[r] * bs: rp[r + 1] * bs]
                e = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
                assert e <= P.REL_TOL, f"{it} row {r}: {e:.2e}"


@pytest.mark.parametrize("name", FIXTURES)
def test_newton_update(gpu_lib, name):
    fx = P.load_fixture(name)
    ctx, model, grid = make_ctx(fx)
    with ctx:
        for it in P.iterations(fx):
            pre = P.group(fx, it + "/pre")
            if not pre:
                continue
            ctx.load_state(P.jac_state(fx, it))
            ctx.get_solution(pre["u"], float(pre["dSmax"][0]))
            for k, f in (("P", "P"), ("Ni", "NI"), ("S", "S"), ("xij", "XIJ")):
                assert np.array_equal(ctx.get(f), pre[k]), f"{it}: {k}"


FLASH_OUT = ("S", "XIJ", "RHO", "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "DSEC_DPRI", "VF", "VFP",
             "VFI", "NT", "PHASE_EXIST", "FTYPE", "FLASH_ITERS", "STATUS", "SKIP_FLAG", "SKIP_MINEIG", "SKIP_P",
             "SKIP_ZI", "KR", "PC", "PORO", "ROCKVP")


def test_batched_variant_against_reference(gpu_lib):
    fx = P.load_fixture("comp8_6x6x4")
    fx["__name__"] = "comp8_6x6x4/batched"
    it = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")][0]
    ctx, model, grid = make_ctx(fx, 1)
    with ctx:
        check_update(ctx, fx, it, model, grid)


TWO_STREAM = dict(fused_blocks=0)
BATCH_CASES = [
    # the default (fused) form
    dict(flash_budget=0), dict(flash_budget=3), dict(), dict(coop_cells=8), dict(coop_cells=0, predefer=1),
    dict(fused_blocks=2), dict(fused_blocks=2, flash_budget=0), dict(fused_blocks=2, flash_budget=3),
    dict(fused_blocks=3, flash_budget=3, coop_cells=0, predefer=1),
    dict(fused_blocks=1, flash_budget=1, coop_cells=0, predefer=0),
    dict(fused_blocks=400, flash_budget=3, coop_cells=0, predefer=1),
    dict(fused_blocks=3, fused_coop_blocks=1, flash_budget=3, coop_cells=0, predefer=1),
    dict(fused_blocks=2, fused_coop_blocks=1, flash_budget=0, predefer=0),
    dict(fused_excl=0, post_block=32, flash_budget=3, coop_cells=0, predefer=1),
    dict(fused_blocks=3, fused_coop_blocks=1, fused_excl=0, post_block=64, flash_budget=3, predefer=1),
    # the two-stream form
    dict(TWO_STREAM, flash_budget=0), dict(TWO_STREAM, flash_budget=3), dict(TWO_STREAM),
    dict(TWO_STREAM, coop_cells=8), dict(TWO_STREAM, coop_cells=0),
    dict(TWO_STREAM, coop_cells=0, predefer=1, pre_blocks=0), dict(TWO_STREAM, coop_cells=0, predefer=1, pre_blocks=3),
    dict(TWO_STREAM, flash_budget=3, coop_cells=0, cell_blocks=2),
    dict(TWO_STREAM, flash_budget=3, coop_cells=0, rounds=2, round_growth=2),
    dict(TWO_STREAM, flash_budget=1, coop_cells=0, predefer=0, rounds=8, round_growth=2, cell_blocks=1),
    dict(TWO_STREAM, flash_budget=0, post_block=32),
]


@pytest.mark.parametrize("name", ["comp6_8x8x3", "comp8_6x6x4"])
@pytest.mark.parametrize("params", BATCH_CASES, ids=lambda p: ",".join(f"{k}={v}" for k, v in p.items()) or "defaults")
def test_batched_variant_matches_plain(gpu_lib, name, params):
    """The batched flash (cost order, work budget, warp-cooperative phase
    equilibrium for the deferred cells) is bit-identical to the plain one,
    whatever its launch parameters: budget 0 sends every cell that needs an
    equilibrium through the cooperative kernel; pre-deferral threshold 1
    sends the cells that needed an equilibrium last time to the second
    stream, on shared-SM or SM-exclusive blocks; persistent blocks run the
    per-cell kernel 32 cells per warp at a time; re-budgeting rounds rerun
    the over-budget cells with growing budgets before the cooperative pass;
    the fused kernel (SM-exclusive blocks, one to three of them, or 400
    blocks that share SMs) consumes the over-budget cells while they are
    being published, also with its first block reserved for the
    cooperative work, and without the SM-exclusive reservation; the kernel
    that finishes the deferred cells with 32 to 128 threads per block."""
    budget = params.get("flash_budget")
    predefer = params.get("predefer")
    fx = P.load_fixture(name)
    its = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")]
    outs = []
    deferred = []
    for variant in (0, 1):
        ctx, model, grid = make_ctx(fx, variant)
        with ctx:
            if variant == 1:
                for k, v in params.items():
                    ctx.set_param(k, v)
            got = []
            for it in its:
                ctx.load_state(P.jac_state(fx, it))
                ctx.load_state(P.group(fx, it + "/pre"))
                ctx.update_property()
                got.append({k: ctx.get(k) for k in FLASH_OUT})
                if variant == 1:
                    deferred.append((ctx.get_param("deferred"), ctx.get_param("predeferred")))
            outs.append(got)
    if budget == 0:
        assert all(d > 0 for d, _ in deferred), deferred
    if predefer == 1:
        assert sum(p for _, p in deferred) > 0, deferred
    for it, a, b in zip(its, outs[0], outs[1]):
        for k in FLASH_OUT:
            assert np.array_equal(a[k], b[k], equal_nan=True), f"{name} {it} {params}: {k} differs"


def test_cooperative_fused_grid_that_does_not_fit_is_refused(gpu_lib):
    """A fused grid with cooperative-only blocks must be resident at once; a
    grid that cannot be is refused before anything is launched, and the
    context stays usable."""
    fx = P.load_fixture("comp6_8x8x3")
    ctx, model, grid = make_ctx(fx, 1)
    with ctx:
        it = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")][0]
        ctx.load_state(P.jac_state(fx, it))
        ctx.load_state(P.group(fx, it + "/pre"))
        ctx.set_param("fused_blocks", 64 * ctx.get_param("sms"))
        ctx.set_param("fused_coop_blocks", 1)
        with pytest.raises(fim.OcpxError, match="resident"):
            ctx.update_property()
        ctx.set_param("fused_blocks", ctx.get_param("sms"))
        ctx.update_property()
        assert np.all(np.isfinite(ctx.get("XI")))


def test_fused_launch_parameters(gpu_lib):
    """Automatic cooperative-only blocks (half of the fused blocks while they
    hold one SM each, none beyond), the small-grid defaults, the refusal of
    cooperative-only blocks with two fused blocks per SM before anything is
    launched, and the ranges of the launch parameters."""
    fx = P.load_fixture("comp6_8x8x3")
    ctx, model, grid = make_ctx(fx, 1)
    with ctx:
        sms = ctx.get_param("sms")
        assert ctx.get_param("fused_blocks") == sms
        assert ctx.get_param("fused_coop_blocks") == sms // 2
        assert ctx.get_param("fused_excl") == 0
        assert ctx.get_param("post_block") == 32
        assert ctx.get_param("flash_budget") == 32
        ctx.set_param("fused_blocks", 2 * sms)
        assert ctx.get_param("fused_coop_blocks") == 0
        it = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")][0]
        ctx.load_state(P.jac_state(fx, it))
        ctx.load_state(P.group(fx, it + "/pre"))
        ctx.set_param("fused_coop_blocks", 1)
        with pytest.raises(fim.OcpxError, match="one block per SM"):
            ctx.update_property()
        ctx.set_param("fused_coop_blocks", -1)
        assert ctx.get_param("fused_coop_blocks") == 0
        ctx.set_param("fused_blocks", sms)
        assert ctx.get_param("fused_coop_blocks") == sms // 2
        for k, v in (("post_block", 48), ("post_block", 256), ("fused_excl", 2), ("fused_coop_blocks", -2)):
            with pytest.raises(fim.OcpxError, match="INVALID_ARG"):
                ctx.set_param(k, v)
        ctx.update_property()
        assert np.all(np.isfinite(ctx.get("XI")))
