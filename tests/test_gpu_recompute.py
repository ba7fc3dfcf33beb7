"""Flash derivatives recomputed where they are used (ocpx_options
recompute_flash_der) against the stored form.

With the option, no dSec_dPri (OCPMixtureMethodComp::CaldXsdXp02,
src/OCPMixtureMethodComp.cpp:565-642) is kept: the flash leaves the two
hydrocarbon phases' mole numbers, and the connection blocks of the Jacobian
(OCP_FIM_Conn::AssembleMat), GetSolution (Bulk::GetSolutionFIM) and the
wells' perforation terms recompute it from the state with the flash's own
statements.  Every result must be bit-identical to the stored form's:

* a sequence of Newton iterations (update, properties, residual, Jacobian) on
  the two compositional golden decks, in the plain form and in the batched form's replayed
  graph, with the DSEC_DPRI field read back (recomputed on the fly);
* the wells inside the step: residual, Jacobian, maxWellRelRes_mol, the bhp
  update;
* the adjoint products inside the step;
* the 36,000-cell bench state with its Peaceman wells;
* the memory the context holds: one np*(nc+1)^2 array and its staging copy
  fewer; DSEC_DPRI cannot be written; black-oil contexts refuse the option.
"""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim, synthetic, wells as WL

pytestmark = pytest.mark.gpu

FIXTURES = ["comp6_8x8x3", "comp8_6x6x4"]
OUT = ("PHASE_EXIST", "S", "XIJ", "RHO", "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "DSEC_DPRI",
       "VF", "VFP", "VFI", "NT", "FTYPE", "FLASH_ITERS", "STATUS", "SKIP_FLAG", "KR", "PC", "PJ", "DKRDS",
       "DPCDS", "PORO", "POROP", "ROCKVP", "UPBLOCK", "CONN_DP", "FLUX_VJ", "FLUX_NI", "RES", "RES_REL_V",
       "RES_REL_N", "P", "NI")


def outputs(ctx):
    out = {k: ctx.get(k) for k in OUT}
    out["JAC"] = ctx.jacobian()[2]
    return out


def same(a, b, what):
    for k in a:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        if np.array_equal(x, y, equal_nan=True):
            continue
        bad = np.nonzero(~((x == y) | (np.isnan(x) & np.isnan(y))))[0] if x.shape == y.shape else []
        raise AssertionError(f"{what}: {k} differs at {len(bad)} of {x.size} entries {bad[:12]}: "
                             f"{x[bad[:4]]} vs {y[bad[:4]]}")


def first_it(fx):
    return [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")][0]


def updates(nb, nc, n, seed, scale_n):
    """Seeded Newton updates: dP ~ N(0, 2) bar, dNi relative N(0, 2e-3)."""
    rng = np.random.default_rng(seed)
    us = []
    for _ in range(n):
        u = np.zeros((nb, nc + 1))
        u[:, 0] = rng.normal(0.0, 2.0, nb)
        u[:, 1:] = scale_n * rng.normal(0.0, 2e-3, (nb, nc))
        us.append(u.ravel())
    return us


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("variant", [0, 1])
def test_newton_sequence_bit_identical(gpu_lib, name, variant):
    fx = P.load_fixture(name)
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    js, pre = P.jac_state(fx, it), P.group(fx, it + "/pre")
    dt, dsmax = float(pre["dt"][0]), float(pre["dSmax"][0])
    nb, nc = grid.nb, model.nc
    Ni = np.asarray(js["Ni"], np.float64).reshape(nb, nc)
    us = updates(nb, nc, 3, 11, Ni)
    with fim.FimContext(model, grid, variant=variant) as st, \
            fim.FimContext(model, grid, variant=variant, recompute=True) as rc:
        assert rc.get_param("recompute_flash_der") == 1 and st.get_param("recompute_flash_der") == 0
        for c in (st, rc):
            c.load_state(js)
            c.update_property()
        assert np.array_equal(st.get("DSEC_DPRI"), rc.get("DSEC_DPRI")), "dSec_dPri after the first flash"
        for k, u in enumerate(us):
            for c in (st, rc):
                if variant == 1:
                    c.get_solution(u, dsmax)
                    c.enqueue_step(dt)
                    c.step_report()
                else:
                    c.step(u=u, dSmax=dsmax, dt=dt)
            same(outputs(rc), outputs(st), f"iteration {k}")
        # a window of cells read back recomputed
        lend = 3 * (nc + 1) ** 2
        w = rc.get_range("DSEC_DPRI", 5, 17)
        assert np.array_equal(w, st.get("DSEC_DPRI")[5 * lend:22 * lend])
        # a checkpoint restores what the recomputation reads
        for c in (st, rc):
            c.checkpoint(0)
            c.get_solution(us[0], dsmax)
            c.update_property()
            c.checkpoint(0, restore=True)
            c.get_solution(us[1], dsmax)
            c.update_property()
            c.cal_res(dt)
            c.assemble_mat(dt)
        same(outputs(rc), outputs(st), "after a checkpoint restore")


def test_wells_bit_identical(gpu_lib):
    import test_gpu_wells_step as T
    from oracle import wells as W
    fx = P.load_fixture("comp6_8x8x3")
    model, grid = fim.model_and_grid_from_dump(fx)
    nb, nc = grid.nb, model.nc
    its = T._iterations("wells_comp6_8x8x3")
    with fim.FimContext(model, grid, variant=1) as st, \
            fim.FimContext(model, grid, variant=1, recompute=True) as rc:
        done = 0
        for it, fw in its:
            post = P.group(fx, it + "/post")
            if "P" not in post:
                continue
            dt = float(fw["dt"][0])
            wells, _, _ = W.split_wells(fw)
            api = T._api_wells(wells)
            for c in (st, rc):
                c.load_state(post)
                c.set_wells(api)
                c.update_property()
                c.cal_res(dt)
                c.assemble_mat(dt)
            same(outputs(rc), outputs(st), it)
            assert st.get_wells()[1] == rc.get_wells()[1]
            u = np.zeros(st.nv)
            u[:nb * (nc + 1)] = updates(nb, nc, 1, 5, np.asarray(post["Ni"]).reshape(nb, nc))[0]
            u[nb * (nc + 1)::nc + 1] = 3.0
            for c in (st, rc):
                c.get_solution(u, 0.2)
                c.enqueue_step(dt)
                c.step_report()
            same(outputs(rc), outputs(st), it + " after the update")
            assert np.array_equal(st.get_wells()[0], rc.get_wells()[0])
            done += 1
        assert done > 0


def test_adjoint_in_step_bit_identical(gpu_lib):
    fx = P.load_fixture("comp8_6x6x4")
    it = first_it(fx)
    model, grid = fim.model_and_grid_from_dump(fx)
    js, pre = P.jac_state(fx, it), P.group(fx, it + "/pre")
    dt, dsmax = float(pre["dt"][0]), float(pre["dSmax"][0])
    nb, nc = grid.nb, model.nc
    u = updates(nb, nc, 1, 3, np.asarray(js["Ni"]).reshape(nb, nc))[0]
    lam = np.random.default_rng(9).normal(size=nb * (nc + 1))
    got = []
    for recompute in (False, True):
        with fim.FimContext(model, grid, variant=1, recompute=recompute) as c:
            c.load_state(js)
            c.update_property()
            c.set_adjoint_seed(lam)
            c.get_solution(u, dsmax)
            c.enqueue_step(dt)
            c.step_report()
            got.append(c.get_adjoint())
    for a, b in zip(*got):
        assert np.array_equal(a, b)


def test_bench_state_with_wells_bit_identical(gpu_lib):
    ncomp, seed, dt, dsmax = 6, 2, 0.1, 0.2
    model = synthetic.comp_model(ncomp, seed)
    grid = synthetic.comp_grid(60, 60, 10)
    k = np.full(grid.nb, 50.0)
    wl = WL.vertical_wells(60, 60, 10, 2, 2, 20.0, 5.0, k, k, grid.depth, ncomp, seed, n_rate=1)
    outs = []
    for recompute in (False, True):
        with fim.FimContext(model, grid, variant=1, recompute=recompute) as c:
            synthetic.ptn_workload(c, grid, ncomp, seed, dt=dt, dsmax=dsmax)
            c.set_wells(wl)
            c.enqueue_step(dt)
            c.step_report()
            o = outputs(c)
            o["BHP"], o["MAXREL"] = c.get_wells()
            outs.append(o)
    same(outs[1], outs[0], "36,000 cells with wells")


def test_memory_and_refusals(gpu_lib):
    fx = P.load_fixture("comp8_6x6x4")
    model, grid = fim.model_and_grid_from_dump(fx)
    nb, nc = grid.nb, model.nc
    lend = 3 * (nc + 1) ** 2
    with fim.FimContext(model, grid) as st, fim.FimContext(model, grid, recompute=True) as rc:
        saved = st.get_param("device_bytes") - rc.get_param("device_bytes")
        # dSec_dPri and its staging copy, less the phase mole numbers, the
        # smaller staging buffer and the slab scratch (here one slab: the whole
        # grid), 256-byte alignment aside
        slab = min(nb, 1 << 19)
        assert saved >= 2 * 8 * nb * lend - 8 * nb * max(3 * nc, 9, 5) - 2 * 8 * nb - 8 * slab * lend - 4096
        with pytest.raises(RuntimeError, match="recomputed"):
            rc.set("DSEC_DPRI", np.zeros(nb * lend))
    bo = P.load_fixture("bo_10x10x3")
    m2, g2 = fim.model_and_grid_from_dump(bo)
    with pytest.raises(RuntimeError, match="compositional"):
        fim.FimContext(m2, g2, recompute=True)
