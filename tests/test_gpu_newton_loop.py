"""One whole time step of Newton iterations on the device: assemble, linear
solve (ocpx_linsolve), device-resident update, property update, residual,
then CalMaxChangeNR and CheckConverge on the device, until converged.
This mirrors IsothermalSolver::GoOneStep's Newton loop (src/IsoThermalSolver.cpp:70-101)
for the bulk (no wells).  The oracle runs the same loop on the host with a
direct solve (tests/oracle restatements of every step); the two must take
the same number of iterations, reach the same control decisions, and agree
on the state to the linear solver's accuracy."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from opencaeporox_gb300 import fim, synthetic
from oracle import nrctl
from oracle.pyoracle import OracleBulk

pytestmark = pytest.mark.gpu

NCOMP, SEED, DT, DSMAX = 6, 3, 2.0, 0.2
# tighter than the golden decks' ControlNRParam (tol 1e-3, dPmin 1 bar, dSmin 0.01), so
# that the step takes several Newton iterations
CTRL = dict(maxIter=12, tol=1e-9, dPmin=1e-4, dSmin=1e-6)


def _start(ctx, grid):
    st = synthetic.comp_initial_state(grid, NCOMP, SEED)
    ctx.load_state(st)
    ctx.update_property()
    scale = ctx.get("ROCKVP") / ctx.get("VF")
    Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    ctx.load_state(st)
    ctx.set("SKIP_FLAG", np.zeros(grid.nb, np.uint8))
    ctx.update_property()
    return {k: ctx.get(k) for k in fim.FIELDS if k not in ("UPBLOCK", "CONN_DP", "FLUX_VJ", "FLUX_NI", "RES",
                                                             "RES_REL_V", "RES_REL_N", "TRANS", "PORO_INIT")}


def _gpu_loop(ctx):
    ctx.update_last_time_step()
    ctx.cal_res(DT)
    ctx.nr_init_step()
    states, decisions = [], []
    for it in range(CTRL["maxIter"]):
        ctx.assemble_mat(DT)
        _, rep = ctx.linsolve(tol=1e-13, maxit=2000, copy_out=False)
        assert rep["converged"], rep
        ctx.newton_update_device(DSMAX)
        ctx.update_property()
        ctx.cal_res(DT)
        ch = ctx.nr_max_change()
        st = ctx.nr_check_converge(fim.NRControl.make(**CTRL, iterNR=it + 1, res_from_host=0))
        states.append({k: ctx.get(k) for k in ("P", "NI", "S")})
        decisions.append((st, ch))
        if st != 1:
            break
    return states, decisions


def _oracle_loop(model, grid, start):
    ob = OracleBulk(model, grid)
    ob.load({fim_name_to_ref(k): v for k, v in start.items() if fim_name_to_ref(k)})
    ob.a["lNi"][:] = ob.a["Ni"]
    n0 = ob.cal_res(DT)
    dim = model.nc + 1
    last = {k: ob.a[k].copy() for k in ("P", "T", "Ni", "S")}
    states, decisions = [], []
    for it in range(CTRL["maxIter"]):
        rp, col, val = ob.assemble(DT)
        J = sp.bsr_matrix((val.reshape(-1, dim, dim), col, rp), shape=(grid.nb * dim, grid.nb * dim)).tocsc()
        u = sla.spsolve(J, ob.res)
        ob.newton_update(u, DSMAX)
        ob.update_property()
        n = ob.cal_res(DT)
        now = {k: ob.a[k].copy() for k in ("P", "T", "Ni", "S", "vf", "rockVp")}
        ch = nrctl.max_change_nr(now, last, model.nc)
        last = {k: now[k] for k in ("P", "T", "Ni", "S")}
        st = nrctl.check_converge(n[0], n0[0], n[1], 0.0, ch["dP"], ch["dS"], it + 1, CTRL["tol"], CTRL["dPmin"],
                                  CTRL["dSmin"], CTRL["maxIter"])
        states.append({"P": now["P"], "NI": now["Ni"], "S": now["S"]})
        decisions.append((st, ch))
        if st != 1:
            break
    return states, decisions


def fim_name_to_ref(field):
    inv = {v: k for k, v in fim.REF_NAMES.items()}
    return inv.get(field)


def test_time_step_on_device_matches_oracle(gpu_lib):
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid(10, 8, 4)
    with fim.FimContext(model, grid, variant=1) as ctx:
        start = _start(ctx, grid)
        g_states, g_dec = _gpu_loop(ctx)
    o_states, o_dec = _oracle_loop(model, grid, start)
    assert [d[0] for d in g_dec] == [d[0] for d in o_dec], (g_dec, o_dec)
    assert g_dec[-1][0] == 0 and len(g_dec) >= 2          # converged, after more than one iteration
    for it, (a, b) in enumerate(zip(g_states, o_states)):
        for k in a:
            err = np.linalg.norm(a[k] - b[k]) / np.linalg.norm(b[k])
            assert err <= 1e-9, (it, k, err)
        for q in ("dP", "dN", "dS"):
            ga, oa = g_dec[it][1][q], o_dec[it][1][q]
            assert abs(ga - oa) <= 1e-8 * max(abs(oa), 1e-12), (it, q, ga, oa)
