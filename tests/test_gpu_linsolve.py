"""Linear solve of the Newton system on the device (ocpx_linsolve) against a
direct solve of the same system (scipy), on the golden fixtures' Jacobians
and on the 36,000-cell bench system.  The reference passes this system to an
external package (FASP, PETSc or PARDISO) that is not part of its sources;
its dump harness solves it directly, as these tests do."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import parity as P
from opencaeporox_gb300 import fim, synthetic

pytestmark = pytest.mark.gpu


def _system(ctx):
    rp, col, val = ctx.jacobian()
    dim = ctx.nc + 1
    J = sp.bsr_matrix((val.reshape(-1, dim, dim), col, rp), shape=(ctx.nb * dim, ctx.nb * dim)).tocsr()
    return J, ctx.get("RES")


@pytest.mark.parametrize("name", ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4"])
def test_linsolve_fixture_systems(gpu_lib, name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    with fim.FimContext(model, grid) as ctx:
        for it in P.iterations(fx)[:3]:
            js = P.jac_state(fx, it)
            dt = float(js["dt"][0])
            ctx.load_state(js)
            ctx.cal_res(dt)
            ctx.assemble_mat(dt)
            J, b = _system(ctx)
            u, rep = ctx.linsolve(tol=1e-12, maxit=2000)
            assert rep["converged"] and not rep["breakdown"], (it, rep)
            assert np.linalg.norm(J @ u - b) <= 1e-11 * np.linalg.norm(b), (it, rep)
            x = sla.spsolve(J.tocsc(), b)
            assert np.linalg.norm(u - x) <= 1e-8 * np.linalg.norm(x), (it, np.linalg.norm(u - x) / np.linalg.norm(x))


def test_linsolve_bench_system_and_device_update(gpu_lib):
    """The 36,000-cell system of the bench step, solved to 1e-10; the
    device-resident update applies exactly as the same update from the host."""
    ncomp, seed = 6, 2
    model = synthetic.comp_model(ncomp, seed)
    grid = synthetic.comp_grid(60, 60, 10)
    with fim.FimContext(model, grid) as ctx:
        synthetic.ptn_workload(ctx, grid, ncomp, seed, dt=0.1, dsmax=0.2)
        ctx.update_property()
        ctx.cal_res(0.1)
        ctx.assemble_mat(0.1)
        J, b = _system(ctx)
        ctx.checkpoint(0)
        u, rep = ctx.linsolve(tol=1e-10, maxit=5000)
        assert rep["converged"] and not rep["breakdown"], rep
        assert np.linalg.norm(J @ u - b) <= 2e-10 * np.linalg.norm(b), rep
        ctx.newton_update_device(0.2)
        dev = {k: ctx.get(k) for k in ("P", "NI", "S", "XIJ")}
        ctx.checkpoint(0, restore=True)
        ctx.get_solution(u, 0.2)
        for k, v in dev.items():
            assert np.array_equal(v, ctx.get(k)), k


def test_linsolve_async_and_graph_replay(gpu_lib):
    """The enqueue-only solve (ocpx_linsolve_async) gives the synchronous
    solve's report and update bit for bit, also when it is captured in a CUDA
    graph on the context stream and replayed."""
    torch = pytest.importorskip("torch")
    fx = P.load_fixture("comp6_8x8x3")
    model, grid = fim.model_and_grid_from_dump(fx)
    keys = ("P", "NI", "S", "XIJ")
    with fim.FimContext(model, grid) as ctx:
        js = P.jac_state(fx, P.iterations(fx)[0])
        dt = float(js["dt"][0])
        ctx.load_state(js)
        ctx.cal_res(dt)
        ctx.assemble_mat(dt)
        ctx.checkpoint(0)
        _, rep = ctx.linsolve(tol=1e-12, maxit=300, copy_out=False)
        assert rep["converged"] and rep["iterations"] > 0
        ctx.newton_update_device(0.2)
        ref = {k: ctx.get(k) for k in keys}

        ctx.checkpoint(0, restore=True)
        ctx.linsolve_async(tol=1e-12, maxit=300)
        assert ctx.linsolve_report() == rep
        ctx.newton_update_device(0.2)
        for k in keys:
            assert np.array_equal(ctx.get(k), ref[k]), k

        ctx.checkpoint(0, restore=True)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=torch.cuda.ExternalStream(ctx.stream)):
            ctx.linsolve_async(tol=1e-12, maxit=300)
        for _ in range(2):
            g.replay()
            torch.cuda.synchronize()
            assert ctx.linsolve_report() == rep
        ctx.newton_update_device(0.2)
        for k in keys:
            assert np.array_equal(ctx.get(k), ref[k]), k
