"""One grid split over two ranks (z-slabs with a ghost layer, the halo
exchange of opencaeporox_gb300.halo) against the same grid in one piece,
with two gloo ranks on the host.

Each rank runs two Newton iterations of the reference's algorithm (the
oracle) on its subdomain: the property update of its own and its ghost
cells, residual and Jacobian.  The Newton updates come from a vector of the
whole grid of which each rank takes only its own cells' part; the ghost part
arrives by the halo exchange.  The residual norms are reduced over the
ranks.  The stitched owned rows (residual, Jacobian values and columns),
upwind choices and norms are bit-identical to the single-domain run.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

NX, NY, NZ, NCOMP, SEED = 6, 5, 4, 4, 8
DT, DSMAX = 0.1, 0.2


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case():
    from opencaeporox_gb300 import synthetic
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid_lognormal(NX, NY, NZ, median=100.0, sigma_ln=1.0, corr_cells=2, seed=SEED)
    return model, grid


def _iterations(model, whole, grid, cells, u_for):
    """Two Newton iterations from the seeded PTN start on the cells `cells`
    of the whole grid `whole` (local grid `grid`); u_for(k, Ni) gives the k-th
    Newton update of the local cells from their moles Ni.  Returns per
    iteration the residual, the Jacobian (rowptr, col, val), the upwind
    choices, the per-cell relative residuals and the oracle's norms."""
    from opencaeporox_gb300 import synthetic
    from oracle.pyoracle import OracleBulk
    st_all = synthetic.comp_initial_state(whole, NCOMP, SEED)
    st = {k: np.asarray(v).reshape(whole.nb, -1)[cells].ravel() for k, v in st_all.items()}
    ob = OracleBulk(model, grid)
    ob.load(st)
    ob.update_property()
    scale = ob.a["rockVp"] / ob.a["vf"]
    Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    ob.load(st)
    ob.a["skip_flag"][:] = 0
    ob.update_property()
    ob.cal_res(DT)
    ob.a["lNi"][:] = ob.a["Ni"]
    out = []
    for k in range(2):
        ob.newton_update(u_for(k, Ni), DSMAX)
        ob.update_property()
        ob.cal_res(DT)
        rp, col, val = ob.assemble(DT)
        r = ob.res.reshape(grid.nb, -1)
        out.append(dict(res=ob.res.copy(), rp=rp, col=col, val=val, upblock=ob.conn["upblock"].copy(),
                        norms=ob.norms.copy(),
                        # per cell: the largest |R_i| / pore volume and |R_i| / Nt (component rows),
                        # whose maxima are maxRelRes_V and maxRelRes_N (IsoT_FIM::CalRes)
                        relV=np.max(np.abs(r) / ob.a["rockVp"][:, None], axis=1),
                        relN=np.max(np.abs(r[:, 1:]) / ob.a["Nt"][:, None], axis=1)))
    return out


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from opencaeporox_gb300 import halo, synthetic
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        model, grid = _case()
        sub = halo.zslab_partition(grid, NX, NY, NZ, world)[rank]
        hx = halo.HaloExchange(sub)
        width = NCOMP + 2

        def u_for(k, Ni_local):
            # the whole grid's update is the same seeded vector; this rank
            # knows only its own cells' part, the ghosts' part is exchanged
            Ni_all = np.zeros((grid.nb, NCOMP + 1))
            Ni_all[sub.cells] = np.asarray(Ni_local).reshape(-1, NCOMP + 1)
            u_all = synthetic.ptn_updates(Ni_all, grid.nb, NCOMP, SEED)[k].reshape(grid.nb, width)
            u = np.zeros((sub.grid.nb, width))
            u[:sub.n_owned] = u_all[sub.owned]
            return hx.exchange(u, width).ravel()

        res = _iterations(model, grid, sub.grid, sub.cells, u_for)
        for r in res:
            owned = slice(0, sub.n_owned)
            r["norms_global"] = hx.max_norms((r["relV"][owned].max(), r["relN"][owned].max()))
        q.put((rank, sub.n_owned, sub.cells, sub.conns, res))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_rank_halo_exchange_matches_single_domain(world):
    """Two ranks (one ghost layer each), and three (the middle rank has a
    ghost layer on both sides)."""
    model, grid = _case()
    from opencaeporox_gb300 import synthetic
    width = NCOMP + 2
    single = _iterations(model, grid, grid, np.arange(grid.nb),
                         lambda k, Ni: synthetic.ptn_updates(Ni, grid.nb, NCOMP, SEED)[k])
    for s in single:
        assert (s["norms"][0], s["norms"][1]) == (s["relV"].max(), s["relN"].max())
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    n1 = width                     # residual entries and block dimension: nc + 1
    bs = n1 * n1
    covered = np.zeros(grid.nb, bool)
    for rank, n_owned, cells, conns, res in got:
        owned = cells[:n_owned]
        covered[owned] = True
        for k, (a, b) in enumerate(zip(res, single)):
            # residual rows of the owned cells
            ra = a["res"].reshape(-1, n1)[:n_owned]
            rb = b["res"].reshape(-1, n1)[owned]
            assert np.array_equal(ra, rb), f"rank {rank} iteration {k}: residual"
            # upwind choices (cell numbers) of every local connection
            assert np.array_equal(cells[a["upblock"].reshape(-1, 3)], b["upblock"].reshape(-1, 3)[conns]), \
                f"rank {rank} iteration {k}: upwind"
            # Jacobian rows: the same blocks in the same order, columns mapped to the whole grid
            for n in range(n_owned):
                g = owned[n]
                ca = cells[a["col"][a["rp"][n]:a["rp"][n + 1]]]
                cb = b["col"][b["rp"][g]:b["rp"][g + 1]]
                assert np.array_equal(ca, cb), f"rank {rank} iteration {k} row {g}: columns"
                va = a["val"][a["rp"][n] * bs:a["rp"][n + 1] * bs]
                vb = b["val"][b["rp"][g] * bs:b["rp"][g + 1] * bs]
                assert np.array_equal(va, vb), f"rank {rank} iteration {k} row {g}: values"
            # the global residual norms (maxRelRes_V, maxRelRes_N)
            assert a["norms_global"] == (b["norms"][0], b["norms"][1]), f"rank {rank} iteration {k}: norms"
    assert covered.all()
