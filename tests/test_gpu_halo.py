"""Subdomains of one grid, each in its own context on the GPU, against the
whole grid in one context: the product path of a grid split over several
GPUs (opencaeporox_gb300.halo), run here with all subdomains on one GPU.

Each subdomain context holds its own cells first and its ghost layers after
them (nb_interior).  The Newton updates of the ghost cells come from their
owners through the halo exchange (on the host, between Newton iterations:
no kernel waits on another context; the contexts advance stage by stage in
turn).  The owned rows of every subdomain
(flash outputs, residual, Jacobian blocks and columns), the upwind choices
and the reduced residual norms are bit-identical to the whole grid's, in the
plain form and in the batched graph-replayed form.
"""
import numpy as np
import pytest

from opencaeporox_gb300 import fim, halo, synthetic

pytestmark = pytest.mark.gpu

NX, NY, NZ, NCOMP, SEED = 12, 10, 9, 6, 11
DT, DSMAX = 0.1, 0.2
CELL_OUT = ("PHASE_EXIST", "S", "XIJ", "RHO", "XI", "MU", "DSEC_DPRI", "VF", "VFP", "VFI", "NT", "KR", "PJ",
            "FTYPE", "FLASH_ITERS", "SKIP_FLAG", "P", "NI")


def drive(ctxs, whole, cells_list, u_for):
    """The bench's Newton iterations (seeded PTN start, pores filled, two
    seeded updates) on each context's cells `cells_list[r]` of the whole
    grid, stage by stage for all contexts in turn (lockstep); u_for(k, Nis)
    gives every context's k-th Newton update from their moles.  The second
    iteration runs as ctx.enqueue_step (a replayed graph in the batched
    form).  Returns per context the cell outputs, residual, Jacobian, upwind
    choices and norms."""
    st_all = synthetic.comp_initial_state(whole, NCOMP, SEED)
    sts, Nis = [], []
    for ctx, cells in zip(ctxs, cells_list):
        st = {k: np.asarray(v).reshape(whole.nb, -1)[cells].ravel() for k, v in st_all.items()}
        nb = cells.size
        ctx.load_state(st)
        ctx.update_property()
        scale = ctx.get("ROCKVP") / ctx.get("VF")
        Ni = (st["Ni"].reshape(nb, -1) * scale[:, None]).ravel()
        st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(nb, -1).sum(axis=1))
        ctx.load_state(st)
        ctx.set("SKIP_FLAG", np.zeros(nb, np.uint8))
        ctx.update_property()
        ctx.cal_res(DT)
        ctx.update_last_time_step()
        Nis.append(Ni)
    for ctx, u in zip(ctxs, u_for(0, Nis)):
        ctx.get_solution(u, DSMAX)
        ctx.update_property()
        ctx.cal_res(DT)
    outs = []
    for ctx, u, cells in zip(ctxs, u_for(1, Nis), cells_list):
        ctx.get_solution(u, DSMAX)
        ctx.checkpoint(0)
        for _ in range(2):                   # capture and a replay
            ctx.checkpoint(0, restore=True)
            ctx.enqueue_step(DT)
            ctx.step_report()
        norms = ctx.cal_res(DT)
        nb = cells.size
        out = {k: ctx.get(k).reshape(nb, -1) for k in CELL_OUT}
        out["RES"] = ctx.get("RES").reshape(nb, -1)
        out["UPBLOCK"] = ctx.get("UPBLOCK").reshape(-1, 3)
        out["JAC"] = ctx.jacobian()
        out["norms"] = (norms.maxRelRes_V, norms.maxRelRes_N)
        outs.append(out)
    return outs


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("nsub", [2, 3])
def test_subdomains_match_the_whole_grid(gpu_lib, variant, nsub):
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid_lognormal(NX, NY, NZ, median=100.0, sigma_ln=1.0, corr_cells=3, seed=SEED)
    width = NCOMP + 2
    with fim.FimContext(model, grid, variant=variant) as ctx:
        whole = drive([ctx], grid, [np.arange(grid.nb)],
                      lambda k, Nis: [synthetic.ptn_updates(Nis[0], grid.nb, NCOMP, SEED)[k]])[0]
    subs = halo.zslab_partition(grid, NX, NY, NZ, nsub)

    def u_for(k, Nis):
        # each subdomain knows only its own cells' part of the update; the
        # ghosts' part comes from their owners by the halo exchange
        own = []
        for s, Ni in zip(subs, Nis):
            Ni_all = np.zeros((grid.nb, NCOMP + 1))
            Ni_all[s.cells] = np.asarray(Ni).reshape(-1, NCOMP + 1)
            u_all = synthetic.ptn_updates(Ni_all, grid.nb, NCOMP, SEED)[k].reshape(grid.nb, width)
            u = np.zeros((s.grid.nb, width))
            u[:s.n_owned] = u_all[s.owned]
            own.append(u)
        return [u.ravel() for u in halo.exchange_in_process(subs, own, width)]

    ctxs = [fim.FimContext(model, s.grid, variant=variant) for s in subs]
    try:
        got = drive(ctxs, grid, [s.cells for s in subs], u_for)
    finally:
        for c in ctxs:
            c.close()
    bs = width * width
    rp_w, col_w, val_w = whole["JAC"]
    normV = normN = 0.0
    for s, g in zip(subs, got):
        own = s.owned
        for k in CELL_OUT:
            assert np.array_equal(g[k][:s.n_owned], whole[k][own], equal_nan=True), f"subdomain {s.rank}: {k}"
            # the ghosts' own copies of their owners' state agree too
            assert np.array_equal(g[k][s.n_owned:], whole[k][s.cells[s.n_owned:]], equal_nan=True), \
                f"subdomain {s.rank}: ghost {k}"
        assert np.array_equal(g["RES"][:s.n_owned], whole["RES"][own]), f"subdomain {s.rank}: residual"
        assert np.all(g["RES"][s.n_owned:] == 0), "ghost rows of the residual are zero"
        assert np.array_equal(s.cells[g["UPBLOCK"]], whole["UPBLOCK"][s.conns]), f"subdomain {s.rank}: upwind"
        rp, col, val = g["JAC"]
        assert rp.size == s.n_owned + 1
        for n in range(s.n_owned):
            w = own[n]
            assert np.array_equal(s.cells[col[rp[n]:rp[n + 1]]], col_w[rp_w[w]:rp_w[w + 1]])
            assert np.array_equal(val[rp[n] * bs:rp[n + 1] * bs], val_w[rp_w[w] * bs:rp_w[w + 1] * bs]), \
                f"subdomain {s.rank} row {w}"
        normV, normN = max(normV, g["norms"][0]), max(normN, g["norms"][1])
    assert (normV, normN) == whole["norms"]
