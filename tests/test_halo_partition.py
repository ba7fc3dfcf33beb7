"""Subdomains by connection (opencaeporox_gb300.halo.partition) on grids a
fixed ghost layer does not serve: a faulted corner-point grid whose
non-neighbour connections reach two layers away, and a deck's grid with
inactive cells.  On each rank the oracle runs the property update, residual
and Jacobian of its own and ghost cells from the whole grid's state; the
owned rows are bit-identical to the whole grid's, and the halo exchange
fills every ghost with its owner's value.  Host only."""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import deck as D
from opencaeporox_gb300 import grid as G
from opencaeporox_gb300 import halo, synthetic
from oracle.pyoracle import OracleBulk

NCOMP, SEED, DT = 3, 4, 0.1


def _state(grid):
    """A physical state of every cell: the seeded PTN start, moles scaled to
    fill the pores, properties updated."""
    model = synthetic.comp_model(NCOMP, SEED)
    st = synthetic.comp_initial_state(grid, NCOMP, SEED)
    ob = OracleBulk(model, grid)
    ob.load(st)
    ob.update_property()
    Ni = (st["Ni"].reshape(grid.nb, -1) * (ob.a["rockVp"] / ob.a["vf"])[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    return model, st


def _run(model, grid, st):
    ob = OracleBulk(model, grid)
    ob.load(st)
    ob.a["skip_flag"][:] = 0
    ob.update_property()
    ob.cal_res(DT)
    rp, col, val = ob.assemble(DT)
    return ob.res.copy(), rp, col, val


def _check(grid, subs, model, st):
    n1 = NCOMP + 2
    bs = n1 * n1
    res, rp, col, val = _run(model, grid, st)
    covered = np.zeros(grid.nb, int)
    for sub in subs:
        local = {k: np.asarray(v).reshape(grid.nb, -1)[sub.cells].ravel() for k, v in st.items()}
        r, lrp, lcol, lval = _run(model, sub.grid, local)
        owned = sub.owned
        covered[owned] += 1
        assert np.array_equal(r.reshape(-1, n1)[:sub.n_owned], res.reshape(-1, n1)[owned])
        for i, c in enumerate(owned):
            a, b = slice(lrp[i], lrp[i + 1]), slice(rp[c], rp[c + 1])
            assert np.array_equal(sub.cells[lcol[a]], col[b]), (sub.rank, c)
            assert np.array_equal(lval[a.start * bs:a.stop * bs], val[b.start * bs:b.stop * bs]), (sub.rank, c)
    assert np.all(covered == 1)
    # the halo exchange gives every ghost its owner's value
    vals = np.arange(grid.nb * 2, dtype=np.float64).reshape(grid.nb, 2)
    arrays = [np.where(np.arange(s.grid.nb)[:, None] < s.n_owned, vals[s.cells], -1.0) for s in subs]
    for s, a in zip(subs, halo.exchange_in_process(subs, arrays, 2)):
        assert np.array_equal(a, vals[s.cells])


@pytest.mark.parametrize("nranks", [2, 3])
def test_faulted_grid_partition(nranks):
    nx, ny, nz, dz = 8, 6, 5, 3.0
    faults = [("x", 3, -4.5, 7.5, 1.5), ("y", 2, 1.2, -2.0, 0.6), ("x", 5, 6.0, 6.0, 0.7)]
    coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, 20.0, dz, 2000.0, 4.0, -3.0, faults, 0.05, seed=11)
    rng = np.random.default_rng(11)
    k = np.exp(rng.normal(np.log(100.0), 1.0, nx * ny * nz))
    grid = G.corner_point_grid(nx, ny, nz, coord, zcorn, k, k, 0.1 * k, 0.2)
    subs = halo.zslab_partition(grid, nx, ny, nz, nranks)
    # a fixed ghost layer would miss some: ghosts two layers from their rank's slab
    far = 0
    for s in subs:
        k0, k1 = s.layers
        kg = s.cells[s.n_owned:] // (nx * ny)
        far += int(np.sum((kg < k0 - 1) | (kg > k1)))
    assert far > 0
    model, st = _state(grid)
    _check(grid, subs, model, st)


def test_deck_grid_with_inactive_cells_partition(tmp_path):
    fx = P.load_fixture("deck_ortho_actnum")
    (tmp_path / "grid.data").write_text(str(fx["deck/main"]))
    (tmp_path / "grid_poro.inc").write_text(str(fx["deck/include"]))
    deck = D.read_grid_deck(str(tmp_path / "grid.data"))
    grid, geo = D.grid_from_deck(deck)
    assert grid.nb < deck.n
    subs = halo.zslab_partition(grid, deck.nx, deck.ny, deck.nz, 2, cell_index=geo["act2all"])
    model, st = _state(grid)
    _check(grid, subs, model, st)


def test_partition_refuses_bad_owner_maps():
    grid = synthetic.comp_grid(3, 2, 2)
    with pytest.raises(ValueError):
        halo.partition(grid, np.zeros(grid.nb - 1, int), 2)
    with pytest.raises(ValueError, match="owns no cell"):
        halo.partition(grid, np.zeros(grid.nb, int), 2)


def _faulted_grid():
    nx, ny, nz = 8, 6, 5
    faults = [("x", 3, -4.5, 7.5, 1.5), ("y", 2, 1.2, -2.0, 0.6), ("x", 5, 6.0, 6.0, 0.7)]
    coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, 20.0, 3.0, 2000.0, 4.0, -3.0, faults, 0.05, seed=11)
    return G.corner_point_grid(nx, ny, nz, coord, zcorn, 100.0, 100.0, 10.0, 0.2), (nx, ny, nz)


def _rank_exchange(rank, world, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        grid, dims = _faulted_grid()
        sub = halo.zslab_partition(grid, *dims, world)[rank]
        vals = np.arange(grid.nb * 3, dtype=np.float64).reshape(grid.nb, 3)
        local = np.where(np.arange(sub.grid.nb)[:, None] < sub.n_owned, vals[sub.cells], -1.0)
        got = halo.HaloExchange(sub).exchange(local, 3)
        norms = halo.HaloExchange(sub).max_norms((float(rank), -float(rank)))
        q.put((rank, bool(np.array_equal(got, vals[sub.cells])), sorted(sub.recv), norms))
    finally:
        dist.destroy_process_group()


def test_rank_exchange_on_the_faulted_grid():
    """Three gloo ranks exchange a cell array over the faulted grid's
    partition, whose ghost sets are irregular (NNC ghosts two layers away):
    every ghost receives its owner's value, and the norms reduce to the
    maximum over the ranks."""
    import socket
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    world = 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_exchange, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, ok, peers, norms in got:
        assert ok, rank
        assert norms == (2.0, 0.0)
    assert got[1][2] == [0, 2]
