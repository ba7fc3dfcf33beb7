"""One grid over several GPUs: z-slab subdomains with a ghost layer, and the
halo exchange of a Newton iteration.

The reference splits its grid with ParMETIS, gives each MPI rank its own
cells plus one layer of ghost cells (copies of neighbouring ranks' cells),
recomputes the ghosts' properties locally (IsoT_FIM::CalFlash runs over all
nb cells, src/IsoThermalMethod.cpp:1016-1025), exchanges the ghosts' primary
variables once per Newton iteration (the Newton update u after the solve,
IsoT_FIM::GetSolution, src/IsoThermalMethod.cpp:1300-1330; the state at the
start, :33-94), and reduces the residual norms over the ranks (MPI_Allreduce,
:1176).  Here the subdomains of a structured grid are slabs of whole layers,
which need no graph partitioner:

* ``partition`` builds the subdomains from an owner rank per cell (from any
  partitioner).  A rank's ghost cells are all the other ranks' cells
  connected to one of its own, as the reference's one layer of ghost cells
  is defined by the grid's connections; a fault's non-neighbour connections
  can reach a second layer away, and such a cell is a ghost too.  Its local
  cell numbers are the owned cells first, in the global order, then the
  ghost cells, in the global order (so the context's nb_interior is the owned
  count).  Its connections are the global connections with at least one
  owned end, in the global order, each end keeping its role (bId, eId): the
  owned rows of the subdomain's residual and Jacobian are then bit-identical
  to the same rows of the whole grid.
* ``zslab_partition`` owns cells (k, j, i), i fastest, by slabs of R runs of
  consecutive layers; for a grid of the active cells of a larger one it
  takes each active cell's index in that grid.
* ``pack`` / ``unpack`` give each neighbour the owned values it holds as
  ghosts and write received values into the ghost cells (the Newton update,
  or any cell array in the reference's layout).  ``HaloExchange`` moves them
  between ranks through host buffers over a torch.distributed process group
  (gloo), one send and one receive per neighbour posted together between
  Newton iterations, and takes global maxima of the residual norms; no kernel
  waits on another rank.  ``exchange_in_process`` does the same for
  subdomains held by one process.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .fim import Grid


@dataclass
class Subdomain:
    rank: int
    layers: tuple            # owned layers [k0, k1) (None for an owner map not by layer)
    cells: np.ndarray        # global cell number of each local cell (owned, then ghost)
    n_owned: int
    grid: Grid               # local grid (nb_interior = n_owned)
    conns: np.ndarray        # global connection number of each local connection
    send: dict               # neighbour rank -> local numbers of owned cells it holds as ghosts
    recv: dict               # neighbour rank -> local numbers of this rank's ghost cells it owns

    @property
    def owned(self):
        return self.cells[:self.n_owned]


def subdomain(grid: Grid, owned: np.ndarray, ghost: np.ndarray):
    """Local grid of the cells `owned` (interior) and `ghost` (global
    numbers, each in increasing order): (Grid, local cell -> global,
    local connection -> global).  Connections with at least one owned end, in
    the global order, ends relabelled, roles kept."""
    cells = np.concatenate([owned, ghost]).astype(np.int64)
    local = np.full(grid.nb, -1, np.int64)
    local[cells] = np.arange(cells.size)
    b = np.asarray(grid.conn_b, np.int64)
    e = np.asarray(grid.conn_e, np.int64)
    is_owned = np.zeros(grid.nb, bool)
    is_owned[owned] = True
    keep = (is_owned[b] | is_owned[e]) & (local[b] >= 0) & (local[e] >= 0)
    conns = np.nonzero(keep)[0]
    g = Grid(v=np.asarray(grid.v)[cells], depth=np.asarray(grid.depth)[cells],
             poro_init=np.asarray(grid.poro_init)[cells], conn_b=local[b[conns]].astype(np.uint32),
             conn_e=local[e[conns]].astype(np.uint32), conn_trans=np.asarray(grid.conn_trans)[conns],
             nb_interior=int(owned.size))
    return g, cells, conns


def layer_bounds(nz: int, nranks: int):
    """Owned layers of each rank: nz split as evenly as possible, lower ranks
    taking the extra layers."""
    base, extra = divmod(nz, nranks)
    k = [0]
    for r in range(nranks):
        k.append(k[-1] + base + (1 if r < extra else 0))
    return [(k[r], k[r + 1]) for r in range(nranks)]


def partition(grid: Grid, owner, nranks: int, layers=None):
    """Subdomains of `grid` from the owner rank of each cell: rank r owns the
    cells with owner r and holds as ghosts every other cell connected to one
    of them.  send[q] / recv[q] list, in the global order, the owned cells
    rank q holds as ghosts and the ghosts rank q owns (local numbers), so
    that the two sides of each exchange agree.  `layers` gives each rank's
    owned layers, for the record."""
    owner = np.asarray(owner, np.int64)
    if owner.shape != (grid.nb,) or owner.min() < 0 or owner.max() >= nranks:
        raise ValueError("owner must give a rank in [0, nranks) for every cell")
    b = np.asarray(grid.conn_b, np.int64)
    e = np.asarray(grid.conn_e, np.int64)
    cross = owner[b] != owner[e]
    # a crossing connection makes each end a ghost of the other end's owner
    g_rank = np.concatenate([owner[b[cross]], owner[e[cross]]])
    g_cell = np.concatenate([e[cross], b[cross]])
    ghosts = [np.unique(g_cell[g_rank == r]) for r in range(nranks)]
    subs = []
    for r in range(nranks):
        owned = np.nonzero(owner == r)[0]
        if not owned.size:
            raise ValueError(f"rank {r} owns no cell")
        ghost = ghosts[r]
        g, cells, conns = subdomain(grid, owned, ghost)
        n = owned.size
        send, recv = {}, {}
        for q in range(nranks):
            if q == r:
                continue
            mine = ghosts[q][owner[ghosts[q]] == r]
            if mine.size:
                send[q] = np.searchsorted(owned, mine)
            theirs = ghost[owner[ghost] == q]
            if theirs.size:
                recv[q] = n + np.searchsorted(ghost, theirs)
        subs.append(Subdomain(r, layers[r] if layers is not None else None, cells, n, g, conns, send, recv))
    return subs


def zslab_partition(grid: Grid, nx: int, ny: int, nz: int, nranks: int, cell_index=None):
    """Subdomains of a grid of nx * ny * nz cells (order k, j, i) in slabs of
    whole layers (partition by layer).  cell_index: for a grid of the active
    cells of that grid, each cell's index in it (the geometry's act2all from
    deck.grid_from_deck or the grid ingest); None when every cell is
    present.  Needs at least one layer per rank."""
    if nranks < 1 or nranks > nz:
        raise ValueError(f"{nranks} ranks for {nz} layers")
    if cell_index is None:
        if grid.nb != nx * ny * nz:
            raise ValueError("grid size does not match nx * ny * nz")
        cell_index = np.arange(grid.nb)
    cell_index = np.asarray(cell_index, np.int64)
    if cell_index.shape != (grid.nb,):
        raise ValueError("cell_index must give one index per cell")
    bounds = layer_bounds(nz, nranks)
    rank_of_layer = np.repeat(np.arange(nranks), [k1 - k0 for k0, k1 in bounds])
    return partition(grid, rank_of_layer[cell_index // (nx * ny)], nranks, layers=bounds)


def pack(sub: Subdomain, values: np.ndarray, width: int) -> dict:
    """Per neighbour, the values of the owned cells it holds as ghosts."""
    v = np.asarray(values, np.float64).reshape(-1, width)
    return {nbr: np.ascontiguousarray(v[idx]) for nbr, idx in sub.send.items()}


def unpack(sub: Subdomain, values: np.ndarray, width: int, received: dict) -> np.ndarray:
    """A copy of values (local cells, width entries per cell) whose ghost
    cells hold the values received from their owners."""
    out = np.array(values, np.float64, copy=True).reshape(-1, width)
    for nbr, idx in sub.recv.items():
        out[idx] = np.asarray(received[nbr]).reshape(idx.size, width)
    return out.reshape(np.shape(values))


def exchange_in_process(subs, arrays, width: int):
    """The halo exchange of subdomains all held by this process: arrays[r]
    holds subdomain r's local values; returns the arrays with ghosts filled."""
    outgoing = [pack(s, a, width) for s, a in zip(subs, arrays)]
    return [unpack(s, a, width, {nbr: outgoing[nbr][s.rank] for nbr in s.recv}) for s, a in zip(subs, arrays)]


class HaloExchange:
    """Owner-to-ghost exchange and global reductions for one subdomain, over
    a torch.distributed process group (gloo: host buffers), which must be
    initialised."""

    def __init__(self, sub: Subdomain):
        import torch.distributed as dist
        self.dist = dist
        self.sub = sub

    def exchange(self, values: np.ndarray, width: int) -> np.ndarray:
        import torch
        reqs, recv = [], {}
        sends = {nbr: torch.from_numpy(b) for nbr, b in pack(self.sub, values, width).items()}
        for nbr, t in sends.items():
            reqs.append(self.dist.isend(t, nbr))
        for nbr, idx in self.sub.recv.items():
            recv[nbr] = torch.empty((idx.size, width), dtype=torch.float64)
            reqs.append(self.dist.irecv(recv[nbr], nbr))
        for q in reqs:
            q.wait()
        return unpack(self.sub, values, width, {nbr: t.numpy() for nbr, t in recv.items()})

    def max_norms(self, norms):
        """Global maxima of the relative residual norms (maxRelRes_V,
        maxRelRes_N) over the ranks, as the reference's MPI_Allreduce."""
        import torch
        t = torch.tensor([float(norms[0]), float(norms[1])], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t[0]), float(t[1])
