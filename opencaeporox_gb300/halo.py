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

* ``zslab_partition`` cuts cells (k, j, i), i fastest, into R slabs of
  consecutive layers.  Subdomain r owns the layers [k0, k1) and has up to one
  ghost layer below and one above.  Its local cell numbers are the owned
  cells first, in the global order, then the ghost cells, in the global
  order (so the context's nb_interior is the owned count).  Its connections
  are the global connections with at least one owned end, in the global
  order, each end keeping its role (bId, eId): the owned rows of the
  subdomain's residual and Jacobian are then bit-identical to the same rows
  of the whole grid.
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
    layers: tuple            # owned layers [k0, k1)
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


def zslab_partition(grid: Grid, nx: int, ny: int, nz: int, nranks: int):
    """Subdomains of a grid of nx * ny * nz cells (order k, j, i; every cell
    active) in slabs of whole layers, one ghost layer on each inner side.
    Needs at least one layer per rank."""
    if nranks < 1 or nranks > nz:
        raise ValueError(f"{nranks} ranks for {nz} layers")
    if grid.nb != nx * ny * nz:
        raise ValueError("grid size does not match nx * ny * nz")
    layer = nx * ny
    bounds = layer_bounds(nz, nranks)
    subs = []
    for r, (k0, k1) in enumerate(bounds):
        owned = np.arange(k0 * layer, k1 * layer)
        below = np.arange((k0 - 1) * layer, k0 * layer) if r > 0 else np.zeros(0, np.int64)
        above = np.arange(k1 * layer, (k1 + 1) * layer) if r < nranks - 1 else np.zeros(0, np.int64)
        ghost = np.concatenate([below, above])
        g, cells, conns = subdomain(grid, owned, ghost)
        n = owned.size
        send, recv = {}, {}
        if r > 0:
            send[r - 1] = np.arange(0, layer)                  # my lowest owned layer
            recv[r - 1] = np.arange(n, n + layer)              # the ghost layer below
        if r < nranks - 1:
            send[r + 1] = np.arange(n - layer, n)              # my highest owned layer
            off = n + (layer if r > 0 else 0)
            recv[r + 1] = np.arange(off, off + layer)          # the ghost layer above
        subs.append(Subdomain(r, (k0, k1), cells, n, g, conns, send, recv))
    return subs


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
