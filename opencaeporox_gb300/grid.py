"""Orthogonal-grid ingest: cells, connections and transmissibilities in the
reference's order, without running the reference.

Follows PreParamGridWell::SetupActiveConnOrthogonalGridSM
(src/PreParamGridWell.cpp:1140-1216): cells are visited in (k, j, i) order
and each cell's forward neighbours +x, +y, +z give the connections with
eId > bId (Reservoir::SetupDistParamGrid, src/Reservoir.cpp:324-384), with
half-cell areas 2*dy*dz/dx etc.; transmissibility as in
BulkConnTransMethod01::CalTrans (src/BulkConnFunc.cpp:15-67):
T = CONV_DARCY / (1/(ntg*k*areaB) + 1/(ntg*k*areaE)) (no ntg along z).
All cells active.
"""
from __future__ import annotations

import numpy as np

from .fim import Grid


def orthogonal_grid(nx, ny, nz, dx, dy, dz, tops, kx, ky, kz, poro, ntg=None, conv_darcy=0.008527):
    n = nx * ny * nz
    f = lambda a: np.broadcast_to(np.asarray(a, np.float64), (n,)).copy() if np.ndim(a) == 0 else np.asarray(a, np.float64).ravel()
    dx, dy, dz, kx, ky, kz, poro = (f(a) for a in (dx, dy, dz, kx, ky, kz, poro))
    ntg = np.ones(n) if ntg is None else f(ntg)
    v = dx * dy * dz * ntg
    # depth: cell centre, tops of the first layer plus accumulated thickness
    top = np.empty(n)
    layer = nx * ny
    top[:layer] = f(tops)[:layer] if np.ndim(tops) else tops
    for k in range(1, nz):
        top[k * layer:(k + 1) * layer] = top[(k - 1) * layer:k * layer] + dz[(k - 1) * layer:k * layer]
    depth = top + dz / 2
    idx = np.arange(n)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // layer
    # per direction, vectorised; then ordered by (bId, direction x < y < z) as
    # the reference's cell loop emits them
    bs, es, ts, keys = [], [], [], []
    for d, (cond, step, area, perm) in enumerate((
            (i < nx - 1, 1, 2 * dy * dz / dx, kx * ntg),
            (j < ny - 1, nx, 2 * dz * dx / dy, ky * ntg),
            (k < nz - 1, layer, 2 * dx * dy / dz, kz))):
        bId = idx[cond]
        eId = bId + step
        T1 = perm[bId] * area[bId]
        T2 = perm[eId] * area[eId]
        bs.append(bId)
        es.append(eId)
        ts.append(1.0 / (1 / T1 + 1 / T2) * conv_darcy)
        keys.append(bId * 3 + d)
    order = np.argsort(np.concatenate(keys), kind="stable")
    b_list = np.concatenate(bs)[order]
    e_list = np.concatenate(es)[order]
    t_list = np.concatenate(ts)[order]
    return Grid(v=v, depth=depth, poro_init=poro, conn_b=np.array(b_list, np.uint32),
                conn_e=np.array(e_list, np.uint32), conn_trans=np.array(t_list))
