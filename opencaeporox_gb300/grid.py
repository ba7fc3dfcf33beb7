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

Corner-point ingest (corner_point_grid) follows OCP_COORD::SetupCornerPoints
(src/CornerGrid.cpp:245-1150) for grids whose neighbouring faces match
(consistent ZCORN, no faults): corner points on the pillars, cell volume,
centre and depth, one half connection per face with the effective area
A.d/(d.d) (ConnGrid::AddHalfConn, :22-53), pairs with both halves positive
(:1120-1150), then the same transmissibility as the orthogonal grid.  Faults
(partly overlapping faces and their non-neighbour connections) are not
handled: such grids are rejected.
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


TINY = 1e-8     # include/OCPConst.hpp
TEENY = 1e-10


def _pillar_points(coord, nx, ny, z, I, J):
    """x, y of the points at depth z on pillars (I, J) (arrays): on a vertical
    pillar its top x, y; otherwise linear along the pillar in z
    (SetupCornerPoints, src/CornerGrid.cpp:262-285)."""
    c = coord.reshape(ny + 1, nx + 1, 2, 3)
    xt, yt, zt = c[J, I, 0, 0], c[J, I, 0, 1], c[J, I, 0, 2]
    xb, yb, zb = c[J, I, 1, 0], c[J, I, 1, 1], c[J, I, 1, 2]
    vert = (np.abs(xt - xb) < TINY) & (np.abs(yt - yb) < TINY)
    with np.errstate(invalid="ignore", divide="ignore"):
        x = np.where(vert, xt, xb - (zb - z) / (zb - zt) * (xb - xt))
        y = np.where(vert, yt, yb - (zb - z) / (zb - zt) * (yb - yt))
    return np.stack([x, y, z], axis=-1)


def _hex_volume(P):
    """Volume of the trilinear hexahedron with corners P[..., 8, 3]
    (p0..p3 the top face counter-clockwise from (i, j), p4..p7 below them):
    the integral of det(dX/dxi) over the unit cube by the 2 x 2 x 2 Gauss
    rule, which is exact here (det is of degree <= 2 in each variable)."""
    g = np.array([0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)])
    loc = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    vol = np.zeros(P.shape[:-2])
    for a in g:
        for b in g:
            for c in g:
                xi = np.array([a, b, c])
                # trilinear shape functions and their derivatives at xi
                w = np.where(loc > 0, xi, 1 - xi)                       # [8, 3]
                dN = np.empty((8, 3))
                for d in range(3):
                    f = np.where(loc[:, d] > 0, 1.0, -1.0)
                    o = [e for e in range(3) if e != d]
                    dN[:, d] = f * w[:, o[0]] * w[:, o[1]]
                J = np.einsum("...kc,kd->...cd", P, dN)                 # dX_c / dxi_d
                vol = vol + np.linalg.det(J) / 8.0
    return vol


def _area_vector(f0, f1, f2, f3):
    """Area vector of the quadrilateral f0 f1 f2 f3: half the cross product of
    its diagonals (equal to HexahedronFace::CalAreaVector's two triangles)."""
    return 0.5 * np.cross(f2 - f0, f3 - f1)


def corner_point_grid(nx, ny, nz, coord, zcorn, kx, ky, kz, poro, ntg=None, conv_darcy=0.008527,
                      return_geometry=False):
    """Cells and connections of a corner-point grid (COORD, ZCORN in Eclipse
    order), in the reference's order; see the module docstring."""
    n = nx * ny * nz
    f = lambda a: np.broadcast_to(np.asarray(a, np.float64), (n,)).copy() if np.ndim(a) == 0 else np.asarray(a, np.float64).ravel()
    kx, ky, kz, poro = (f(a) for a in (kx, ky, kz, poro))
    ntg = np.ones(n) if ntg is None else f(ntg)
    coord = np.asarray(coord, np.float64).ravel()
    z = np.asarray(zcorn, np.float64).reshape(nz, 2, ny, 2, nx, 2)   # [K][top/bottom][J][y-/y+][I][x-/x+]
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    corners = []
    # p0..p3 top, p4..p7 bottom; pillars (I,J), (I+1,J), (I+1,J+1), (I,J+1)
    for tb in range(2):
        for (dj, di) in ((0, 0), (0, 1), (1, 1), (1, 0)):
            corners.append(_pillar_points(coord, nx, ny, z[K, tb, J, dj, I, di], I + di, J + dj))
    P = np.stack(corners, axis=-2).reshape(n, 8, 3)
    v = np.abs(_hex_volume(P - P[:, :1]))   # corners relative to p0: the same Jacobian, less cancellation
    center = P.sum(axis=1) * 0.125
    depth = center[:, 2]
    p = [P[:, q] for q in range(8)]
    faces = {  # per direction: the face's corners in HexahedronFace order
        "xm": (p[0], p[4], p[7], p[3]), "xp": (p[2], p[6], p[5], p[1]),
        "ym": (p[1], p[5], p[4], p[0]), "yp": (p[3], p[7], p[6], p[2]),
        "zm": (p[0], p[3], p[2], p[1]), "zp": (p[5], p[6], p[7], p[4])}
    c = coord.reshape(ny + 1, nx + 1, 2, 3)
    flag = 1.0 if c[1, 0, 0, 1] > c[0, 0, 0, 1] else -1.0
    half = {}
    for d, fc in faces.items():
        A = _area_vector(*fc)
        dv = 0.25 * (fc[0] + fc[1] + fc[2] + fc[3]) - center
        half[d] = np.einsum("ij,ij->i", A, dv) / np.einsum("ij,ij->i", dv, dv) * flag
    # faults: a face that does not coincide with its neighbour's
    idx = np.arange(n)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    for (d, dn, cond, step) in (("xp", "xm", i < nx - 1, 1), ("yp", "ym", j < ny - 1, nx),
                                ("zp", "zm", k < nz - 1, nx * ny)):
        a = idx[cond]
        mine = np.stack(faces[d], axis=1)[a]
        # the neighbour's face lists the shared corners in the opposite order
        theirs = np.stack(faces[dn], axis=1)[a + step][:, ::-1]
        if a.size and np.max(np.abs(mine[..., 2] - theirs[..., 2])) > TEENY:
            raise ValueError("corner-point grid with non-matching faces (faults): not supported")
    bs, es, ts, keys, aB, aE, dirs = [], [], [], [], [], [], []
    for dd, (d, dn, cond, step, perm) in enumerate((
            ("xp", "xm", i < nx - 1, 1, kx * ntg),
            ("yp", "ym", j < ny - 1, nx, ky * ntg),
            ("zp", "zm", k < nz - 1, nx * ny, kz))):
        b = idx[cond]
        e = b + step
        hb, he = half[d][b], half[dn][e]
        ok = (hb > 0) & (he > 0)
        b, e, hb, he = b[ok], e[ok], hb[ok], he[ok]
        if dd < 2:
            T1 = ntg[b] * (kx if dd == 0 else ky)[b] * hb
            T2 = ntg[e] * (kx if dd == 0 else ky)[e] * he
        else:
            T1 = kz[b] * hb
            T2 = kz[e] * he
        bs.append(b); es.append(e); aB.append(hb); aE.append(he)
        ts.append(1.0 / (1 / T1 + 1 / T2) * conv_darcy)
        keys.append(b * 3 + dd)
        dirs.append(np.full(b.size, dd))
    order = np.argsort(np.concatenate(keys), kind="stable")
    cat = lambda L: np.concatenate(L)[order]
    grid = Grid(v=v, depth=depth, poro_init=poro, conn_b=np.array(cat(bs), np.uint32),
                conn_e=np.array(cat(es), np.uint32), conn_trans=cat(ts))
    if return_geometry:
        return grid, dict(areaB=cat(aB), areaE=cat(aE), direction=cat(dirs), center=center, corners=P)
    return grid
