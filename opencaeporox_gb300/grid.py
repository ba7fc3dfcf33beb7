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
(src/CornerGrid.cpp:245-1150): corner points on the pillars, cell volume,
centre and depth; per cell its half connections with the effective area
A.d/(d.d) (ConnGrid::AddHalfConn, :22-53) in the reference's order (x-, x+,
y-, y+, z-, z+; along x and y the neighbour in the same layer, then the
non-neighbour connections (NNCs) of a fault, upward then downward); pairs of
half connections with both halves positive (:1120-1150), then the same
transmissibility as the orthogonal grid.  Faults are handled as the
reference handles them: OCP_COORD::SetAllFlags (:173-243) classifies the
overlap of two lateral faces by the depths of their corners on the shared
pillars, a quadrilateral overlap takes the area vector of the intersected
face, any other overlap the reference's piecewise area of the faces
projected on the vertical plane (CalAreaNotQuadr, src/UtilMesh.cpp:202-565)
with the direction of the cell's own face.  The search for NNCs keeps the
reference's flags from one probe to the next, so it visits the same cells.
Every step runs over arrays of faces; the NNC search advances all faulted
faces one layer per pass.
"""
from __future__ import annotations

import numpy as np

from .fim import Grid


def active_cells(v, poro, actnum=None, eps_v=1e-6, eps_poro=1e-6):
    """Cells the reference keeps: pore fraction and volume at least 1e-6 and
    ACTNUM not 0 (ActiveGridCheck::CheckActivityIsoT,
    src/PreParamGridWell.cpp:856-872)."""
    act = (poro >= eps_poro) & (v >= eps_v)
    if actnum is not None:
        act &= np.asarray(actnum).ravel() != 0
    return act


def _trans(mult, T1, T2, conv_darcy):
    """BulkConnTransMethod01::CalTrans (src/BulkConnFunc.cpp:15-67)."""
    return mult / (1 / T1 + 1 / T2) * conv_darcy


def _compress(n, act, b, e, t, v, depth, poro, geo):
    """The active cells' grid: cells renumbered in order, connections between
    active cells (their order is kept)."""
    a2 = np.full(n, -1, np.int64)
    a2[act] = np.arange(int(act.sum()))
    keep = act[b] & act[e]
    g = Grid(v=v[act], depth=depth[act], poro_init=poro[act], conn_b=a2[b[keep]].astype(np.uint32),
             conn_e=a2[e[keep]].astype(np.uint32), conn_trans=t[keep])
    geo = {k: (x[act] if np.ndim(x) and len(x) == n else x) for k, x in geo.items()}
    geo["act2all"] = np.nonzero(act)[0]
    geo["conn_keep"] = keep
    return g, geo


def orthogonal_grid(nx, ny, nz, dx, dy, dz, tops, kx, ky, kz, poro, ntg=None, conv_darcy=0.008527, actnum=None,
                    multz=None, return_geometry=False):
    """Cells and connections of a block-centred grid in the reference's order
    (see the module docstring).  As the reference: the pore fraction is
    PORO * NTG when NTG is given, the volume dx dy dz, and NTG scales the
    transmissibility across x and y; only active cells are kept (active_cells,
    with ACTNUM); a cell whose neighbour across x (or y) is inactive gets no
    connection in the later directions either (the loop's `continue`,
    src/PreParamGridWell.cpp:1166-1167); MULTZ of the upper cell scales the
    transmissibility across z.  return_geometry adds, per active cell, its
    index among all cells, dx, dy, dz, NTG and the permeabilities."""
    n = nx * ny * nz
    f = lambda a: np.broadcast_to(np.asarray(a, np.float64), (n,)).copy() if np.ndim(a) == 0 else np.asarray(a, np.float64).ravel()
    dx, dy, dz, kx, ky, kz, poro = (f(a) for a in (dx, dy, dz, kx, ky, kz, poro))
    ntg_given = ntg is not None
    ntg = f(ntg) if ntg_given else np.ones(n)
    if ntg_given:
        poro = poro * ntg
    v = dx * dy * dz
    # depth of the cell centres: the top layer from TOPS, then each layer half
    # a thickness below the centre of the one above plus half its own
    # (CalDepthVOrthogonalGrid, src/PreParamGridWell.cpp:1036-1064)
    layer = nx * ny
    depth = np.empty(n)
    t = np.broadcast_to(np.asarray(tops, np.float64), (layer,)) if np.ndim(tops) == 0 else np.asarray(tops, np.float64).ravel()[:layer]
    depth[:layer] = t + dz[:layer] / 2
    for k in range(1, nz):
        cur, prev = slice(k * layer, (k + 1) * layer), slice((k - 1) * layer, k * layer)
        depth[cur] = depth[prev] + dz[prev] / 2 + dz[cur] / 2
    act = active_cells(v, poro, actnum)
    idx = np.arange(n)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // layer
    # per direction, vectorised; a cell stops at its first inactive neighbour
    # (x, then y, then z); then ordered by (bId, direction x < y < z) as the
    # reference's cell loop emits them
    mz = np.ones(n) if multz is None else f(multz)
    going = act.copy()
    bs, es, ts, keys = [], [], [], []
    for d, (cond, step, area, perm, mult) in enumerate((
            (i < nx - 1, 1, 2 * dy * dz / dx, kx * ntg, np.ones(n)),
            (j < ny - 1, nx, 2 * dz * dx / dy, ky * ntg, np.ones(n)),
            (k < nz - 1, layer, 2 * dx * dy / dz, kz, mz))):
        cand = going & cond
        nb_ = np.minimum(idx + step, n - 1)
        ok = cand & act[nb_]
        going &= ~(cand & ~act[nb_])
        bId = idx[ok]
        eId = bId + step
        bs.append(bId)
        es.append(eId)
        ts.append(_trans(mult[bId], perm[bId] * area[bId], perm[eId] * area[eId], conv_darcy))
        keys.append(bId * 3 + d)
    order = np.argsort(np.concatenate(keys), kind="stable")
    b_list = np.concatenate(bs)[order]
    e_list = np.concatenate(es)[order]
    t_list = np.concatenate(ts)[order]
    grid, geo = _compress(n, act, b_list, e_list, t_list, v, depth, poro,
                          dict(dx=dx, dy=dy, dz=dz, ntg=ntg, kx=kx, ky=ky, kz=kz))
    return (grid, geo) if return_geometry else grid


TINY = 1e-8     # include/OCPConst.hpp:30
TEENY = 1e-3    # include/CornerGrid.hpp:21: depth tolerance of the corner-point fault tests


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
    Pt = np.ascontiguousarray(np.swapaxes(P, -1, -2)).reshape(-1, 8)   # rows (cell, coordinate)
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
                J = (Pt @ dN).reshape(P.shape[:-2] + (3, 3))          # dX_c / dxi_d
                det = (J[..., 0, 0] * (J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1])
                       - J[..., 0, 1] * (J[..., 1, 0] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 0])
                       + J[..., 0, 2] * (J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]))
                vol = vol + det / 8.0
    return vol


def _cross(a, b):
    """a x b, component by component as the reference writes it."""
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _area_vector(f0, f1, f2, f3):
    """Area vector of the quadrilateral f0 f1 f2 f3 as the sum of the
    triangles (f2, f1, f0) and (f0, f3, f2) (HexahedronFace::CalAreaVector,
    src/UtilMesh.cpp:148-157)."""
    return 0.5 * (_cross(f2 - f1, f0 - f1) + _cross(f0 - f3, f2 - f3))


def _face_flags(of, f):
    """The overlap of a lateral face f with the other cell's face of (the
    points of both as [m, 4, 3], p0/p3 the upper edge, p1/p2 the lower edge,
    p0/p1 on one pillar and p3/p2 on the other), by the depths of their
    corners (OCP_COORD::SetAllFlags, src/CornerGrid.cpp:173-243).  Returns
    (inter, jump, quad, up, down): the intersected face, no overlap, a
    quadrilateral overlap, and whether the search for NNCs continues upward or
    downward."""
    z, oz = f[..., 2], of[..., 2]
    d01, d32 = f[:, 0] - f[:, 1], f[:, 3] - f[:, 2]
    line = (np.sqrt(d01[:, 0] * d01[:, 0] + d01[:, 1] * d01[:, 1] + d01[:, 2] * d01[:, 2]) <= TEENY) & \
           (np.sqrt(d32[:, 0] * d32[:, 0] + d32[:, 1] * d32[:, 1] + d32[:, 2] * d32[:, 2]) <= TEENY)
    inter = f.copy()
    flags = []
    up = np.zeros(len(f), bool)
    down = np.zeros(len(f), bool)
    for q in range(4):
        upper = q in (0, 3)       # the upper edge takes the deeper point, the lower edge the shallower
        take = (oz[:, q] > z[:, q] + TEENY) if upper else (oz[:, q] < z[:, q] - TEENY)
        other = (oz[:, q] < z[:, q] - TEENY) if upper else (oz[:, q] > z[:, q] + TEENY)
        inter[take, q] = of[take, q]
        if upper:
            up |= take
            flags.append(np.where(take, 1, np.where(other, -1, 0)))
        else:
            down |= take
            flags.append(np.where(take, -1, np.where(other, 1, 0)))
    jump = ((oz[:, 1] <= z[:, 0]) & (oz[:, 2] <= z[:, 3])) | ((oz[:, 0] >= z[:, 1]) & (oz[:, 3] >= z[:, 2]))
    quad = (flags[0] * flags[3] >= 0) & (oz[:, 0] <= z[:, 1]) & (oz[:, 3] <= z[:, 2]) & \
           (flags[1] * flags[2] >= 0) & (oz[:, 1] >= z[:, 0]) & (oz[:, 2] >= z[:, 3])
    # a face reduced to a line overlaps nothing and starts no search
    inter[line] = f[line]
    jump = jump | line
    up &= ~line
    down &= ~line
    return inter, jump, quad, up, down


def _crossing(a0, a1, b0, b1):
    """Crossing point of the lines a0 a1 and b0 b1 in the plane (Cramer's
    rule), or a0 when they are parallel (CalCrossingPoint,
    src/UtilMesh.cpp:166-200)."""
    a11, a12 = a1[:, 1] - a0[:, 1], a0[:, 0] - a1[:, 0]
    a21, a22 = b1[:, 1] - b0[:, 1], b0[:, 0] - b1[:, 0]
    r1 = a11 * a0[:, 0] + a12 * a0[:, 1]
    r2 = a21 * b0[:, 0] + a22 * b0[:, 1]
    det = a11 * a22 - a12 * a21
    ok = np.abs(det) > 1e-10
    with np.errstate(divide="ignore", invalid="ignore"):
        p = np.stack([(r1 * a22 - r2 * a12) / det, (a11 * r2 - a21 * r1) / det], axis=-1)
    return np.where(ok[:, None], p, a0)


def _quad_z(p0, p1, p2, p3):
    """|z| of the area vector of a quadrilateral in the plane."""
    v0, v1, v2, v3 = p2 - p1, p0 - p1, p0 - p3, p2 - p3
    return np.abs(0.5 * ((v0[:, 0] * v1[:, 1] - v0[:, 1] * v1[:, 0]) + (v2[:, 0] * v3[:, 1] - v2[:, 1] * v3[:, 0])))


def _tri_z(p1, p2, p3):
    """Area of the triangle p1 p2 p3 in the plane."""
    a, b = p1 - p3, p2 - p3
    return np.abs(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]) * 0.5


def overlap_pattern(f, g):
    """The crossing points of the edges of two faces projected on a vertical
    plane (as _overlap_area takes them) and the pattern of which edge pairs
    cross strictly inside face f's edge: bit 0 upper/upper, 1 lower of f with
    upper of g, 2 upper of f with lower of g, 3 lower/lower."""
    F = [f[:, q] for q in range(4)]
    G = [g[:, q] for q in range(4)]
    cp = [_crossing(F[0], F[1], G[0], G[1]), _crossing(F[2], F[3], G[0], G[1]),
          _crossing(F[0], F[1], G[2], G[3]), _crossing(F[2], F[3], G[2], G[3])]
    edge = [(0, 1), (2, 3), (0, 1), (2, 3)]
    iret = np.zeros(len(f), np.int64)
    for b in range(4):
        a0, a1 = F[edge[b][0]], F[edge[b][1]]
        iret += np.where((cp[b][:, 0] - a0[:, 0]) * (cp[b][:, 0] - a1[:, 0]) < 0, 1 << b, 0)
    return cp, iret


def _overlap_area(f, g):
    """Area common to two faces projected on a vertical plane (points
    [m, 4, 2], x along the plane, y the depth; p0/p1 the upper edge, p3/p2
    the lower edge), by the reference's case table on which of the four
    edge pairs cross (CalAreaNotQuadr, src/UtilMesh.cpp:202-565): the
    overlap is cut into one or two quadrilaterals or a triangle from the
    crossing points and the inner corners, some closed at a midpoint as the
    reference closes them.  Pairs with any other crossing pattern get 0."""
    def sel(c, a, b):
        return np.where(c[:, None], a, b)

    def mid(a, b):
        return np.stack([0.5 * (a[:, 0] + b[:, 0]), 0.5 * (a[:, 1] + b[:, 1])], axis=-1)

    F = [f[:, q] for q in range(4)]
    G = [g[:, q] for q in range(4)]
    cp, iret = overlap_pattern(f, g)
    y = lambda P: P[:, 1]
    # the inner corners of the two faces: on each pillar the deeper of the
    # upper corners (0, 1) and the shallower of the lower corners (3, 2)
    in0 = sel(y(F[0]) > y(G[0]), F[0], G[0])
    in1 = sel(y(F[1]) > y(G[1]), F[1], G[1])
    in3 = sel(y(F[3]) > y(G[3]), G[3], F[3])
    in2 = sel(y(F[2]) > y(G[2]), G[2], F[2])
    area = np.zeros(len(f))
    for case in (1, 2, 3, 4, 5, 8, 9, 10, 11, 12, 13, 15):
        m = iret == case
        if not m.any():
            continue
        Fm, Gm, C = [P[m] for P in F], [P[m] for P in G], [P[m] for P in cp]
        i0, i1, i2, i3 = in0[m], in1[m], in2[m], in3[m]
        fy, gy = [y(P) for P in Fm], [y(P) for P in Gm]
        if case == 1:
            m32 = mid(i3, i2)
            a = _quad_z(i0, C[0], m32, i3) + _quad_z(C[0], i1, i2, m32)
        elif case == 2:
            c = fy[3] > gy[0]
            a = _tri_z(sel(c, Fm[3], Fm[2]), sel(c, Gm[0], Gm[1]), C[1])
        elif case == 3:
            c = fy[0] < gy[0]
            a = _quad_z(C[0], C[1], sel(c, Fm[2], Fm[3]), sel(c, Fm[1], Fm[0]))
        elif case == 4:
            c = fy[0] < gy[3]
            a = _tri_z(sel(c, Fm[0], Fm[1]), sel(c, Gm[3], Gm[2]), C[2])
        elif case == 5:
            c = gy[3] > fy[0]
            a = _quad_z(C[0], C[2], sel(c, Gm[3], Gm[2]), sel(c, Gm[0], Gm[1]))
        elif case == 8:
            m01 = mid(i0, i1)
            a = _quad_z(i0, m01, C[3], i3) + _quad_z(m01, i1, i2, C[3])
        elif case == 9:
            a = _quad_z(i0, C[0], C[3], i3) + _quad_z(C[0], i1, i2, C[3])
        elif case == 10:
            c = fy[2] > gy[1]
            a = _quad_z(C[1], C[3], sel(c, Gm[1], Gm[3]), sel(c, Gm[2], Gm[0]))
        elif case == 11:
            c = fy[0] < gy[0]
            p1, p2 = sel(c, Fm[1], Fm[0]), sel(c, Gm[2], Gm[3])
            m01 = mid(C[0], p1)
            a = _quad_z(C[0], m01, C[3], C[1]) + _quad_z(m01, p1, p2, C[3])
        elif case == 12:
            c = fy[2] > gy[2]
            a = _quad_z(C[2], C[3], sel(c, Fm[3], Fm[2]), sel(c, Fm[0], Fm[1]))
        elif case == 13:
            c = fy[2] > gy[2]
            p0, p3 = sel(c, Gm[0], Gm[1]), sel(c, Fm[3], Fm[2])
            m01 = mid(p0, C[0])
            a = _quad_z(p0, m01, C[3], p3) + _quad_z(m01, C[0], C[2], C[3])
        else:
            a = _quad_z(C[0], C[2], C[3], C[1])
        area[m] = a
    return area


def _projected_area(F, O, Fa, axis):
    """Area vector of the overlap of lateral faces F and O ([m, 4, 3]) that is
    not a quadrilateral: the overlap's area on the vertical plane across the
    face (y-z for a face across x, x-z across y) with the direction of F's own
    area vector Fa, scaled so that its component across the face is that area
    (src/CornerGrid.cpp:410-432).  A face whose component across is below
    1e-6 keeps its own area vector, as in the reference."""
    h = 1 if axis == 0 else 0
    # the projected corners with the upper edge first (CalAreaNotQuadr's order)
    order = [3, 0, 1, 2] if axis == 0 else [0, 3, 2, 1]
    f = F[:, order][:, :, [h, 2]]
    g = O[:, order][:, :, [h, 2]]
    a = _overlap_area(f, g)
    out = Fa.copy()
    c = Fa[:, axis]
    ok = np.abs(c) >= 1e-6
    o = [q for q in range(3) if q != axis]
    with np.errstate(divide="ignore", invalid="ignore"):
        for q in o:
            out[ok, q] = Fa[ok, q] / np.abs(c[ok]) * a[ok]
    out[ok, axis] = np.where(c[ok] >= 0, 1.0, -1.0) * a[ok]
    return out


def corner_point_grid(nx, ny, nz, coord, zcorn, kx, ky, kz, poro, ntg=None, conv_darcy=0.008527,
                      return_geometry=False, actnum=None, multz=None):
    """Cells and connections of a corner-point grid (COORD, ZCORN in Eclipse
    order), in the reference's order; see the module docstring.  As the
    reference: the pore fraction is PORO * NTG when NTG is given, NTG scales
    the transmissibility across x and y, MULTZ of the upper cell the one
    across z; the connections are found among all cells, then only active
    cells (active_cells, with ACTNUM) and the connections between them are
    kept.  return_geometry adds the half areas, the axis of each connection,
    and per active cell its index among all cells, dx, dy, dz (between the
    centres of opposite faces), NTG and the permeabilities."""
    n = nx * ny * nz
    f = lambda a: np.broadcast_to(np.asarray(a, np.float64), (n,)).copy() if np.ndim(a) == 0 else np.asarray(a, np.float64).ravel()
    kx, ky, kz, poro = (f(a) for a in (kx, ky, kz, poro))
    ntg_given = ntg is not None
    ntg = f(ntg) if ntg_given else np.ones(n)
    if ntg_given:
        poro = poro * ntg
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
    c = coord.reshape(ny + 1, nx + 1, 2, 3)
    flag = 1.0 if c[1, 0, 0, 1] > c[0, 0, 0, 1] else -1.0
    # half connections, per cell in the reference's order: slot = direction
    # (x-, x+, y-, y+, z-, z+) * (2 nz + 1) + 0 for the neighbour in the same
    # layer, 1.. for the NNCs upward, nz + 1.. for those downward.  Per
    # direction the face's corners in HexahedronFace order, and the corners of
    # the other cell's face toward it with the same corners first.
    FACE = ((0, 4, 7, 3), (2, 6, 5, 1), (1, 5, 4, 0), (3, 7, 6, 2), (0, 3, 2, 1), (5, 6, 7, 4))
    OTHER = ((1, 5, 6, 2), (3, 7, 4, 0), (2, 6, 7, 3), (0, 4, 5, 1))
    idx = np.arange(n)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    nxny = nx * ny
    span = 2 * nz + 1
    hb, he, hslot, hAd = [], [], [], []

    def emit(cells, others, slot, area, face):
        """Half connections cells -> others with area vector `area`; the
        effective area A.d/(d.d) with d from the cell's centre to the centre
        of its own face (ConnGrid::AddHalfConn, src/CornerGrid.cpp:22-53)."""
        D = 0.25 * (face[:, 0] + face[:, 1] + face[:, 2] + face[:, 3]) - center[cells]
        dd2 = D[:, 0] * D[:, 0] + D[:, 1] * D[:, 1] + D[:, 2] * D[:, 2]
        with np.errstate(divide="ignore", invalid="ignore"):
            ad = (area[:, 0] * D[:, 0] + area[:, 1] * D[:, 1] + area[:, 2] * D[:, 2]) / dd2 * flag
        if np.any(~np.isfinite(ad) & (dd2 >= TINY)):
            raise ValueError("corner-point grid: effective area is not finite")
        hb.append(cells); he.append(others); hslot.append(np.full(cells.shape, slot)); hAd.append(ad)

    lateral = ((i > 0, -1, 0), (i < nx - 1, 1, 0), (j > 0, -nx, 1), (j < ny - 1, nx, 1))
    for dd, (cond, step, axis) in enumerate(lateral):
        fidx, oidx = np.array(FACE[dd]), np.array(OTHER[dd])

        def probe(cells, dk, slot):
            """SetAllFlags for the faces of `cells` against the cells dk
            layers away across the face; emits the overlapping ones."""
            others = cells + step + dk * nxny
            F = P[cells[:, None], fidx]
            inter, jump, quad, up, down = _face_flags(P[others[:, None], oidx], F)
            keep = ~jump
            area = _area_vector(*(inter[keep, q] for q in range(4)))
            nq = ~quad[keep]
            if nq.any():
                Fk = F[keep][nq]
                area[nq] = _projected_area(Fk, P[others[keep][nq][:, None], oidx],
                                           _area_vector(*(Fk[:, q] for q in range(4))), axis)
            emit(cells[keep], others[keep], dd * span + slot, area, F[keep])
            return up, down

        act = idx[cond]
        up, act_down = probe(act, 0, 0)
        # upward while the last probe says so; the downward search then starts
        # from the flags of the last probe, upward or not, as in the reference
        go, dk = up, -1
        while go.any():
            pos = np.nonzero(go)[0]
            pos = pos[k[act[pos]] + dk >= 0]
            if not pos.size:
                break
            u, dn = probe(act[pos], dk, -dk)
            act_down[pos] = dn
            go = np.zeros_like(go)
            go[pos] = u
            dk -= 1
        go, dk = act_down, 1
        while go.any():
            pos = np.nonzero(go)[0]
            pos = pos[k[act[pos]] + dk <= nz - 1]
            if not pos.size:
                break
            _, dn = probe(act[pos], dk, nz + dk)
            go = np.zeros_like(go)
            go[pos] = dn
            dk += 1
    for dd, cond, step in ((4, k > 0, -nxny), (5, k < nz - 1, nxny)):
        cells = idx[cond]
        F = P[cells[:, None], np.array(FACE[dd])]
        emit(cells, cells + step, dd * span, _area_vector(*(F[:, q] for q in range(4))), F)
    hb, he, hslot, Ad = (np.concatenate(a) for a in (hb, he, hslot, hAd))
    # pair each half connection with the first of the other cell's toward
    # this one; keep pairs with both halves positive (:1120-1150) and eId > bId
    order = np.argsort(hb.astype(np.int64) * (6 * span) + hslot, kind="stable")
    hb, he, hslot, Ad = hb[order], he[order], hslot[order], Ad[order]
    key = hb.astype(np.int64) * n + he
    ukey, first = np.unique(key, return_index=True)
    rev = he.astype(np.int64) * n + hb
    pos = np.minimum(np.searchsorted(ukey, rev), ukey.size - 1)
    found = ukey[pos] == rev
    partner = first[pos]
    keep = found & (he > hb) & ~(Ad <= 0) & ~(Ad[partner] <= 0)
    b, e, aB, aE = hb[keep], he[keep], Ad[keep], Ad[partner][keep]
    direction = hslot[keep] // span
    axis = np.array([0, 0, 1, 1, 2, 2])[direction]
    perm = np.stack([kx, ky, kz])
    T1 = np.where(axis < 2, ntg[b], 1.0) * perm[axis, b] * aB
    T2 = np.where(axis < 2, ntg[e], 1.0) * perm[axis, e] * aE
    mult = np.ones(b.size) if multz is None else np.where(direction == 5, f(multz)[b], 1.0)
    trans = _trans(mult, T1, T2, conv_darcy)
    # dx, dy, dz: between the centres of opposite faces, each taken from the
    # cell centre as the reference forms them (src/CornerGrid.cpp:1085-1094)
    half = [0.25 * (P[:, a] + P[:, b_] + P[:, c_] + P[:, d_]) - center for (a, b_, c_, d_) in FACE]
    size = []
    for lo, hi in ((0, 1), (2, 3), (4, 5)):
        dp = half[hi] - half[lo]
        size.append(np.sqrt(dp[:, 0] * dp[:, 0] + dp[:, 1] * dp[:, 1] + dp[:, 2] * dp[:, 2]))
    act = active_cells(v, poro, actnum)
    grid, geo = _compress(n, act, b, e, trans, v, depth, poro,
                          dict(dx=size[0], dy=size[1], dz=size[2], ntg=ntg, kx=kx, ky=ky, kz=kz))
    if return_geometry:
        k = geo.pop("conn_keep")
        geo.update(areaB=aB[k], areaE=aE[k], axis=axis[k], center=center[act], corners=P[act])
        return grid, geo
    return grid
