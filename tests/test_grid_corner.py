"""Corner-point grid ingest (opencaeporox_gb300.grid.corner_point_grid)
against the reference's own ingest (OCP_COORD::SetupCornerPoints and the
transmissibility of BulkConnTransMethod01::CalTrans), dumped by the harness
(tests/golden/gen_fixtures.py) for a 6 x 5 x 4 grid with dipping layers and
leaning pillars (cpg_6x5x4.npz) and for an 8 x 6 x 5 grid of the same kind
cut by three faults (cpg_fault_8x6x5.npz: scissor faults whose throw changes
sign, thickness changes across them, a throw of two layers).  The overlap
area of non-quadrilateral fault faces is checked against the reference's
CalAreaNotQuadr on 1,536 seeded face pairs covering its twelve cases
(overlap_area.npz), and the oracle's Newton iteration on the faulted grid,
fed by this ingest, against the reference's (fault_comp3_8x6x5.npz)."""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import grid, synthetic


def _ingest(fx, **kw):
    nx, ny, nz = (int(v) for v in fx["input/dims"])
    return grid.corner_point_grid(nx, ny, nz, fx["input/coord"], fx["input/zcorn"], fx["input/kx"], fx["input/ky"],
                                  fx["input/kz"], fx["input/poro"],
                                  conv_darcy=float(fx["model/CONV_DARCY"].ravel()[0]), **kw)


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_against_reference_dump():
    fx = P.load_fixture("cpg_6x5x4")
    g, geo = _ingest(fx, return_geometry=True)
    # connections: the same pairs in the same order
    assert np.array_equal(g.conn_b, fx["model/conn_bId"]) and np.array_equal(g.conn_e, fx["model/conn_eId"])
    # depth is the mean of the corner depths, as the reference forms it
    assert np.array_equal(g.depth, fx["model/depth"])
    # half areas and transmissibilities bit for bit; the volume to rounding
    # (exact Gauss quadrature rather than the expanded polynomial the
    # reference evaluates in absolute coordinates)
    assert np.array_equal(geo["areaB"], fx["model/conn_areaB"])
    assert np.array_equal(geo["areaE"], fx["model/conn_areaE"])
    assert np.array_equal(g.conn_trans, fx["model/conn_trans"])
    assert _rel(g.v, fx["model/v"]) < 1e-13
    # the grid is genuinely corner-point: leaning pillars, non-box cells
    assert np.ptp(fx["model/v"]) > 1e-3 * np.mean(fx["model/v"])


def test_flat_vertical_grid_is_the_orthogonal_grid():
    coord, zcorn = synthetic.dipping_corner_point(5, 4, 3, 20.0, 2.0, 2000.0, 0.0, 0.0, 0.0)
    a = grid.corner_point_grid(5, 4, 3, coord, zcorn, 100.0, 80.0, 10.0, 0.2)
    b = grid.orthogonal_grid(5, 4, 3, 20.0, 20.0, 2.0, 2000.0, 100.0, 80.0, 10.0, 0.2)
    assert np.array_equal(a.conn_b, b.conn_b) and np.array_equal(a.conn_e, b.conn_e)
    assert np.array_equal(a.conn_trans, b.conn_trans) and np.array_equal(a.depth, b.depth)
    assert _rel(a.v, b.v) < 1e-13


def test_faulted_grid_against_reference_dump():
    fx = P.load_fixture("cpg_fault_8x6x5")
    nx, ny, nz = (int(v) for v in fx["input/dims"])
    g, geo = _ingest(fx, return_geometry=True)
    assert np.array_equal(g.conn_b, fx["model/conn_bId"]) and np.array_equal(g.conn_e, fx["model/conn_eId"])
    assert np.array_equal(geo["areaB"], fx["model/conn_areaB"])
    assert np.array_equal(geo["areaE"], fx["model/conn_areaE"])
    assert np.array_equal(g.conn_trans, fx["model/conn_trans"])
    assert np.array_equal(g.depth, fx["model/depth"])
    assert _rel(g.v, fx["model/v"]) < 1e-13
    # the faults matter: NNCs (neighbours in another layer across x or y) and
    # more connections than the unfaulted grid has
    b, e = g.conn_b.astype(np.int64), g.conn_e.astype(np.int64)
    nnc = (e // (nx * ny) != b // (nx * ny)) & (e - b != nx * ny)
    assert nnc.sum() > 50
    assert g.conn_b.size > 3 * nx * ny * nz - nx * nz - ny * nz - nx * ny


def test_overlap_area_against_reference():
    fx = P.load_fixture("overlap_area")
    f, g = fx["pairs"][:, 0], fx["pairs"][:, 1]
    assert np.array_equal(grid._overlap_area(f, g), fx["area"])
    _, pattern = grid.overlap_pattern(f, g)
    assert {1, 2, 3, 4, 5, 8, 9, 10, 11, 12, 13, 15} <= set(pattern.tolist())


def test_zero_throw_fault_is_the_unfaulted_grid():
    nx, ny, nz = 5, 4, 3
    a = grid.corner_point_grid(nx, ny, nz, *synthetic.dipping_corner_point(nx, ny, nz, 20.0, 2.0, 2000.0, 3.0, 1.0,
                                                                           0.04, seed=3), 100.0, 80.0, 10.0, 0.2)
    coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, 20.0, 2.0, 2000.0, 3.0, 1.0, [("x", 2, 0.0, 0.0)], 0.04,
                                                  seed=3)
    b = grid.corner_point_grid(nx, ny, nz, coord, zcorn, 100.0, 80.0, 10.0, 0.2)
    assert np.array_equal(a.conn_b, b.conn_b) and np.array_equal(a.conn_e, b.conn_e)
    assert np.array_equal(a.conn_trans, b.conn_trans) and np.array_equal(a.v, b.v)


def test_throw_of_a_whole_layer_connects_across_layers():
    """A throw of exactly one layer thickness along an x fault: the cells
    beyond it meet the cells one layer down (NNCs), and nothing meets its
    own layer across the fault."""
    nx, ny, nz, dz = 4, 3, 3, 2.0
    coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, 20.0, dz, 2000.0, 0.0, 0.0, [("x", 1, dz, dz)])
    g = grid.corner_point_grid(nx, ny, nz, coord, zcorn, 100.0, 100.0, 10.0, 0.2)
    pairs = set(zip(g.conn_b.tolist(), g.conn_e.tolist()))
    cell = lambda i, j, k: (k * ny + j) * nx + i
    for j in range(ny):
        for k in range(nz):
            assert (cell(1, j, k), cell(2, j, k)) not in pairs
            if k + 1 < nz:
                assert (cell(2, j, k), cell(1, j, k + 1)) in pairs


def test_fault_newton_iteration_with_own_ingest():
    """The oracle's residual and Jacobian on the faulted grid, with the grid
    from this ingest (not from the reference's dump), match the reference's
    within 1e-10 per row."""
    from opencaeporox_gb300 import fim
    from oracle.pyoracle import OracleBulk
    fx = P.load_fixture("fault_comp3_8x6x5")
    model, dumped = fim.model_and_grid_from_dump(fx)
    own = _ingest(fx)
    assert np.array_equal(own.conn_b, dumped.conn_b) and np.array_equal(own.conn_e, dumped.conn_e)
    assert np.array_equal(own.conn_trans, dumped.conn_trans)
    g = fim.Grid(v=own.v, depth=own.depth, poro_init=dumped.poro_init, conn_b=own.conn_b, conn_e=own.conn_e,
                 conn_trans=own.conn_trans)
    bs = (model.nc + 1) ** 2
    for it in P.iterations(fx):
        js = P.jac_state(fx, it)
        ob = OracleBulk(model, g)
        ob.load(js)
        ob.cal_res(float(js["dt"][0]))
        rp, col, val = ob.assemble(float(js["dt"][0]))
        assert np.array_equal(rp, js["jac_rowptr"]) and np.array_equal(col, js["jac_col"])
        ref = js["jac_val"]
        e = max(np.linalg.norm(val[rp[r] * bs: rp[r + 1] * bs] - ref[rp[r] * bs: rp[r + 1] * bs]) /
                max(np.linalg.norm(ref[rp[r] * bs: rp[r + 1] * bs]), 1e-300) for r in range(g.nb))
        assert e <= P.REL_TOL, (it, e)
