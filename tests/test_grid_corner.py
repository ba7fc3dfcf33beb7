"""Corner-point grid ingest (opencaeporox_gb300.grid.corner_point_grid)
against the reference's own ingest (OCP_COORD::SetupCornerPoints and the
transmissibility of BulkConnTransMethod01::CalTrans), dumped by the harness
for a 6 x 5 x 4 grid with dipping layers and leaning pillars
(tests/golden/cpg_6x5x4.npz, made by tests/golden/gen_fixtures.py)."""
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
    # geometry and transmissibilities: rounding only (areas from the face
    # diagonals, volume by exact Gauss quadrature rather than the expanded
    # polynomial the reference evaluates in absolute coordinates)
    assert _rel(geo["areaB"], fx["model/conn_areaB"]) < 1e-14
    assert _rel(geo["areaE"], fx["model/conn_areaE"]) < 1e-14
    assert _rel(g.conn_trans, fx["model/conn_trans"]) < 1e-14
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


def test_faulted_grid_is_rejected():
    nx, ny, nz = 4, 3, 2
    coord, zcorn = synthetic.dipping_corner_point(nx, ny, nz, 20.0, 2.0, 2000.0, 0.0, 0.0, 0.0)
    z = zcorn.reshape(nz, 2, ny, 2, nx, 2).copy()
    z[:, :, :, :, 2:, :] += 1.0          # a throw between columns 1 and 2
    with pytest.raises(ValueError, match="faults"):
        grid.corner_point_grid(nx, ny, nz, coord, z.ravel(), 100.0, 100.0, 10.0, 0.2)
