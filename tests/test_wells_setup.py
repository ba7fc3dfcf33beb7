"""The host-side well set-up: the vectorised Peaceman well index of
opencaeporox_gb300.wells against the oracle's restatement of
PeacemanWell::CalWI (src/WellPeaceman.cpp:277-361), and the layout of the
synthetic vertical wells."""
import numpy as np
import pytest

from opencaeporox_gb300 import wells as W
from oracle import wells as OW


@pytest.mark.parametrize("direction", [0, 1, 2])
def test_peaceman_wi_matches_the_reference_formula(direction):
    rng = np.random.default_rng(31 + direction)
    n = 64
    dx, dy, dz = (rng.uniform(2.0, 40.0, n) for _ in range(3))
    kx, ky, kz = (10 ** rng.uniform(-1.0, 3.0, n) for _ in range(3))
    ntg = rng.uniform(0.5, 1.0, n)
    radius, skin = 0.1, 0.5
    got = W.peaceman_wi(direction, dx, dy, dz, kx, ky, kz, ntg, radius, skin)
    ref = np.array([OW.well_index(direction, dx[i], dy[i], dz[i], ntg[i], kx[i], ky[i], kz[i],
                                  radius, skin, 0.008527)[0] for i in range(n)])
    np.testing.assert_array_equal(got, ref)


def test_peaceman_wi_rejects_an_unknown_direction():
    with pytest.raises(ValueError):
        W.peaceman_wi(3, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0)


def test_vertical_wells_layout():
    nx, ny, nz, ncomp = 6, 5, 4, 3
    nb = nx * ny * nz
    rng = np.random.default_rng(5)
    k = rng.uniform(10.0, 200.0, nb)
    depth = np.repeat(1000.0 + 5.0 * np.arange(nz), nx * ny)
    wells = W.vertical_wells(nx, ny, nz, 2, 3, 20.0, 5.0, k, 0.1 * k, depth, ncomp, 9, n_rate=1, corners=True)
    assert len(wells) == 5
    assert [w["type"] for w in wells] == [0, 0, 1, 1, 1]
    assert [w["mode"] for w in wells] == [0, 0, 0, 0, 1]
    cols = set()
    for w in wells:
        cells = np.asarray(w["cell"])
        assert cells.size == nz
        col = int(cells[0])
        assert np.array_equal(cells, col + nx * ny * np.arange(nz))
        cols.add(col)
        wi = W.peaceman_wi(2, 20.0, 20.0, 5.0, k[cells], k[cells], 0.1 * k[cells])
        np.testing.assert_array_equal(np.asarray(w["WI"]), wi)
        assert w["dG"][0] == 0.0 and np.all(np.diff(w["dG"]) > 0)
    assert len(cols) == 5
    assert int(np.asarray(wells[0]["cell"])[0]) == 0
    assert int(np.asarray(wells[2]["cell"])[0]) == nx * ny - 1
