"""Per cell, the GPU's compositional flash against the reference: every flash
output within 1e-10, or, for the cells that are not, within four times that
cell's own libm sensitivity.

The reference's results depend on how its C library rounds exp, log, pow,
acos and cos; CUDA's functions round differently (up to about 2 ulp per call).
For each cell above 1e-10 the oracle (which reproduces the reference bit for
bit on these fixtures) is rerun on that cell alone with every transcendental
moved by one or two ulp under 86 seeded patterns (bench.NUDGES and
bench.RECHECK); the cell passes when the GPU's error is at most four times the
largest deviation those runs show.  The cells above 1e-10 are printed (run
with -s to see them): they are the explicit list of where 1e-10 is not met.
"""
import numpy as np
import pytest

import bench
import parity as P
from opencaeporox_gb300 import fim

pytestmark = pytest.mark.gpu


def _per_cell(state):
    return {k: np.asarray(v) for k, v in state.items() if k in fim.REF_NAMES}


def _check(model, grid, state, got, ref, label):
    nb, nc = grid.nb, model.nc
    g = {k: np.asarray(got[k], np.float64).reshape(nb, -1) for k in bench.FLASH_KEYS}
    r = {k: np.asarray(ref[v], np.float64).reshape(nb, -1) for k, v in bench.FLASH_KEYS.items()}
    pe = np.asarray(ref["phaseExist"]).reshape(nb, 3).astype(bool)
    e = bench.cell_errors(g, r, pe, nc)
    above = np.nonzero(e > P.REL_TOL)[0]
    print(f"CELLS {label}: {above.size} of {nb} above 1e-10: "
          + ", ".join(f"{c} ({e[c]:.2e})" for c in above))
    if not above.size:
        return
    rows = {k: v.reshape(nb, -1)[above].ravel() for k, v in _per_cell(state).items() if v.size % nb == 0}
    unexplained = bench.recheck_cells(model, (np.asarray(grid.v)[above], np.asarray(grid.depth)[above],
                                              np.asarray(grid.poro_init)[above]),
                                      rows, {k: v[above] for k, v in g.items()},
                                      nudges=bench.NUDGES + bench.RECHECK)
    assert unexplained == 0, f"{label}: {unexplained} cells above four times their libm sensitivity"


@pytest.mark.parametrize("name", ["comp6_8x8x3", "comp8_6x6x4"])
def test_fixture_flash_cells(gpu_lib, name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    with fim.FimContext(model, grid) as ctx:
        for it in P.iterations(fx):
            post = P.group(fx, it + "/post")
            if "P" not in post:
                continue
            state = dict(P.jac_state(fx, it))
            state.update(P.group(fx, it + "/pre"))
            ctx.load_state(P.jac_state(fx, it))
            ctx.load_state(P.group(fx, it + "/pre"))
            ctx.update_property()
            got = {k: ctx.get(k) for k in bench.FLASH_KEYS}
            assert np.array_equal(ctx.get("PHASE_EXIST"), post["phaseExist"].astype(np.uint8))
            _check(model, grid, state, got, post, f"{name} {it}")


def test_flash10_cells(gpu_lib):
    fx = P.load_fixture("flash10")
    model, grid, state, ref = P.flash_case(fx)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(state)
        ctx.update_property()
        got = {k: ctx.get(k) for k in bench.FLASH_KEYS}
        assert np.array_equal(ctx.get("PHASE_EXIST"), ref["phaseExist"].astype(np.uint8))
    refd = {v: ref[v] for v in set(bench.FLASH_KEYS.values()) if v in ref}
    refd["phaseExist"] = ref["phaseExist"]
    _check(model, grid, state, got, refd, "flash10")
