"""The per-cell flash check of the bench's parity object (bench.recheck_cells)
on the host: a result the reference algorithm itself reaches when its
transcendentals round differently is explained; a planted error is not.

The GPU's flash differs from the oracle's where CUDA's transcendentals round
differently from glibc's; the parity object bounds each cell's error by four
times the oracle's own sensitivity to such roundings (seeded one- and two-ulp
perturbations of every exp, log, pow, acos and cos).  Here the "GPU" result
is another perturbed oracle run, so every cell must be explained, and the
same result with a relative error of 1e-8 planted (in the checked copy, on
the host) must not be."""
import numpy as np

import bench
import parity as P
from opencaeporox_gb300 import fim
from oracle.pyoracle import OracleBulk


def _cells(name, it_index=0):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    its = [it for it in P.iterations(fx) if "P" in P.group(fx, it + "/post")]
    state = dict(P.jac_state(fx, its[it_index]))
    state.update(P.group(fx, its[it_index] + "/pre"))
    return model, grid, state


def test_recheck_explains_a_perturbed_run_and_flags_a_planted_error():
    model, grid, state = _cells("comp8_6x6x4")
    ob = OracleBulk(model, grid, variant="ulp")
    ob.set_nudge_seed(1234, 2)
    ob.load(state)
    ob.update_property()
    nb = grid.nb
    got = {k: ob.a[v].reshape(nb, -1).copy() for k, v in bench.FLASH_KEYS.items()}
    inputs = {k: np.asarray(v).ravel() for k, v in state.items() if np.asarray(v).size % nb == 0}
    geometry = (grid.v, grid.depth, grid.poro_init)
    nudges = bench.RECHECK[:8] + bench.RECHECK[40:48]
    assert bench.recheck_cells(model, geometry, inputs, got, nudges=nudges) == 0
    planted = {k: v * (1 + 1e-8) for k, v in got.items()}
    assert bench.recheck_cells(model, geometry, inputs, planted, nudges=nudges) > nb // 2
