"""The synthetic workload builders reproduce the reference's own setup
(model arrays and grid) bit for bit, checked against the reference dumps in
the golden fixtures."""
import numpy as np

import parity as P
from opencaeporox_gb300 import synthetic
from opencaeporox_gb300.grid import orthogonal_grid

MODEL_KEYS = ["Tc", "Pc", "MWC", "acf", "Vc", "Vcvis", "OmegaA", "OmegaB", "Vshift", "BIC", "LBCcoef", "flash_ctrl",
              "PVTW", "stdRhoW", "stdVw", "SWOF", "SGOF", "rock_Pref", "rock_cp1", "rock_cp2", "GRAVITY_FACTOR",
              "CONV_DARCY", "GAS_CONSTANT", "CONV1", "CONV3", "CONV4", "skipPSA", "nc"]


def test_comp_model_matches_reference_setup():
    for name, ncomp, seed in (("comp6_8x8x3", 6, 2), ("comp8_6x6x4", 8, 4)):
        ref = P.group(P.load_fixture(name), "model")
        m = synthetic.comp_model(ncomp, seed).arrays
        for k in MODEL_KEYS:
            assert np.array_equal(np.asarray(m[k], float).ravel(), np.asarray(ref[k], float).ravel()), (name, k)


def test_grid_matches_reference_connections():
    for name, dims in (("bo_10x10x3", (10, 10, 3)), ("comp6_8x8x3", (8, 8, 3))):
        m = P.group(P.load_fixture(name), "model")
        g = orthogonal_grid(*dims, m["dx"], m["dy"], m["dz"], 2000.0, m["rockKx"], m["rockKy"], m["rockKz"],
                            m["poroInit"], ntg=m["ntg"], conv_darcy=float(m["CONV_DARCY"][0]))
        assert np.array_equal(g.conn_b, m["conn_bId"]) and np.array_equal(g.conn_e, m["conn_eId"])
        assert np.array_equal(g.conn_trans, m["conn_trans"])
        assert np.array_equal(g.depth, m["depth"]) and np.array_equal(g.v, m["v"])
