"""The GRID-section deck reader (opencaeporox_gb300.deck) against the
reference's own reading and grid set-up: four decks made by
tests/golden/gen_fixtures.py (grid_deck_texts) were read by the reference,
whose harness dumped the grid it built (deck_*.npz).  Block-centred and
faulted corner-point grids, with inactive cells (ACTNUM, an EQUALS box of
ACTNUM, zero porosity) and NTG, or with NTG and MULTZ; arrays given as plain
values, m*v repeats, COPY / MULTIPLY / EQUALS boxes and an INCLUDE file.
Host only."""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import deck as D

DECKS = ["deck_ortho_actnum", "deck_ortho_multz", "deck_corner_actnum", "deck_corner_multz"]


def _read(fx, tmp_path):
    (tmp_path / "grid.data").write_text(str(fx["deck/main"]))
    (tmp_path / "grid_poro.inc").write_text(str(fx["deck/include"]))
    return D.read_grid_deck(str(tmp_path / "grid.data"))


@pytest.mark.parametrize("name", DECKS)
def test_grid_from_deck_against_reference(name, tmp_path):
    fx = P.load_fixture(name)
    deck = _read(fx, tmp_path)
    g, geo = D.grid_from_deck(deck, float(fx["model/CONV_DARCY"].ravel()[0]))
    m = lambda k: fx["model/" + k]
    assert g.nb == int(m("nb").ravel()[0])
    assert np.array_equal(g.conn_b, m("conn_bId")) and np.array_equal(g.conn_e, m("conn_eId"))
    assert np.array_equal(g.conn_trans, m("conn_trans"))
    assert np.array_equal(g.depth, m("depth")) and np.array_equal(g.poro_init, m("poroInit"))
    for k, mk in (("dx", "dx"), ("dy", "dy"), ("dz", "dz"), ("ntg", "ntg"), ("kx", "rockKx"), ("ky", "rockKy"),
                  ("kz", "rockKz")):
        assert np.array_equal(geo[k], m(mk)), k
    if deck.corner:
        # Gauss quadrature against the reference's expanded polynomial
        assert np.max(np.abs(g.v - m("v")) / m("v")) < 1e-13
    else:
        assert np.array_equal(g.v, m("v"))
    if name.endswith("_actnum"):
        assert g.nb < deck.n


def test_inactive_x_neighbour_ends_the_cells_connections(tmp_path):
    """A cell whose +x neighbour is inactive gets no +y or +z connection
    either (the reference's loop leaves the cell at the first inactive
    neighbour), and the reference's own grid agrees (previous test)."""
    fx = P.load_fixture("deck_ortho_actnum")
    deck = _read(fx, tmp_path)
    g, geo = D.grid_from_deck(deck)
    nx, ny, n = deck.nx, deck.ny, deck.n
    a2 = np.full(n, -1)
    a2[geo["act2all"]] = np.arange(g.nb)
    pairs = set(zip(g.conn_b.tolist(), g.conn_e.tolist()))
    seen = 0
    for c in geo["act2all"]:
        i, j = c % nx, (c // nx) % ny
        if i < nx - 1 and a2[c + 1] < 0 and j < ny - 1 and a2[c + nx] >= 0:
            assert (a2[c], a2[c + nx]) not in pairs
            seen += 1
    assert seen >= 1


def _write(tmp_path, text, name="d.data"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reader_syntax(tmp_path):
    text = """-- a comment
# another
DIMENS
2 2 2 /
DX 99 99
8*10.0
/
DY
4*5.0 4*6.0 /
DZ
1, 2, 3, 4 -- trailing words are not values
/
-- the data above stops at the first '/', the rest of the line is dropped
TOPS
'100' 100 101 101
/
PORO
8*0.25
/
EQUALS
PORO 0.1 1 1 1 1 1 2 /
TOPS 50 2 2 2* 2 2 /
/
MULTIPLY
DX 2 1 1 6* /
/
SOMEKEY
1 2 3 /
/
"""
    with pytest.raises(ValueError):
        # "--" is not a value: the reference stops on it too
        D.read_grid_deck(_write(tmp_path, text))
    text = text.replace(" -- trailing words are not values", " /")
    d = D.read_grid_deck(_write(tmp_path, text))
    A = d.arrays
    assert (d.nx, d.ny, d.nz) == (2, 2, 2)
    # MULTIPLY DX 2 over i = 1 (all j, k): cells with i == 0 doubled
    assert np.array_equal(A["DX"], np.where(np.arange(8) % 2 == 0, 20.0, 10.0))
    assert np.array_equal(A["DY"], np.r_[[5.0] * 4, [6.0] * 4])
    assert np.array_equal(A["DZ"], [1.0, 2.0, 3.0, 4.0])
    # TOPS: the EQUALS box (i = 2, every j, k = 2) is cut to the top layer
    assert np.array_equal(A["TOPS"], [100.0, 50.0, 101.0, 50.0])
    # EQUALS PORO over i = 1, j = 1, k = 1..2
    assert np.array_equal(A["PORO"], np.where(np.arange(8) % 4 == 0, 0.1, 0.25))


def test_include_copy_and_errors(tmp_path):
    (tmp_path / "perm.inc").write_text("PERMX\n4*100 4*200\n/\n")
    main = _write(tmp_path, """DIMENS
2 2 2 /
INCLUDE
'perm.inc' /
COPY
PERMX PERMY 6* /
PERMX PERMZ 1 1 1 2 1 2 /
/
""")
    d = D.read_grid_deck(main)
    A = d.arrays
    assert np.array_equal(A["PERMY"], A["PERMX"])
    assert np.array_equal(A["PERMZ"], np.where(np.arange(8) % 2 == 0, A["PERMX"], 0.0))
    with pytest.raises(ValueError, match="not given"):
        D.read_grid_deck(_write(tmp_path, "DIMENS\n2 2 2 /\nMULTIPLY\nPORO 2 6* /\n/\n", "m.data"))
    with pytest.raises(ValueError, match="PORO"):
        D.grid_from_deck(d)
    # a '/' ends the line, in the reference's reader as in this one
    with pytest.raises(ValueError, match="INCLUDE"):
        D.read_grid_deck(_write(tmp_path, "DIMENS\n2 2 2 /\nINCLUDE\n'sub/perm.inc' /\n", "i.data"))


def test_ntg_and_actnum_of_the_wrong_length_are_dropped(tmp_path):
    base = """DIMENS
2 1 1 /
DX
2*10 /
DY
2*10 /
DZ
2*2 /
TOPS
2*1000 /
PORO
2*0.2 /
PERMX
2*100 /
PERMY
2*100 /
PERMZ
2*10 /
"""
    g0, _ = D.grid_from_deck(D.read_grid_deck(_write(tmp_path, base, "a.data")))
    g1, geo = D.grid_from_deck(D.read_grid_deck(_write(tmp_path, base + "NTG\n3*0.5 /\nACTNUM\n0 /\n", "b.data")))
    assert g1.nb == 2 and np.array_equal(g1.poro_init, g0.poro_init) and np.array_equal(geo["ntg"], [1.0, 1.0])
    assert np.array_equal(g1.conn_trans, g0.conn_trans)
    g2, _ = D.grid_from_deck(D.read_grid_deck(_write(tmp_path, base + "NTG\n0.5 1 /\nACTNUM\n1 0 /\n", "c.data")))
    assert g2.nb == 1 and g2.poro_init[0] == 0.2 * 0.5 and g2.conn_b.size == 0


def test_grid_corpus_against_reference(tmp_path):
    """Forty seeded small grids (tests/golden/gen_fixtures.py corpus_case):
    twenty corner-point grids cut by random faults (throws up to two layers,
    scissor faults, thickness changes, leaning pillars) and twenty
    block-centred grids with per-cell sizes; random inactive cells, NTG and
    MULTZ.  Each GRID section was read by the reference itself; the deck
    reader's grid equals the reference's in every case."""
    fx = P.load_fixture("grid_corpus")
    cases = sorted({k.split("/")[0] for k in fx})
    assert len(cases) == 40
    for c in cases:
        m = P.group(fx, c)
        assert "refused" not in m, c
        path = tmp_path / f"{c}.data"
        path.write_text(str(m["grid"]))
        deck = D.read_grid_deck(str(path))
        g, geo = D.grid_from_deck(deck, float(m["CONV_DARCY"].ravel()[0]))
        assert g.nb == int(m["nb"].ravel()[0]), c
        assert np.array_equal(g.conn_b, m["conn_bId"]) and np.array_equal(g.conn_e, m["conn_eId"]), c
        assert np.array_equal(g.conn_trans, m["conn_trans"]), c
        assert np.array_equal(g.depth, m["depth"]) and np.array_equal(g.poro_init, m["poroInit"]), c
        for k, mk in (("dx", "dx"), ("dy", "dy"), ("dz", "dz"), ("ntg", "ntg"), ("kx", "rockKx"), ("ky", "rockKy"),
                      ("kz", "rockKz")):
            assert np.array_equal(geo[k], m[mk]), (c, k)
        if deck.corner:
            assert np.array_equal(geo["areaB"], m["conn_areaB"]) and np.array_equal(geo["areaE"], m["conn_areaE"]), c
            assert np.max(np.abs(g.v - m["v"]) / m["v"]) < 1e-13, c
        else:
            assert np.array_equal(g.v, m["v"]), c


def test_well_perforations_against_reference(tmp_path):
    """WELSPECS/COMPDAT on the faulted grid with inactive cells, read by the
    reference (deck_wells.npz): the perforations it keeps (one in an inactive
    cell is dropped), their cells, well indices, kh, radius, skin and
    direction, bit for bit.  The records cover x, y and z perforations, a
    given kh, a skin, a given WI and a well name given by its prefix."""
    fx = P.load_fixture("deck_wells")
    w, m = P.group(fx, "wells"), P.group(fx, "model")
    deck = _read(fx, tmp_path)
    wells = D.read_wells(str(tmp_path / "grid.data"))
    g, geo = D.grid_from_deck(deck, float(m["CONV_DARCY"].ravel()[0]))
    perfs = D.well_perforations(wells, deck, g, geo, float(m["CONV_DARCY"].ravel()[0]), float(m["CONV1"].ravel()[0]))
    assert [p["name"] for p in perfs] == ["INJE1", "PROD1"]
    assert [p["cell"].size for p in perfs] == list(np.asarray(w["well_nperf"]).ravel())
    cat = lambda k: np.concatenate([p[k] for p in perfs])
    for k, rk in (("cell", "perf_loc"), ("WI", "perf_WI"), ("kh", "perf_kh"), ("radius", "perf_radius"),
                  ("skin", "perf_skin"), ("direction", "perf_dir")):
        assert np.array_equal(cat(k), np.asarray(w[rk]).ravel()), k
    assert sum(len(x.perfs) for x in wells) == int(np.sum(w["well_nperf"])) + 1


def test_read_wells_records(tmp_path):
    text = """WELSPECS
'A1' 'G' 2 3 1* 'OIL' /
'A2' 'G' 1 1 1* 'OIL' /
'B1' 'G' 4 4 1* 'GAS' /
/
COMPDAT
'A*' 2* 1 2 1* 0.5 3* /
'B1' 3 3 2 2 7.5 0.2 100 2.0 'x' /
/
"""
    wells = D.read_wells(_write(tmp_path, text))
    a1, a2, b1 = wells
    assert [p[:3] for p in a1.perfs] == [(2, 3, 1), (2, 3, 2)]
    assert [p[:3] for p in a2.perfs] == [(1, 1, 1), (1, 1, 2)]
    assert a1.perfs[0][3:] == (-1.0, 0.5, -1.0, 0.0, 2)
    assert b1.perfs == [(3, 3, 2, 7.5, 0.2, 100.0, 2.0, 0)]
    with pytest.raises(ValueError, match="direction"):
        D.read_wells(_write(tmp_path, "WELSPECS\n'C' 'G' 1 1 1* 'OIL' /\n/\nCOMPDAT\n'C' 2* 1 1 1* 0.2 2* 'q' /\n/\n",
                            "bad.data"))


def _decks_module():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks.py")
    spec = importlib.util.spec_from_file_location("golden_decks", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# the decks the FIM fixtures were made from (tests/golden/gen_fixtures.py)
FIXTURE_DECKS = {
    "comp6_8x8x3": lambda d: d.comp_deck(8, 8, 3, 6, seed=2, tsteps=(0.02, 0.05, 0.1), smooth=True)[1],
    "comp8_6x6x4": lambda d: d.comp_deck(6, 6, 4, 8, seed=4, tsteps=(0.02, 0.05, 0.1), smooth=True)[1],
    "bo_10x10x3": lambda d: d.blackoil_deck(seed=1),
}


def _model_equal(model, ref):
    for k, v in model.arrays.items():
        assert k in ref, k
        a, b = np.asarray(v, float).ravel(), np.asarray(ref[k], float).ravel()
        assert a.shape == b.shape and np.array_equal(a, b), k


@pytest.mark.parametrize("name", sorted(FIXTURE_DECKS))
def test_model_from_deck_against_reference(name, tmp_path):
    """The device's Model read from a deck equals the reference's model dump
    of the same deck, every array bit for bit."""
    text = FIXTURE_DECKS[name](_decks_module())
    model = D.read_model(_write(tmp_path, text))
    _model_equal(model, P.group(P.load_fixture(name), "model"))


def test_model_variants_against_reference(tmp_path):
    """FIELD units, GRAVITY, VCRIT, OMEGAA / OMEGAB, SSHIFT, VCRITVIS, LBCCOEF
    with defaults, a full BIC matrix, LINEAR02 rock and a black-oil deck with
    GRAVITY (props_variants.npz, read by the reference)."""
    fx = P.load_fixture("props_variants")
    names = sorted({k.split("/")[0] for k in fx})
    assert names == ["bo_field_gravity", "comp_field_gravity", "comp_fullbic"]
    for name in names:
        ref = P.group(fx, name)
        _model_equal(D.read_model(_write(tmp_path, str(ref["deck"]), name + ".data")), ref)


def test_deck_drives_the_reference_algorithm(tmp_path):
    """Grid and Model read from the deck of comp6_8x8x3, with the reference's
    states of its Newton iterations: the oracle's residual and Jacobian equal
    the reference's (rows within 1e-10), so a deck reaches the device path
    without the reference."""
    from oracle.pyoracle import OracleBulk
    path = _write(tmp_path, FIXTURE_DECKS["comp6_8x8x3"](_decks_module()))
    model = D.read_model(path)
    grid, _ = D.grid_from_deck(D.read_grid_deck(path), float(model.arrays["CONV_DARCY"][0]))
    fx = P.load_fixture("comp6_8x8x3")
    ref = P.group(fx, "model")
    assert np.array_equal(grid.conn_trans, ref["conn_trans"]) and np.array_equal(grid.v, ref["v"])
    bs = (model.nc + 1) ** 2
    for it in P.iterations(fx):
        js = P.jac_state(fx, it)
        ob = OracleBulk(model, grid)
        ob.load(js)
        ob.cal_res(float(js["dt"][0]))
        assert P.res_err(ob.res, js["res_bulk"], js["rockVp"], js["Nt"], model.nc) <= P.REL_TOL
        rp, col, val = ob.assemble(float(js["dt"][0]))
        assert np.array_equal(rp, js["jac_rowptr"]) and np.array_equal(col, js["jac_col"])
        v, r = val, js["jac_val"]
        e = max(np.linalg.norm(v[rp[i] * bs:rp[i + 1] * bs] - r[rp[i] * bs:rp[i + 1] * bs]) /
                max(np.linalg.norm(r[rp[i] * bs:rp[i + 1] * bs]), 1e-300) for i in range(grid.nb))
        assert e <= P.REL_TOL, (it, e)


def test_props_errors(tmp_path):
    with pytest.raises(ValueError, match="SWOF"):
        D.read_model(_write(tmp_path, "METRIC\nCOMPS\n2 /\n", "e1.data"))
    with pytest.raises(ValueError, match="regions"):
        D.read_props(_write(tmp_path, "SWOF\n0.2 0 1 0 /\n0.3 0.1 0.8 0 /\n/\n", "e2.data"))
    with pytest.raises(ValueError, match="linear"):
        D.read_props(_write(tmp_path, "ROCK\nEXPONENT 200 1e-5 /\n/\n", "e3.data"))


def test_box_out_of_range_is_refused(tmp_path):
    with pytest.raises(ValueError, match="out of range"):
        D.read_grid_deck(_write(tmp_path, "DIMENS\n2 2 2 /\nEQUALS\nPORO 0.1 1 3 1 1 1 1 /\n/\n", "r.data"))
    d = D.read_grid_deck(_write(tmp_path, "DIMENS\n2 1 1 /\nACTNUM\n1.0 0 /\n", "a.data"))
    assert np.array_equal(d.arrays["ACTNUM"], [1, 0])


def test_initial_state_against_reference(tmp_path):
    """A PTN start with every array in the deck (PRESSURE, TEMPER, PHASEP,
    COMPM-0..3) on a grid with inactive cells (deck_ptn.npz): pressure,
    temperature and moles of the active cells equal the reference's initial
    state.  (The reference's initial flash and CalKrPc then set Pj from the
    capillary pressures, as the device's property update does, so the
    dumped Pj is not the deck's.)"""
    fx = P.load_fixture("deck_ptn")
    deck = _read(fx, tmp_path)
    props = D.read_props(str(tmp_path / "grid.data"))
    model = D.model_from_props(props)
    grid, geo = D.grid_from_deck(deck, float(model.arrays["CONV_DARCY"][0]))
    assert grid.nb == int(fx["model/nb"].ravel()[0]) < deck.n
    st = D.initial_state(deck, geo, model, props["rtemp"])
    for k in ("P", "T", "Ni"):
        assert np.array_equal(st[k], np.asarray(fx["init/" + k]).ravel()), k
    assert np.array_equal(st["Pj"].reshape(-1, 3)[:, 1], np.asarray(deck.arrays["PHASEP-1"])[geo["act2all"]])
    assert not st["phaseExist"].any()


def test_ptn1_arrays_list_the_active_cells(tmp_path):
    """With INITPTN1 the PTN arrays give the active cells only, in order
    (InitialReservoir::PostProcess); with INITPTN0 every cell."""
    base = """DIMENS
3 1 1 /
DX
3*10 /
DY
3*10 /
DZ
3*2 /
TOPS
3*1000 /
PORO
0.2 0.2 0.2 /
PERMX
3*100 /
PERMY
3*100 /
PERMZ
3*10 /
ACTNUM
1 0 1 /
"""
    from opencaeporox_gb300 import synthetic
    model = synthetic.comp_model(2, 3)          # three components with water
    ptn1 = base + "INITPTN1\nPRESSURE\n100 300 /\nPHASEP-0\n100 300 /\nPHASEP-1\n100 300 /\nPHASEP-2\n100 300 /\n" \
                  "COMPM-0\n1 2 /\nCOMPM-1\n3 4 /\nCOMPM-2\n5 6 /\n"
    deck = D.read_grid_deck(_write(tmp_path, ptn1, "p1.data"))
    grid, geo = D.grid_from_deck(deck)
    st = D.initial_state(deck, geo, model, rtemp=70.0)
    assert grid.nb == 2 and np.array_equal(st["P"], [100.0, 300.0]) and np.array_equal(st["T"], [70.0, 70.0])
    assert np.array_equal(st["Ni"], [1.0, 3.0, 5.0, 2.0, 4.0, 6.0])
    ptn0 = ptn1.replace("INITPTN1", "INITPTN0").replace("100 300 /", "100 200 300 /").replace(
        "1 2 /", "1 9 2 /").replace("3 4 /", "3 9 4 /").replace("5 6 /", "5 9 6 /")
    deck0 = D.read_grid_deck(_write(tmp_path, ptn0, "p0.data"))
    st0 = D.initial_state(deck0, D.grid_from_deck(deck0)[1], model, rtemp=70.0)
    for k in ("P", "T", "Ni", "Pj"):
        assert np.array_equal(st0[k], st[k]), k
