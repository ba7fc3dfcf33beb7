"""Generates the golden fixtures in tests/golden/ by running the reference
simulator itself (its own C++ sources, compiled by oracle/ref/Makefile into
oracle/_ref/ocp_ref_dump) on seeded synthetic decks from decks.py.

Run in a container that holds the reference sources (they are not needed
afterwards; the fixtures are committed):

    python tests/golden/gen_fixtures.py [--only NAME]

Fixtures (compressed .npz, one key per dumped array, "<group>/<name>"):

* ``bo_10x10x3``   three-phase black-oil FIM, 300 cells, every Newton
  iteration of the first time steps (model, init, itNNN/{jac_state,pre,post}).
* ``comp6_8x8x3``  six-component PR-EoS FIM, 192 cells with per-cell random
  feeds and pressures (a slice of the 60x60x10 case), PTN start.
* ``comp8_6x6x4``  eight-component PR-EoS FIM, 144 cells.
* ``flash10``      ten-component flash-only cells: FlashDer from flash type 0
  without phase history, random and near-saturation feeds.
* ``wells_bo_10x10x3``, ``wells_comp6_8x8x3``  the same runs as the FIM
  fixtures above, with the wells' part of each iteration's residual: the
  perforations' data and fluxes and the residual with and without the wells.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import decks  # noqa: E402

REF_DIR = os.path.join(REPO, "oracle", "ref")
DUMP = os.path.join(REPO, "oracle", "_ref", "ocp_ref_dump")

# arrays kept per dump group (everything the GPU path reads or writes)
STATE_KEYS = ["P", "T", "Pb", "Ni", "Nt", "vf", "Pj", "Pc", "S", "phaseExist", "xij", "rho", "xi",
              "mu", "kr", "rhoP", "xiP", "muP", "rhox", "xix", "mux", "vfP", "vfi", "dKrdS",
              "dPcdS", "dSec_dPri", "poro", "poroP", "rockVp", "lNi",
              "skip_flag", "skip_minEigen", "skip_P", "skip_T", "skip_zi"]
RES_KEYS = ["upblock", "dP", "flux_vj", "flux_ni", "res_bulk", "resRelV", "resRelN", "maxRelRes_V",
            "maxRelRes_N", "maxId_V", "maxId_N"]


REFERENCE = os.environ.get("OCPX_REFERENCE_DIR", "/root/reference")


def build_reference():
    subprocess.run(["make", "-C", REF_DIR, "-j8", f"REF={REFERENCE}"], check=True, stdout=subprocess.DEVNULL)


def load_dir(path, keys=None):
    out = {}
    for f in sorted(os.listdir(path)):
        if not f.endswith(".npy"):
            continue
        k = f[:-4]
        if keys is None or k in keys:
            out[k] = np.load(os.path.join(path, f))
    return out


# Newton control after each iteration (the harness's finish_nr) and, on the
# last iteration of a time step, the time-step control (dump_finish_step)
NR_KEYS = ["nr_dPBmax", "nr_dPWmax", "nr_dTmax", "nr_dNmax", "nr_dSmax", "nr_eVmax", "nr_maxRelRes_V",
           "nr_maxRelRes0_V", "nr_maxRelRes_N", "nr_maxWellRelRes_mol", "nr_iter", "nr_tol", "nr_dPmin",
           "nr_dSmin", "nr_maxIter", "nr_state", "nr_finish",
           "ts_dPmax", "ts_dPBmax", "ts_dPWmax", "ts_dTmax", "ts_dNmax", "ts_dSmax", "ts_eVmax", "ts_iter",
           "ts_last_dt", "ts_current_time", "ts_next_dt", "ts_predict_dt", "ts_maxIncreFac", "ts_minChopFac",
           "ts_dPlim", "ts_dSlim", "ts_timeMax", "ts_timeMin", "ts_end_time", "ts_time_before"]

PRE_KEYS = ["P", "T", "Pb", "Ni", "Nt", "Pj", "S", "phaseExist", "xij", "lNi",
            "skip_flag", "skip_minEigen", "skip_P", "skip_T", "skip_zi", "u", "dt", "dSmax"]


def pack_fim(outdir):
    """Packs one run.  ``itNNN/jac_state`` holds the state the Jacobian of
    iteration NNN was assembled from; where that state equals the previous
    iteration's ``post`` state (all but lNi, which only enters the residual)
    only the arrays that differ are stored and ``jac_state/from_post`` names
    the iteration to take the rest from."""
    data = {}
    for k, v in load_dir(os.path.join(outdir, "model")).items():
        data[f"model/{k}"] = v
    for k, v in load_dir(os.path.join(outdir, "init"), set(STATE_KEYS)).items():
        data[f"init/{k}"] = v
    log = np.load(os.path.join(outdir, "log.npy"))
    data["log"] = log
    prev_post = None
    for it in range(len(log)):
        base = os.path.join(outdir, f"it{it:03d}")
        js = load_dir(os.path.join(base, "jac_state"),
                      set(STATE_KEYS + RES_KEYS + ["jac_rowptr", "jac_col", "jac_val", "dt"]))
        if prev_post is not None and all(
                k in ("lNi",) or k not in prev_post[1] or np.array_equal(js[k], prev_post[1][k])
                for k in STATE_KEYS if k in js):
            js = {k: v for k, v in js.items() if k not in STATE_KEYS or k == "lNi"}
            js["from_post"] = np.array([prev_post[0]])
        for k, v in js.items():
            data[f"it{it:03d}/jac_state/{k}"] = v
        pre = os.path.join(base, "pre")
        if os.path.isdir(pre):
            for k, v in load_dir(pre, set(PRE_KEYS)).items():
                data[f"it{it:03d}/pre/{k}"] = v
        post = os.path.join(base, "post")
        prev_post = None
        if os.path.isdir(post) and os.path.exists(os.path.join(post, "P.npy")):
            pd = load_dir(post, set(STATE_KEYS + RES_KEYS + NR_KEYS + ["flash_ftype", "flash_iters"]))
            for k, v in pd.items():
                data[f"it{it:03d}/post/{k}"] = v
            prev_post = (it, pd)
    return data


# the wells' part of the residual (harness dump_wells) and the bulk state it reads
WELL_KEYS = ["well_type", "well_mode", "well_nperf", "well_bhp", "well_tar_bhp", "well_tar_rate", "well_factor",
             "well_inj_zi", "well_qi", "perf_loc", "perf_WI", "perf_mult", "perf_dG", "perf_P", "perf_transj",
             "perf_trans_inj", "perf_xi", "perf_qi", "res_bulk", "res_full", "maxWellRelRes_mol",
             "perf_dir", "perf_kh", "perf_radius", "perf_skin", "perf_cell_dx", "perf_cell_dy", "perf_cell_dz",
             "perf_cell_ntg", "perf_cell_kx", "perf_cell_ky", "perf_cell_kz", "conv_darcy",
             "P", "Pj", "phaseExist", "kr", "mu", "xi", "xij"]


# the wells' part of the Jacobian: the system after the bulk assembly and after
# the wells' (all rows), the wells as assembled, and the bulk state it reads
WELL_JAC_KEYS = [k for k in WELL_KEYS if k.startswith(("well_", "perf_"))] + [
    "jac_rowptr", "jac_col", "jac_val", "jacw_rowptr", "jacw_col", "jacw_val", "dt",
    "P", "Pj", "phaseExist", "kr", "mu", "muP", "xi", "xiP", "xij", "xix", "mux", "dKrdS", "dPcdS", "dSec_dPri"]


def pack_wells(outdir, max_its=4):
    """The wells' part of each Newton iteration: at its post state the
    perforation data, fluxes and the residual with and without the wells; at
    its Jacobian state ("jac/") the system before and after the wells'
    assembly and what that assembly read."""
    data = {}
    for k, v in load_dir(os.path.join(outdir, "model")).items():
        if k in ("nb", "np", "nc", "numWell"):
            data[f"model/{k}"] = v
    n = 0
    for it in range(len(np.load(os.path.join(outdir, "log.npy")))):
        post = os.path.join(outdir, f"it{it:03d}", "post")
        if not os.path.exists(os.path.join(post, "well_type.npy")) or n >= max_its:
            continue
        for k, v in load_dir(post, set(WELL_KEYS)).items():
            data[f"it{it:03d}/{k}"] = v
        data[f"it{it:03d}/dt"] = np.load(os.path.join(outdir, f"it{it:03d}", "pre", "dt.npy"))
        js = os.path.join(outdir, f"it{it:03d}", "jac_state")
        if os.path.exists(os.path.join(js, "jacw_rowptr.npy")):
            for k, v in load_dir(js, set(WELL_JAC_KEYS)).items():
                data[f"it{it:03d}/jac/{k}"] = v
        n += 1
    return data


def run_fim(deck_text, name, max_iters, ni=None, calibrate=False, packer=pack_fim):
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, name + ".data")
        with open(deck, "w") as f:
            f.write(deck_text)
        if ni is not None:
            ni.astype("<f8").tofile(deck + ".ptn_ni")
            if calibrate:
                # scale the moles so the initial fluid volume fills the pores
                out0 = os.path.join(tmp, "out0")
                subprocess.run([DUMP, "fim", deck, out0, "0"], check=True, stdout=subprocess.DEVNULL)
                vf = np.load(os.path.join(out0, "init", "vf.npy"))
                vp = np.load(os.path.join(out0, "init", "rockVp.npy"))
                ni = ni * (vp / vf)[:, None]
                ni.astype("<f8").tofile(deck + ".ptn_ni")
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "fim", deck, out, str(max_iters)], check=True, stdout=subprocess.DEVNULL)
        data = packer(out)
        if ni is not None:
            data["ptn_ni"] = ni
    return data


def flash_cells(ncomp, n, seed, temp_k=345.0):
    """Random flash inputs: P ~ U(50, 400) bar, z ~ Dirichlet(1.5), unit moles."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(50.0, 400.0, n)
    z = rng.dirichlet(np.full(ncomp, 1.5), n)
    ni = np.concatenate([z * 10.0, np.full((n, 1), 1.0)], axis=1)
    t = np.full(n, temp_k - 273.15)
    return np.concatenate([p[:, None], t[:, None], ni], axis=1)


def run_flash(ncomp, ncell, seed):
    ni, deck_text = decks.comp_deck(1, 1, 1, ncomp, seed=seed, wells=False)
    cells = flash_cells(ncomp, ncell, seed + 7)
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "fluid.data")
        with open(deck, "w") as f:
            f.write(deck_text)
        ni.astype("<f8").tofile(deck + ".ptn_ni")
        cf = os.path.join(tmp, "cells.f64")
        cells.astype("<f8").tofile(cf)
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "flash", deck, cf, str(ncell), out], check=True, stdout=subprocess.DEVNULL)
        data = {f"model/{k}": v for k, v in load_dir(os.path.join(out, "model")).items()}
        for k, v in load_dir(os.path.join(out, "flash")).items():
            data[f"flash/{k}"] = v
    data["cells"] = cells
    return data


def _comp_fim(nx, ny, nz, ncomp, seed, name, max_iters, packer=pack_fim):
    ni, text = decks.comp_deck(nx, ny, nz, ncomp, seed=seed, tsteps=(0.02, 0.05, 0.1), smooth=True)
    data = run_fim(text, name, max_iters, ni=ni, calibrate=True, packer=packer)
    if packer is not pack_fim:
        data.pop("ptn_ni", None)
    return data


# faults of the faulted corner-point fixture (axis, index, throw at the first
# and last pillar, layer thickness factor of the moved side): a scissor fault
# along x whose throw changes sign, with thicker layers beyond it; a scissor
# fault along y with thinner layers; an x fault throwing two layers (NNCs
# across two layers)
CPG_FAULTS = [("x", 3, -4.5, 7.5, 1.5), ("y", 2, 1.2, -2.0, 0.6), ("x", 5, 6.0, 6.0, 0.7)]


def corner_inputs(nx, ny, nz, seed, faults=None):
    """COORD, ZCORN and rock arrays of a seeded dipping corner-point grid with
    leaning pillars (cut by `faults`, see synthetic.faulted_corner_point)."""
    sys.path.insert(0, REPO)
    from opencaeporox_gb300 import synthetic
    if faults:
        coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, 20.0, 3.0, 2000.0, 4.0, -3.0, faults, 0.05,
                                                      seed=seed)
    else:
        coord, zcorn = synthetic.dipping_corner_point(nx, ny, nz, 20.0, 3.0, 2000.0, 4.0, -3.0, 0.05, seed=seed)
    n = nx * ny * nz
    rng = np.random.default_rng(seed)
    kx = np.exp(rng.normal(np.log(100.0), 1.0, n))
    ky = kx * rng.uniform(0.5, 1.5, n)
    kz = 0.1 * kx
    poro = rng.uniform(0.15, 0.3, n)
    return coord, zcorn, kx, ky, kz, poro


def fault_fim_fixture(nx=8, ny=6, nz=5, seed=11, ncomp=3, max_iters=3):
    """Newton iterations of the reference on the faulted corner-point grid of
    cpg_fault_8x6x5 (a compositional deck with two wells), dumped like the
    other FIM fixtures, plus the grid inputs."""
    coord, zcorn, kx, ky, kz, poro = corner_inputs(nx, ny, nz, seed, CPG_FAULTS)
    text = decks.corner_grid_block(nx, ny, nz, coord, zcorn, poro, kx, ky, kz)
    ni, deck_text = decks.comp_deck(nx, ny, nz, ncomp, seed, grid_text=text, tsteps=(0.02, 0.05, 0.1), smooth=True)
    data = run_fim(deck_text, "fault", max_iters, ni=ni, calibrate=True)
    data.update({"input/dims": np.array([nx, ny, nz]), "input/coord": coord, "input/zcorn": zcorn,
                 "input/kx": kx, "input/ky": ky, "input/kz": kz, "input/poro": poro})
    return data


def corner_fixture(nx=6, ny=5, nz=4, seed=7, faults=None):
    """The reference's corner-point ingest (COORD / ZCORN) on a dipping grid
    with leaning pillars (cut by `faults`): the model dump (cells,
    connections, half areas, transmissibilities) and the inputs that produced
    it."""
    coord, zcorn, kx, ky, kz, poro = corner_inputs(nx, ny, nz, seed, faults)
    text = decks.corner_grid_block(nx, ny, nz, coord, zcorn, poro, kx, ky, kz)
    ni, deck_text = decks.comp_deck(nx, ny, nz, 3, seed, grid_text=text)
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "cpg.data")
        with open(deck, "w") as f:
            f.write(deck_text)
        ni.astype("<f8").tofile(deck + ".ptn_ni")
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "fim", deck, out, "0"], check=True, stdout=subprocess.DEVNULL)
        data = {f"model/{k}": v for k, v in load_dir(os.path.join(out, "model")).items()}
    data.update({"input/dims": np.array([nx, ny, nz]), "input/coord": coord, "input/zcorn": zcorn,
                 "input/kx": kx, "input/ky": ky, "input/kz": kz, "input/poro": poro})
    return data


def overlap_pairs(n=1536, seed=5):
    """Seeded pairs of faces on a vertical plane between two slightly leaning
    pillars 20 m apart (points (x, depth): p0 upper and p3 lower on the right
    pillar, p1 upper and p2 lower on the left), with independent tops and
    thicknesses so that every crossing pattern of their edges occurs; the last
    64 pairs have parallel upper edges."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 2, 4, 2))
    for s in range(2):
        top_r, top_l = rng.uniform(0, 10, n), rng.uniform(0, 10, n)
        th_r, th_l = rng.uniform(0.5, 10, n), rng.uniform(0.5, 10, n)
        lean = rng.uniform(-0.05, 0.05, (n, 2))
        if s == 1:
            top_r[-64:] = out[-64:, 0, 0, 1] + 1.5
            top_l[-64:] = out[-64:, 0, 1, 1] + 1.5
            lean[-64:] = 0.0
        d = np.stack([top_r, top_l, top_l + th_l, top_r + th_r], 1)
        if s == 0:
            lean[-64:] = 0.0
        x = np.stack([20.0 + lean[:, 0] * d[:, 0], lean[:, 1] * d[:, 1], lean[:, 1] * d[:, 2],
                      20.0 + lean[:, 0] * d[:, 3]], 1)
        out[:, s, :, 0], out[:, s, :, 1] = x, d
    return out


def overlap_fixture():
    """The reference's CalAreaNotQuadr on overlap_pairs()."""
    pairs = overlap_pairs()
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "pairs.f64")
        pairs.astype("<f8").tofile(f)
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "overlap", f, str(len(pairs)), out], check=True, stdout=subprocess.DEVNULL)
        area = np.load(os.path.join(out, "area.npy"))
    return {"pairs": pairs, "area": area}


def grid_deck_texts(kind, seed=21):
    """GRID sections for the deck-reader fixtures: `kind` is "ortho" or
    "corner" (the faulted grid of cpg_fault_8x6x5), then "_actnum" (inactive
    cells by ACTNUM, by an EQUALS box of ACTNUM and by zero porosity, with
    NTG) or "_multz" (all cells active, with NTG and MULTZ).  Arrays come as
    plain values, `m*v` repeats, EQUALS / MULTIPLY / COPY boxes and one
    INCLUDE file.  Returns (nx, ny, nz, grid_text, include_text)."""
    rng = np.random.default_rng(seed)
    corner = kind.startswith("corner")
    nx, ny, nz = (8, 6, 5) if corner else (7, 5, 4)
    n = nx * ny * nz
    lines = [f"DIMENS\n{nx} {ny} {nz} /\n"]
    if corner:
        coord, zcorn, kx, ky, kz, poro = corner_inputs(nx, ny, nz, 11, CPG_FAULTS)
        lines.append(f"COORD\n{decks._fmt(coord)}\n/\nZCORN\n{decks._fmt(zcorn)}\n/\n")
    else:
        dx = np.repeat(rng.uniform(15.0, 25.0, nx)[None, :], ny * nz, 0).ravel()
        dy = np.tile(np.repeat(rng.uniform(15.0, 25.0, ny), nx), nz)
        dz = np.repeat(rng.uniform(2.0, 6.0, nz), nx * ny) * rng.uniform(0.9, 1.1, n)
        tops = 2000.0 + rng.uniform(-3.0, 3.0, nx * ny)
        lines.append(f"DX\n{decks._fmt(dx)}\n/\nDY\n{decks._fmt(dy)}\n/\n"
                     f"-- layer thicknesses vary cell by cell\nDZ\n{decks._fmt(dz)}\n/\n"
                     f"TOPS\n{decks._fmt(tops)}\n/\n")
        kx = np.exp(rng.normal(np.log(100.0), 1.0, n))
        poro = rng.uniform(0.15, 0.3, n)
    ntg = rng.uniform(0.5, 1.0, n)
    if kind.endswith("_actnum"):
        poro = poro.copy()
        poro[[5, 17, n - 9]] = 0.0                       # inactive by the pore-volume cut
    include = f"PORO\n{decks._fmt(poro)}\n/\n"
    lines.append("INCLUDE\n'grid_poro.inc' /\n")
    lines.append(f"PERMX\n{decks._fmt(kx)}\n/\n")
    lines.append(f"NTG\n{decks._fmt(ntg)}\n/\n")
    # PERMY from PERMX, scaled in a box; PERMZ a tenth of PERMX
    lines.append("COPY\nPERMX PERMY 6* /\nPERMX PERMZ 6* /\n/\n")
    lines.append(f"MULTIPLY\nPERMY 0.7 2 {nx - 1} 1* {ny} 2* /\nPERMZ 0.1 6* /\n/\n")
    lines.append(f"EQUALS\nPERMY 55.5 1 2 1 1 1 {nz} /\n/\n")
    if kind.endswith("_actnum"):
        act = np.ones(n, np.int64)
        off = [3 + nx * 2, 4 + nx * 2 + nx * ny, 2 + nx * (ny - 2) + 2 * nx * ny, 1 + nx + nx * ny]
        act[off] = 0
        # one run of repeats, as decks write long runs
        body = " ".join(f"{v}" for v in act[:nx * ny]) + "\n" + f"{n - nx * ny - 1}*1 1"
        tail = act[nx * ny:]
        if np.all(tail == 1):
            text = body
        else:
            text = " ".join(f"{v}" for v in act[:nx * ny]) + "\n" + " ".join(f"{v}" for v in tail)
        lines.append(f"ACTNUM\n{text}\n/\n")
        # and a box of inactive cells away from the wells' columns
        lines.append(f"EQUALS\nACTNUM 0 {nx - 2} {nx - 2} 2 3 2 2 /\n/\n")
    else:
        multz = rng.uniform(0.05, 1.0, n)
        lines.append(f"MULTZ\n{decks._fmt(multz)}\n/\n")
    return nx, ny, nz, "".join(lines), include


def deck_grid_fixture(kind):
    """The reference's grid from a GRID section of grid_deck_texts(kind)
    inside a compositional deck with two wells: the model dump and the deck
    texts (the test reads them with opencaeporox_gb300.deck)."""
    nx, ny, nz, grid_text, include = grid_deck_texts(kind)
    ni, deck_text = decks.comp_deck(nx, ny, nz, 3, 21, grid_text=grid_text)
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "grid.data")
        with open(deck, "w") as f:
            f.write(deck_text)
        with open(os.path.join(tmp, "grid_poro.inc"), "w") as f:
            f.write(include)
        ni.astype("<f8").tofile(deck + ".ptn_ni")
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "fim", deck, out, "0"], check=True, stdout=subprocess.DEVNULL)
        data = {f"model/{k}": v for k, v in load_dir(os.path.join(out, "model")).items()}
    data["deck/main"] = np.array(deck_text)
    data["deck/include"] = np.array(include)
    return data


def corpus_case(seed):
    """One seeded small grid for the grid corpus: (nx, ny, nz, GRID text).
    Even seeds: corner-point with one to three random faults (throws up to
    two layers, scissor faults, thickness changes) and leaning pillars; odd
    seeds: block-centred with per-cell sizes.  Random inactive cells
    (ACTNUM or zero porosity) in half the cases, NTG in half, MULTZ where
    every cell is active."""
    sys.path.insert(0, REPO)
    from opencaeporox_gb300 import synthetic
    rng = np.random.default_rng(1000 + seed)
    nx, ny, nz = int(rng.integers(3, 8)), int(rng.integers(3, 7)), int(rng.integers(2, 6))
    n = nx * ny * nz
    dz = float(rng.uniform(2.0, 5.0))
    lines = [f"DIMENS\n{nx} {ny} {nz} /\n"]
    if seed % 2 == 0:
        faults = []
        for _ in range(int(rng.integers(1, 4))):
            axis = "x" if rng.random() < 0.5 else "y"
            index = int(rng.integers(0, (nx if axis == "x" else ny) - 1))
            t0, t1 = rng.uniform(-2.2, 2.2, 2) * dz
            faults.append((axis, index, float(t0), float(t1), float(rng.uniform(0.5, 1.8))))
        coord, zcorn = synthetic.faulted_corner_point(nx, ny, nz, float(rng.uniform(10, 30)), dz, 2000.0,
                                                      float(rng.uniform(-6, 6)), float(rng.uniform(-6, 6)),
                                                      faults, float(rng.uniform(0, 0.08)), seed=seed)
        lines.append(f"COORD\n{decks._fmt(coord)}\n/\nZCORN\n{decks._fmt(zcorn)}\n/\n")
    else:
        lines.append(f"DX\n{decks._fmt(rng.uniform(10, 30, n))}\n/\nDY\n{decks._fmt(rng.uniform(10, 30, n))}\n/\n"
                     f"DZ\n{decks._fmt(rng.uniform(1, 6, n))}\n/\nTOPS\n{decks._fmt(2000 + rng.uniform(-5, 5, nx * ny))}\n/\n")
    poro = rng.uniform(0.1, 0.3, n)
    inactive = rng.random() < 0.5
    if inactive:
        poro[rng.choice(n, size=max(1, n // 15), replace=False)] = 0.0
    lines.append(f"PORO\n{decks._fmt(poro)}\n/\n")
    kx = np.exp(rng.normal(np.log(100.0), 1.0, n))
    lines.append(f"PERMX\n{decks._fmt(kx)}\n/\nPERMY\n{decks._fmt(kx * rng.uniform(0.5, 1.5, n))}\n/\n"
                 f"PERMZ\n{decks._fmt(0.1 * kx)}\n/\n")
    if rng.random() < 0.5:
        lines.append(f"NTG\n{decks._fmt(rng.uniform(0.5, 1.0, n))}\n/\n")
    if inactive:
        act = (rng.random(n) > 0.1).astype(int)
        # keep the two wells' columns (first and last) active
        col = np.arange(n) % (nx * ny)
        act[(col == 0) | (col == nx * ny - 1)] = 1
        lines.append("ACTNUM\n" + " ".join(str(a) for a in act) + "\n/\n")
    else:
        lines.append(f"MULTZ\n{decks._fmt(rng.uniform(0.05, 1.0, n))}\n/\n")
    return nx, ny, nz, "".join(lines)


def grid_corpus(ncase=40):
    """The reference's grid (model dump) for each corpus_case, with the GRID
    texts; cases the reference refuses are recorded as refused."""
    data = {}
    for seed in range(ncase):
        nx, ny, nz, grid_text = corpus_case(seed)
        col = np.arange(nx * ny * nz) % (nx * ny)
        ni, deck_text = decks.comp_deck(nx, ny, nz, 3, 7, grid_text=grid_text)
        with tempfile.TemporaryDirectory() as tmp:
            deck = os.path.join(tmp, "case.data")
            with open(deck, "w") as f:
                f.write(deck_text)
            ni.astype("<f8").tofile(deck + ".ptn_ni")
            out = os.path.join(tmp, "out")
            r = subprocess.run([DUMP, "fim", deck, out, "0"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            data[f"case{seed:03d}/grid"] = np.array(grid_text)
            if r.returncode != 0:
                data[f"case{seed:03d}/refused"] = np.array(r.returncode)
                continue
            m = load_dir(os.path.join(out, "model"))
            for k in ("nb", "conn_bId", "conn_eId", "conn_trans", "conn_areaB", "conn_areaE", "v", "depth",
                      "poroInit", "ntg", "rockKx", "rockKy", "rockKz", "dx", "dy", "dz", "CONV_DARCY"):
                data[f"case{seed:03d}/{k}"] = m[k]
    return data


def deck_wells_fixture():
    """The reference's perforations and well indices from WELSPECS/COMPDAT
    on the faulted grid with inactive cells (grid_deck_texts("corner_actnum")):
    default and explicit directions, a given kh, a skin, a given WI, a record
    naming its wells by a prefix and one in an inactive cell.  One Newton
    iteration, for the well dump."""
    nx, ny, nz, grid_text, include = grid_deck_texts("corner_actnum")
    ni, deck_text = decks.comp_deck(nx, ny, nz, 3, 21, grid_text=grid_text)
    compdat = f"""COMPDAT
'INJE1'   2*   1   2     1*   0.2   3*   /
'INJE1'   4   3   1   1   1*   0.2   3*   /
'INJE1'   2   1   3   {nz}   1*   0.25   1*   1.5   'X'   /
'PROD*'   2*   1   2   1*   0.3   40.0   1*   'Y'   /
'PROD1'   {nx - 1}   {ny}   3   3   1*   0.2   3*   /
'PROD1'   2*   4   {nz}   25.0   0.2   3*   /
/
"""
    i = deck_text.index("COMPDAT")
    j = deck_text.index("/\n/\n", i) + 4
    deck_text = deck_text[:i] + compdat + deck_text[j:]
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "grid.data")
        with open(deck, "w") as f:
            f.write(deck_text)
        with open(os.path.join(tmp, "grid_poro.inc"), "w") as f:
            f.write(include)
        ni.astype("<f8").tofile(deck + ".ptn_ni")
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "fim", deck, out, "1"], check=True, stdout=subprocess.DEVNULL)
        data = {f"model/{k}": v for k, v in load_dir(os.path.join(out, "model")).items()
                if k in ("nb", "CONV_DARCY", "CONV1")}
        for k, v in load_dir(os.path.join(out, "it000", "jac_state")).items():
            if k.startswith("perf_") or k.startswith("well_"):
                data[f"wells/{k}"] = v
    data["deck/main"] = np.array(deck_text)
    data["deck/include"] = np.array(include)
    return data


def props_variant_texts():
    """Decks for the PROPS reader that take the branches the other fixtures
    do not: FIELD units, GRAVITY, VCRIT, OMEGAA / OMEGAB, SSHIFT, VCRITVIS,
    LBCCOEF with defaults, a full BIC matrix, LINEAR02 rock, and a black-oil
    deck with GRAVITY.  Returns {name: deck text}."""
    out = {}
    ncomp = 4
    comp = decks.seeded_components(ncomp, 13)
    ni, base = decks.comp_deck(4, 3, 2, ncomp, seed=13)
    rng = np.random.default_rng(13)
    vc = comp["Zc"] * 10.73159 * comp["Tc"] / comp["Pc"] * 0.08
    extra = (f"VCRIT\n{decks._fmt(vc, 1)}\n/\nOMEGAA\n{decks._fmt(0.457235529 * rng.uniform(0.98, 1.02, ncomp), 1)}\n/\n"
             f"OMEGAB\n{decks._fmt(0.077796074 * rng.uniform(0.98, 1.02, ncomp), 1)}\n/\n"
             f"SSHIFT\n{decks._fmt(rng.uniform(-0.1, 0.1, ncomp), 1)}\n/\n"
             f"VCRITVIS\n{decks._fmt(vc * 1.1, 1)}\n/\nLBCCOEF\n0.1025 2* -0.0408 1* /\n")
    t = base.replace("ZCRIT", "ZCRIT_UNUSED").replace("NCOMPS", extra + "NCOMPS", 1)
    t = t.replace("METRIC", "FIELD").replace("DENSITY\n850.0 1000.0 0.9 /", "GRAVITY\n40.0 1.02 0.75 /")
    t = t.replace("LINEAR01 200.0 4.5E-5", "LINEAR02 3000.0 3.0E-6 1.0E-7")
    out["comp_field_gravity"] = (t, ni)
    full = " ".join(f"{v:.17g}" for v in comp["BIC"].ravel())
    i = base.index("BIC")
    j = base.index("/", i)
    t2 = base[:i] + "BIC\n" + full + " " + base[j:]
    out["comp_fullbic"] = (t2, ni)
    bo = decks.blackoil_deck(seed=3)
    bo = bo.replace("DENSITY\n850.0 1000.0 0.9 /", "GRAVITY\n35.0 1.01 0.7 /").replace("METRIC", "FIELD")
    out["bo_field_gravity"] = (bo, None)
    return out


def props_fixture():
    """The reference's model dump for each props_variant_texts deck, with the
    deck text."""
    data = {}
    for name, (text, ni) in props_variant_texts().items():
        with tempfile.TemporaryDirectory() as tmp:
            deck = os.path.join(tmp, "props.data")
            with open(deck, "w") as f:
                f.write(text)
            if ni is not None:
                ni.astype("<f8").tofile(deck + ".ptn_ni")
            out = os.path.join(tmp, "out")
            r = subprocess.run([DUMP, "fim", deck, out, "0"], stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                               text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{name}: the reference refused the deck: {r.stderr[-400:]}")
            for k, v in load_dir(os.path.join(out, "model")).items():
                if not k.startswith("conn_") and k not in ("v", "depth", "poroInit", "ntg", "rockKx", "rockKy",
                                                            "rockKz", "dx", "dy", "dz"):
                    data[f"{name}/{k}"] = v
        data[f"{name}/deck"] = np.array(text)
    return data


def deck_ptn_fixture(kind="INITPTN0"):
    """The reference's state after a PTN start whose arrays are all in the
    deck (three hydrocarbon components and water, so every COMPM array fits
    the reference's limit of 30 per-cell arrays; no side file): PRESSURE,
    TEMPER, PHASEP-0..2 and COMPM-0..3 per cell, on the block-centred grid
    with inactive cells of deck_ortho_actnum.  The model's initial dump."""
    nx, ny, nz, grid_text, include = grid_deck_texts("ortho_actnum")
    n = nx * ny * nz
    ni, text = decks.comp_deck(nx, ny, nz, 3, 21, grid_text=grid_text)
    rng = np.random.default_rng(77)
    p = rng.uniform(100.0, 300.0, n)
    t = 70.0 + rng.uniform(-2.0, 2.0, n)
    i = text.index("INITPTN0")
    j = text.index("PROPS")
    init = ["INITPTN0", "PRESSURE", decks._fmt(p), "/", "TEMPER", decks._fmt(t), "/"]
    for k in range(3):
        init += [f"PHASEP-{k}", decks._fmt(p + k), "/"]
    for c in range(ni.shape[1]):
        init += [f"COMPM-{c}", decks._fmt(ni[:, c]), "/"]
    text = text[:i] + "\n".join(init) + "\n\n" + text[j:]
    with tempfile.TemporaryDirectory() as tmp:
        deck = os.path.join(tmp, "grid.data")
        with open(deck, "w") as f:
            f.write(text)
        with open(os.path.join(tmp, "grid_poro.inc"), "w") as f:
            f.write(include)
        out = os.path.join(tmp, "out")
        subprocess.run([DUMP, "fim", deck, out, "0"], check=True, stdout=subprocess.DEVNULL)
        data = {f"init/{k}": v for k, v in load_dir(os.path.join(out, "init"), {"P", "T", "Ni", "Pj"}).items()}
        data["model/nb"] = np.load(os.path.join(out, "model", "nb.npy"))
    data["deck/main"] = np.array(text)
    data["deck/include"] = np.array(include)
    return data


def field_fim_fixture():
    """Newton iterations of the reference on a compositional deck in FIELD
    units with GRAVITY (the other FIM fixtures are METRIC with DENSITY): the
    unit constants (CONV1, the gas constant, the gravity factor, the Darcy
    factor) and the standard water density from GRAVITY enter every
    property, residual and Jacobian."""
    ni, text = decks.comp_deck(6, 5, 3, 4, seed=9, tsteps=(0.02, 0.05, 0.1), smooth=True)
    text = text.replace("METRIC", "FIELD").replace("DENSITY\n850.0 1000.0 0.9 /", "GRAVITY\n40.0 1.02 0.75 /")
    return run_fim(text, "field", 3, ni=ni, calibrate=True)


def fim_corpus(ncase=6):
    """Two Newton iterations of the reference on each of `ncase` seeded small
    decks: the grids of corpus_case (faulted corner-point or block-centred,
    inactive cells, NTG, MULTZ) with 3 to 5 components and the two wells of
    the compositional deck.  Packed per case under case<NNN>/."""
    data = {}
    for seed in range(ncase):
        nx, ny, nz, grid_text = corpus_case(seed)
        ncomp = 3 + seed % 3
        ni, text = decks.comp_deck(nx, ny, nz, ncomp, seed=50 + seed, grid_text=grid_text,
                                   tsteps=(0.02, 0.05), smooth=True)
        # the harness reads the side file's moles per active cell
        sys.path.insert(0, REPO)
        from opencaeporox_gb300 import deck as D
        with tempfile.TemporaryDirectory() as tmp:
            g = os.path.join(tmp, "g.data")
            with open(g, "w") as f:
                f.write(grid_text)
            _, geo = D.grid_from_deck(D.read_grid_deck(g))
        d = run_fim(text, f"corpus{seed}", 2, ni=ni[geo["act2all"]], calibrate=True)
        for k, v in d.items():
            data[f"case{seed:03d}/{k}"] = v
    return data


FIXTURES = {
    "bo_10x10x3": lambda: run_fim(decks.blackoil_deck(seed=1), "bo", 12),
    "comp6_8x8x3": lambda: _comp_fim(8, 8, 3, 6, 2, "c6", 4),
    "comp8_6x6x4": lambda: _comp_fim(6, 6, 4, 8, 4, "c8", 4),
    "flash10": lambda: run_flash(10, 1024, 3),
    "cpg_6x5x4": corner_fixture,
    "cpg_fault_8x6x5": lambda: corner_fixture(8, 6, 5, 11, faults=CPG_FAULTS),
    "overlap_area": overlap_fixture,
    "fault_comp3_8x6x5": fault_fim_fixture,
    "deck_ortho_actnum": lambda: deck_grid_fixture("ortho_actnum"),
    "deck_ortho_multz": lambda: deck_grid_fixture("ortho_multz"),
    "deck_corner_actnum": lambda: deck_grid_fixture("corner_actnum"),
    "deck_corner_multz": lambda: deck_grid_fixture("corner_multz"),
    "grid_corpus": grid_corpus,
    "deck_wells": deck_wells_fixture,
    "props_variants": props_fixture,
    "deck_ptn": deck_ptn_fixture,
    "comp4_field_6x5x3": field_fim_fixture,
    "fim_corpus": fim_corpus,
    "bo_field_10x10x3": lambda: run_fim(decks.blackoil_deck(seed=1).replace("METRIC", "FIELD").replace(
        "DENSITY\n850.0 1000.0 0.9 /", "GRAVITY\n35.0 1.01 0.7 /"), "bof", 6),
    "wells_bo_10x10x3": lambda: run_fim(decks.blackoil_deck(seed=1), "bo", 12, packer=pack_wells),
    "wells_comp6_8x8x3": lambda: _comp_fim(8, 8, 3, 6, 2, "c6", 4, packer=pack_wells),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    build_reference()
    for name, fn in FIXTURES.items():
        if args.only and name != args.only:
            continue
        data = fn()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print(f"{name}: {len(data)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
