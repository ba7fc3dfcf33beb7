"""An ECL-style input deck, as far as the device path needs it, read as the
reference reads it, and what the reference builds from it:

- the GRID section (PreParamGridWell::InputFile,
  src/PreParamGridWell.cpp:25-150) and the grid (PreParamGridWell::Setup,
  :876-1020): the cells that stay active, their geometry and the connections
  between them (read_grid_deck, grid_from_deck);
- the wells' perforations and Peaceman indices from WELSPECS / COMPDAT
  (read_wells, well_perforations);
- the fluid, rock and tables of the device's Model (read_model).

The GRID section in detail:

Read as the reference reads it:

- line by line; blank lines and lines starting with `#` or `--` are skipped;
  a line ends at its first `/`, which stands as the line's last token;
  quotes and commas separate tokens;
- the first token of a line names a keyword; lines whose first token names
  none are skipped (so the data of other keywords is passed over);
- DIMENS: nx ny nz on the next line;
- grid arrays (DX DY DZ TOPS COORD ZCORN PORO NTG PERMX PERMY PERMZ MULTZ
  ACTNUM): the values on the following lines up to a line starting with `/`,
  `m*v` meaning v repeated m times; values on the keyword's own line are not
  read;
- EQUALS, MULTIPLY (name value box) and COPY (source target box), one record
  per line up to a line starting with `/`; the box is i1 i2 j1 j2 k1 k2
  (1-based, inclusive), `m*` leaves m of its bounds at their default (the
  whole grid); for TOPS the box is the top layer;
- INCLUDE: the file named on the next line, relative to the main deck's
  directory (so the name holds no `/`, which would end the line).

Then PostProcessInput (:196-213): NTG of the wrong length is dropped (NTG 1),
otherwise PORO becomes PORO * NTG; ACTNUM of the wrong length is dropped (all
cells active).  A grid is corner-point when COORD or ZCORN is given,
block-centred (DX DY DZ TOPS) otherwise.

Two points where this reader accepts more than the reference: values before
a `/` that ends a data line are read (the reference stops with an error on
such a line), and an EQUALS/MULTIPLY/COPY record with fewer than six box
bounds leaves the missing ones at their default (the reference reads past the
record).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import grid as G
from . import wells as W

REAL_ARRAYS = ("DX", "DY", "DZ", "TOPS", "COORD", "ZCORN", "NTG", "PORO", "PERMX", "PERMY", "PERMZ", "MULTZ",
               # the PTN start (read by the same reader in the reference)
               "PRESSURE", "TEMPER", "PHASEP-0", "PHASEP-1", "PHASEP-2") + tuple(f"COMPM-{i}" for i in range(10))
INT_ARRAYS = ("ACTNUM",)


@dataclass
class GridDeck:
    """The GRID-section input of a deck: dimensions and arrays as read, in
    the reference's cell order (i fastest, then j, then k)."""
    nx: int = 0
    ny: int = 0
    nz: int = 0
    arrays: dict = field(default_factory=dict)
    init: str = ""           # INITPTN0 (arrays of every cell) or INITPTN1 (of the active cells)

    @property
    def n(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def corner(self) -> bool:
        return "COORD" in self.arrays or "ZCORN" in self.arrays


def _tokens(line: str):
    """ReadLine (src/UtilInput.cpp:14-52) on one line: None for a skipped
    line, else its tokens."""
    s = line.lstrip(" \t\r")
    if not s.strip() or s[0] == "#" or s.startswith("--"):
        return None
    cut = s.find("/")
    if cut >= 0:
        s = s[:cut] + "/"
    s = s.replace("'", " ").replace(",", " ")
    toks = s.split()
    return toks or None


def _lines(path: str):
    with open(path) as fh:
        for line in fh:
            t = _tokens(line)
            if t is not None:
                yield t


def _expand(tok: str, cast):
    """`m*v` as m copies of v, otherwise the value itself."""
    star = tok.find("*")
    if star < 0:
        return [cast(tok)]
    return [cast(tok[star + 1:])] * int(tok[:star])


def _box(tokens, nx, ny, nz):
    """The 0-based inclusive box of an EQUALS/MULTIPLY/COPY record (tokens
    after the first two), `m*` defaults expanded (DealDefault,
    src/UtilInput.cpp:54-76)."""
    vals = []
    for t in tokens:
        if t == "/":
            break
        star = t.find("*")
        if star >= 0 and t[:star].isdigit() and int(t[:star]) > 0:
            m = int(t[:star])
            vals += ([None] * m) if star == len(t) - 1 else [t[star + 1:]] * m
        else:
            vals.append(t)
    box = [0, nx - 1, 0, ny - 1, 0, nz - 1]
    for q in range(6):
        if q < len(vals) and vals[q] is not None:
            box[q] = int(vals[q]) - 1
    return box


def _box_index(box, nx, ny, nz, tops=False):
    i0, i1, j0, j1, k0, k1 = box
    if tops:
        k0 = k1 = 0
    if min(i0, j0, k0) < 0 or i1 >= nx or j1 >= ny or k1 >= nz:
        raise ValueError(f"box {[b + 1 for b in box]} out of range")
    k, j, i = np.meshgrid(np.arange(k0, k1 + 1), np.arange(j0, j1 + 1), np.arange(i0, i1 + 1), indexing="ij")
    return (k * nx * ny + j * nx + i).ravel()


def read_grid_deck(path: str, deck: GridDeck | None = None, workdir: str | None = None) -> GridDeck:
    """Read the grid keywords of the deck file `path` (and of the files it
    includes)."""
    deck = deck or GridDeck()
    workdir = workdir if workdir is not None else os.path.dirname(os.path.abspath(path))
    lines = _lines(path)
    A = deck.arrays

    def size_of(name):
        return deck.nx * deck.ny if name == "TOPS" else deck.n

    def target(name):
        if name not in REAL_ARRAYS + INT_ARRAYS:
            raise ValueError(f"unknown grid array {name}")
        a = A.get(name)
        if a is None or len(a) < size_of(name):
            # EQUALS on an array not read yet starts from zeros
            b = np.zeros(size_of(name), np.int64 if name in INT_ARRAYS else np.float64)
            if a is not None:
                b[:len(a)] = a
            A[name] = a = b
        return a

    for toks in lines:
        key = toks[0]
        if key == "DIMENS":
            dims = next(lines)
            deck.nx, deck.ny, deck.nz = (int(x) for x in dims[:3])
        elif key in ("INITPTN0", "INITPTN1"):
            deck.init = key
        elif key in REAL_ARRAYS or key in INT_ARRAYS:
            # integer arrays are read as numbers and truncated, as the reference stores them
            cast = (lambda x: int(float(x))) if key in INT_ARRAYS else float
            vals = []
            for t in lines:
                if t[0] == "/":
                    break
                for tok in t:
                    if tok != "/":
                        vals += _expand(tok, cast)
                if t[-1] == "/":
                    break
            new = np.array(vals, np.int64 if key in INT_ARRAYS else np.float64)
            A[key] = np.concatenate([A[key], new]) if key in A else new
        elif key in ("EQUALS", "MULTIPLY"):
            for t in lines:
                if t[0] == "/":
                    break
                name, val = t[0], float(t[1])
                idx = _box_index(_box(t[2:], deck.nx, deck.ny, deck.nz), deck.nx, deck.ny, deck.nz, name == "TOPS")
                if key == "EQUALS":
                    a = target(name)
                    a[idx] = int(val) if name in INT_ARRAYS else val
                else:
                    if name not in A or len(A[name]) < size_of(name):
                        raise ValueError(f"MULTIPLY of {name}, which is not given")
                    if name in INT_ARRAYS:
                        raise ValueError(f"MULTIPLY of the integer array {name}")
                    A[name][idx] = A[name][idx] * val
        elif key == "COPY":
            for t in lines:
                if t[0] == "/":
                    break
                src, dst = t[0], t[1]
                if src not in A:
                    raise ValueError(f"COPY from {src}, which is not given")
                if (src in INT_ARRAYS) != (dst in INT_ARRAYS):
                    raise ValueError(f"COPY between {src} and {dst} of different types")
                idx = _box_index(_box(t[2:], deck.nx, deck.ny, deck.nz), deck.nx, deck.ny, deck.nz)
                a = A.get(dst)
                if a is None or len(a) != len(A[src]):
                    b = np.zeros(len(A[src]), A[src].dtype)
                    if a is not None:
                        b[:min(len(a), len(b))] = a[:len(b)]
                    A[dst] = a = b
                a[idx] = A[src][idx]
        elif key == "INCLUDE":
            name = next(lines)[0]
            if name.endswith("/"):
                raise ValueError(f"INCLUDE {name!r}: a '/' ends the line, so the file name cannot hold one")
            read_grid_deck(os.path.join(workdir, name), deck, workdir)
    return deck


def grid_from_deck(deck: GridDeck, conv_darcy: float = 0.008527):
    """The active cells and their connections as the reference builds them
    from `deck` (grid.orthogonal_grid or grid.corner_point_grid on the
    post-processed arrays).  Returns (Grid, geometry): geometry holds per
    active cell its index among all cells (act2all), dx, dy, dz, NTG and the
    permeabilities."""
    n, A = deck.n, deck.arrays
    if n == 0:
        raise ValueError("DIMENS is not given")
    for name in ("PORO", "PERMX", "PERMY", "PERMZ"):
        if name not in A or len(A[name]) != n:
            raise ValueError(f"{name} must give {n} values")
    ntg = A.get("NTG")
    ntg = ntg if ntg is not None and len(ntg) == n else None
    actnum = A.get("ACTNUM")
    actnum = actnum if actnum is not None and len(actnum) == n else None
    multz = A.get("MULTZ")
    if multz is not None and len(multz) != n:
        raise ValueError(f"MULTZ must give {n} values")
    common = dict(ntg=ntg, conv_darcy=conv_darcy, actnum=actnum, multz=multz, return_geometry=True)
    if deck.corner:
        if len(A.get("COORD", ())) != (deck.nx + 1) * (deck.ny + 1) * 6 or len(A.get("ZCORN", ())) != 8 * n:
            raise ValueError("COORD or ZCORN of the wrong length")
        return G.corner_point_grid(deck.nx, deck.ny, deck.nz, A["COORD"], A["ZCORN"], A["PERMX"], A["PERMY"],
                                   A["PERMZ"], A["PORO"], **common)
    for name in ("DX", "DY", "DZ"):
        if name not in A or len(A[name]) != n:
            raise ValueError(f"{name} must give {n} values")
    if "TOPS" not in A or len(A["TOPS"]) != deck.nx * deck.ny:
        raise ValueError(f"TOPS must give {deck.nx * deck.ny} values")
    return G.orthogonal_grid(deck.nx, deck.ny, deck.nz, A["DX"], A["DY"], A["DZ"], A["TOPS"], A["PERMX"],
                             A["PERMY"], A["PERMZ"], A["PORO"], **common)


# ------------------------------------------------------------------ wells ---
@dataclass
class WellSpec:
    """A structured well of WELSPECS with its COMPDAT perforations, one per
    layer: (I, J, K, WI, diameter, kh, skin, direction), 1-based cells, -1 for
    a WI or kh not given."""
    name: str
    I: int
    J: int
    perfs: list = field(default_factory=list)


def _defaults(tokens):
    """DealDefault: m* as m DEFAULT entries, m*v as m copies of v."""
    out = []
    for t in tokens:
        star = t.find("*")
        num = int(t[:star]) if star > 0 and t[:star].isdigit() else 0
        if num == 0:
            out.append(t)
        else:
            out += ["DEFAULT" if star == len(t) - 1 else t[star + 1:]] * num
    return out


def read_wells(path: str, workdir: str | None = None, wells: list | None = None) -> list:
    """WELSPECS and COMPDAT of a deck (and the files it includes), as
    PreParamGridWell::InputWELSPECS / InputCOMPDAT and WellParam read them
    (src/PreParamGridWell.cpp:554-600, src/ParamWell.cpp:50-128): a COMPDAT
    record names a well, or with a trailing `*` every well whose name starts
    so; I J default to the well's; K1..K2 give one perforation per layer;
    then WI, diameter (default 1), kh, skin (default 0) and direction (x, y,
    z; default z).  Wells given by coordinates are not read."""
    wells = [] if wells is None else wells
    workdir = workdir if workdir is not None else os.path.dirname(os.path.abspath(path))
    lines = _lines(path)
    for toks in lines:
        key = toks[0]
        if key == "WELSPECS":
            for t in lines:
                if t[0] == "/":
                    break
                v = _defaults(t)
                if "COORDINATE" in v[-2:]:
                    raise ValueError(f"well {v[0]}: wells given by coordinates are not read")
                wells.append(WellSpec(v[0], int(v[2]), int(v[3])))
        elif key == "COMPDAT":
            for t in lines:
                if t[0] == "/":
                    break
                v = _defaults(t)
                v = v[:-1] if v[-1] == "/" else v
                v += ["DEFAULT"] * (10 - len(v))
                name = v[0]
                star = name.find("*")
                match = (lambda w: w.name[:star] == name[:star]) if star >= 0 else (lambda w: w.name == name)
                for w in wells:
                    if not match(w):
                        continue
                    I, J = (w.I, w.J) if "DEFAULT" in (v[1], v[2]) else (int(v[1]), int(v[2]))
                    for k in range(int(v[3]), int(v[4]) + 1):
                        d = v[9].lower() if v[9] != "DEFAULT" else "z"
                        if d not in ("x", "y", "z"):
                            raise ValueError(f"well {w.name}: perforation direction {v[9]!r}")
                        w.perfs.append((I, J, k, -1.0 if v[5] == "DEFAULT" else float(v[5]),
                                        1.0 if v[6] == "DEFAULT" else float(v[6]),
                                        -1.0 if v[7] == "DEFAULT" else float(v[7]),
                                        0.0 if v[8] == "DEFAULT" else float(v[8]), "xyz".index(d)))
        elif key == "INCLUDE":
            name = next(lines)[0]
            if name.endswith("/"):
                raise ValueError(f"INCLUDE {name!r}: a '/' ends the line, so the file name cannot hold one")
            read_wells(os.path.join(workdir, name), workdir, wells)
    return wells


def well_perforations(wells: list, deck: GridDeck, grid, geo, conv_darcy: float = 0.008527, conv1: float = 1.0):
    """Per well the perforations the reference keeps and their indices, ready
    for the device's well set (ocpx_set_wells): a perforation whose cell is
    inactive or holds no pore space (pore fraction not above 1e-6) is dropped
    (ActiveGridCheck::IfFluid, src/PreParamGridWell.cpp:874-878); WI as
    PeacemanWell::CalWI forms it (src/WellPeaceman.cpp:277-361), including
    that a WI given in the deck is scaled by CONV1 at the well's first such
    perforation and the well's later perforations are left as read.
    Returns dicts with cell (active numbering), WI, kh, radius, skin and
    direction (0 x, 1 y, 2 z)."""
    n, A = deck.n, deck.arrays
    a2 = np.full(n, -1, np.int64)
    a2[geo["act2all"]] = np.arange(grid.nb)
    ntg = A.get("NTG")
    poro = np.asarray(A["PORO"], np.float64)
    if ntg is not None and len(ntg) == n:
        poro = poro * ntg
    out = []
    for w in wells:
        cells, perfs = [], []
        for (I, J, K, wi, diam, kh, skin, d) in w.perfs:
            c = (K - 1) * deck.nx * deck.ny + (J - 1) * deck.nx + (I - 1)
            if not (0 <= c < n) or a2[c] < 0 or not poro[c] > 1e-6:
                continue
            cells.append(int(a2[c]))
            perfs.append([wi, diam / 2.0, kh, skin, d])
        if not cells:
            raise ValueError(f"every perforation of well {w.name} is in an inactive cell")
        WI = np.array([p[0] for p in perfs])
        KH = np.array([p[2] for p in perfs])
        for q, (wi, radius, kh, skin, d) in enumerate(perfs):
            if wi > 0:
                WI[q] = wi * conv1
                break
            c = cells[q]
            WI[q], KH[q] = W.peaceman_index(d, geo["dx"][c], geo["dy"][c], geo["dz"][c], geo["ntg"][c], geo["kx"][c],
                                            geo["ky"][c], geo["kz"][c], radius, skin, kh, conv_darcy)
        out.append(dict(name=w.name, cell=np.array(cells, np.int32), WI=WI, kh=KH,
                        radius=np.array([p[1] for p in perfs]), skin=np.array([p[3] for p in perfs]),
                        direction=np.array([p[4] for p in perfs], np.int32)))
    return out


# ------------------------------------------------------------------ PROPS ---
UNITS = {
    # src/OCPUnits.cpp:17-56, include/OCPUnits.hpp:46-103 (CONV3 and CONV4 as the reference sets them)
    "METRIC": dict(GRAVITY_FACTOR=0.0000980665, CONV_DARCY=0.008527, GAS_CONSTANT=0.083143, CONV1=1.0, CONV3=1.0,
                   CONV4=273.15, RHOW_STD=999.014, RHOAIR_STD=1.2232),
    "FIELD": dict(GRAVITY_FACTOR=0.00694444, CONV_DARCY=0.001127 * 5.61458, GAS_CONSTANT=10.73159, CONV1=5.61458,
                  CONV3=1000 / 5.61458, CONV4=459.67, RHOW_STD=62.3664, RHOAIR_STD=0.076362),
}
TABLE_COLUMNS = {"SWOF": 4, "SGOF": 4, "PVCO": 6, "PVDG": 3, "PVTW": 5}
COMPONENT_ARRAYS = ("TCRIT", "PCRIT", "VCRIT", "ZCRIT", "MW", "ACF", "OMEGAA", "OMEGAB", "SSHIFT", "VCRITVIS")
LBC_DEFAULT = (0.1023, 0.023364, 0.058533, -0.040758, 0.0093324)   # ComponentParam::Init


def _stod(tok: str) -> float:
    """The leading number of a token, as std::stod reads it."""
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eEdD][+-]?\d+)?|\.\d+([eEdD][+-]?\d+)?)", tok)
    if not m:
        raise ValueError(f"not a number: {tok!r}")
    return float(m.group(0).replace("d", "e").replace("D", "e"))


def read_props(path: str, p: dict | None = None, workdir: str | None = None) -> dict:
    """The keywords of a deck that the device's Model needs, read as the
    reference's ParamRead::ReadFile dispatches them
    (src/ParamRead.cpp:60-360): units, the model (BLACKOIL / COMPS), the
    tables (ParamReservoir::InputTABLE), ROCK, DENSITY / GRAVITY, and the
    component data (ComponentParam: TCRIT ... VCRITVIS, LBCCOEF, BIC and the
    flash controls SSMSTA NRSTA SSMSP NRSP RR), and RTEMP for a PTN start.
    One PVT / saturation region."""
    p = dict(units="FIELD", blackoil=False, ncomp=0, tables={}, rock=None, density=None, gravity=None,
             comp={}, bic=None, lbc=list(LBC_DEFAULT), flash={}, rtemp=60.0) if p is None else p
    workdir = workdir if workdir is not None else os.path.dirname(os.path.abspath(path))
    lines = _lines(path)
    for toks in lines:
        key = toks[0]
        if key in ("FIELD", "METRIC"):
            p["units"] = key
        elif key in ("SPE11A", "SPE11Amg"):
            raise ValueError(f"unit system {key} is not read")
        elif key == "BLACKOIL":
            p["blackoil"] = True
        elif key in ("COMPS", "NCOMPS"):
            p["ncomp"] = int(next(lines)[0])
        elif key in TABLE_COLUMNS:
            ncol, rows, regions = TABLE_COLUMNS[key], [], []
            for t in lines:
                if t[0] == "/":
                    break
                rows.append([_stod(t[i]) for i in range(ncol)])
                if t[-1] == "/":
                    regions.append(rows)
                    rows = []
            if rows:
                regions.append(rows)
            if len(regions) != 1:
                raise ValueError(f"{key}: {len(regions)} regions; one region is read")
            p["tables"][key] = np.array(regions[0], np.float64)
        elif key == "ROCK":
            for t in lines:
                if t[0] == "/":
                    break
                if p["rock"] is not None:
                    raise ValueError("ROCK: more than one rock region")
                kind = t[0]
                if kind not in ("LINEAR01", "LINEAR02"):
                    raise ValueError(f"ROCK {kind}: only the linear rock models are read")
                cp1 = _stod(t[2])
                cp2 = 0.0
                if kind == "LINEAR02":
                    cp2 = _stod(t[3]) if len(t) > 3 and t[3] != "/" else cp1
                p["rock"] = (_stod(t[1]), cp1, cp2)
        elif key in ("DENSITY", "GRAVITY"):
            t = next(lines)
            if key == "GRAVITY":
                p["gravity"] = [45.5, 1.0, 0.7773]          # ParamReservoir::Init, active once the keyword appears
            if t[0] == "/":
                continue
            v = _defaults(t)
            v = v[:-1] if v[-1] == "/" else v
            if len(v) != 3:
                raise ValueError(f"{key} takes three values")
            if key == "GRAVITY":
                p["gravity"] = [p["gravity"][i] if v[i] == "DEFAULT" else _stod(v[i]) for i in range(3)]
            elif any(x != "DEFAULT" for x in v):
                base = p["density"] or [37.457, 62.366416, 0.062428]
                p["density"] = [base[i] if v[i] == "DEFAULT" else _stod(v[i]) for i in range(3)]
        elif key in COMPONENT_ARRAYS:
            vals = []
            for t in lines:
                if t[0] == "/":
                    break
                vals += [_stod(x) for x in t if x != "/"]
                if t[-1] == "/":
                    break
            n = p["ncomp"]
            if n <= 0:
                raise ValueError(f"{key} before the number of components")
            p["comp"][key] = np.array((vals + [0.0] * n)[:n], np.float64)
        elif key == "LBCCOEF":
            v = _defaults(next(lines))
            for i in range(5):
                if i < len(v) and v[i] not in ("DEFAULT", "/"):
                    p["lbc"][i] = _stod(v[i])
        elif key == "BIC":
            vals = []
            for t in lines:
                if t[0] == "/":
                    break
                vals += [_stod(x) for x in t if x != "/"]
                if t[-1] == "/":
                    break
            p["bic"] = np.array(vals, np.float64)
        elif key in ("SSMSTA", "NRSTA", "SSMSP", "NRSP", "RR"):
            p["flash"][key] = next(lines)
        elif key == "RTEMP":
            t = next(lines)              # ParamReservoir::InputRTEMP; 60 when not given
            if t[0] != "/":
                p["rtemp"] = _stod(t[0])
        elif key == "INCLUDE":
            name = next(lines)[0]
            if name.endswith("/"):
                raise ValueError(f"INCLUDE {name!r}: a '/' ends the line, so the file name cannot hold one")
            read_props(os.path.join(workdir, name), p, workdir)
    return p


def model_from_props(p: dict):
    """The device's Model as the reference sets it up from the read keywords
    (OCPMixtureMethodComp01 with EoS_PR, OCPPhaseEquilibrium::Setup and
    ViscosityMethod03, src/OCPMixtureMethodComp.cpp:650-668,
    src/OCPEoS.cpp:19-66, src/OCPPhaseEquilibrium.cpp:15-69,
    src/OCPFuncPVT.cpp:414-446; or the black-oil OGW01 mixture,
    src/OCPMixtureMethodK.cpp:418-436), in the arrays of a model dump."""
    from .fim import Model
    u = UNITS[p["units"]]
    R = u["GAS_CONSTANT"]
    a = {k: np.array([v]) for k, v in u.items() if k not in ("RHOW_STD", "RHOAIR_STD")}
    T = p["tables"]
    for name in ("SWOF", "SGOF", "PVTW"):
        if name not in T:
            raise ValueError(f"{name} is not given")
        a[name] = T[name].T.ravel().copy()
        a[name + "_nrow"] = np.array([T[name].shape[0]])
    pref, cp1, cp2 = p["rock"] if p["rock"] is not None else (14.7, 3.406e-6, 0.0)
    a.update(rock_Pref=np.array([pref]), rock_cp1=np.array([cp1]), rock_cp2=np.array([cp2]))
    if p["blackoil"]:
        for name in ("PVCO", "PVDG"):
            if name not in T:
                raise ValueError(f"{name} is not given (only the live-oil OGW black-oil model is read)")
            a[name] = T[name].T.ravel().copy()
            a[name + "_nrow"] = np.array([T[name].shape[0]])
        if p["density"] is not None:
            ro, rw, rg = p["density"]
        else:
            g = p["gravity"] or [45.5, 1.0, 0.7773]
            ro = (141.5 * u["RHOW_STD"]) / (g[0] + 131.5)
            rw = u["RHOW_STD"] * g[1]
            rg = u["RHOAIR_STD"] * g[2]
        a.update(mixture_comp=np.array([0]), nc=np.array([3]), stdRhoO=np.array([ro]), stdRhoG=np.array([rg]),
                 stdRhoW=np.array([rw]), stdVo=np.array([1.0]), stdVg=np.array([1.0]), stdVw=np.array([1.0]))
        return Model(a)
    n = p["ncomp"]
    C = p["comp"]
    for name in ("TCRIT", "PCRIT", "MW", "ACF"):
        if name not in C:
            raise ValueError(f"{name} is not given")
    Tc, Pc = C["TCRIT"], C["PCRIT"]
    if "VCRIT" in C:
        Vc = C["VCRIT"]
    elif "ZCRIT" in C:
        Vc = np.array([R * C["ZCRIT"][i] * Tc[i] / Pc[i] for i in range(n)])
    else:
        raise ValueError("VCRIT or ZCRIT is not given")
    oa = C.get("OMEGAA", np.full(n, 0.457235529))
    ob = C.get("OMEGAB", np.full(n, 0.077796074))
    bic = np.zeros(n * n)
    b = p["bic"] if p["bic"] is not None else np.zeros(0)
    if b.size == n * n:
        bic = b.copy()
    else:
        it = 0
        for i in range(1, n):
            for j in range(i):
                bic[i * n + j] = bic[j * n + i] = b[it] if it < b.size else 0.0
                it += 1
    if "SSHIFT" in C:
        vshift = np.array([C["SSHIFT"][i] * (R * ob[i] * Tc[i] / Pc[i]) for i in range(n)])
    else:
        vshift = np.zeros(n)
    if "VCRITVIS" in C:
        vcvis = C["VCRITVIS"]
    elif "VCRIT" in C:
        vcvis = C["VCRIT"]
    else:
        vcvis = np.array([10.73159 * C["ZCRIT"][i] * Tc[i] / Pc[i] for i in range(n)])
    F = p["flash"]
    for name in ("SSMSTA", "NRSTA", "SSMSP", "NRSP", "RR"):
        if name not in F:
            raise ValueError(f"flash control {name} is not given")
    ssm = F["SSMSTA"]
    flash = [int(ssm[0]), _stod(ssm[1]), _stod(ssm[2]), 1e-4, 1e-6,
             int(F["NRSTA"][0]), _stod(F["NRSTA"][1]), int(F["SSMSP"][0]), _stod(F["SSMSP"][1]),
             int(F["NRSP"][0]), _stod(F["NRSP"][1]), int(F["RR"][0]), _stod(F["RR"][1])]
    if p["gravity"] is not None:
        rhow = u["RHOW_STD"] * p["gravity"][1]
    if p["density"] is not None:
        rhow = u["RHOW_STD"]          # the reference's choice whenever DENSITY is given
    if p["gravity"] is None and p["density"] is None:
        raise ValueError("DENSITY or GRAVITY is not given")
    a.update(mixture_comp=np.array([1]), nc=np.array([n + 1]), NC=np.array([n]), Tc=Tc.copy(), Pc=Pc.copy(),
             Vc=np.asarray(Vc, np.float64), MWC=C["MW"].copy(), acf=C["ACF"].copy(), OmegaA=np.asarray(oa, np.float64),
             OmegaB=np.asarray(ob, np.float64), BIC=bic, Vshift=vshift, Vcvis=np.asarray(vcvis, np.float64),
             LBCcoef=np.array(p["lbc"]) * 10, flash_ctrl=np.array(flash, np.float64), stdRhoW=np.array([rhow]),
             stdVw=np.array([1.0]), skipPSA=np.array([1]))
    return Model(a)


def read_model(path: str):
    """The device's Model from a deck file (read_props, model_from_props)."""
    return model_from_props(read_props(path))


# ---------------------------------------------------------- initial state ---
def initial_state(deck: GridDeck, geo, model, rtemp: float = 60.0) -> dict:
    """The state a PTN start gives the active cells, as
    BulkInitializer::InitPTNi sets it (src/BulkInitializer.cpp:104-144):
    pressure, temperature (TEMPER, else RTEMP), the moles of each component
    from COMPM-0.. (water last) and the phase pressures from PHASEP-0..2,
    every phase absent.  With INITPTN1 the arrays list the active cells only
    (InitialReservoir::PostProcess).  The dict is ready for
    FimContext.load_state."""
    if deck.init not in ("INITPTN0", "INITPTN1"):
        raise ValueError("the deck has no PTN start (INITPTN0 or INITPTN1)")
    A, nb, nc = deck.arrays, len(geo["act2all"]), model.nc
    take = (lambda a: np.asarray(a, np.float64)[geo["act2all"]]) if deck.init == "INITPTN0" \
        else (lambda a: np.asarray(a, np.float64)[:nb])
    need = deck.n if deck.init == "INITPTN0" else nb

    def arr(name):
        a = A.get(name)
        if a is None or len(a) < need:
            raise ValueError(f"{name} must give {need} values")
        return take(a)

    comps = [f"COMPM-{i}" for i in range(10) if f"COMPM-{i}" in A]
    if len(comps) != nc:
        raise ValueError(f"{len(comps)} COMPM arrays for {nc} components")
    P = arr("PRESSURE")
    T = arr("TEMPER") if "TEMPER" in A else np.full(nb, float(rtemp))
    Ni = np.stack([arr(f"COMPM-{i}") for i in range(nc)], axis=1).ravel()
    Pj = np.stack([arr(f"PHASEP-{j}") for j in range(3)], axis=1).ravel()
    return dict(P=P, T=T, Ni=Ni, Pj=Pj, phaseExist=np.zeros(nb * 3, np.uint8))
