"""The GRID section of an ECL-style input deck, read as the reference reads it
(PreParamGridWell::InputFile, src/PreParamGridWell.cpp:25-150), and the grid
the reference builds from it (PreParamGridWell::Setup, :876-1020): the cells
that stay active, their geometry and the connections between them, ready for
ocpx_create.

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

REAL_ARRAYS = ("DX", "DY", "DZ", "TOPS", "COORD", "ZCORN", "NTG", "PORO", "PERMX", "PERMY", "PERMZ", "MULTZ")
INT_ARRAYS = ("ACTNUM",)


@dataclass
class GridDeck:
    """The GRID-section input of a deck: dimensions and arrays as read, in
    the reference's cell order (i fastest, then j, then k)."""
    nx: int = 0
    ny: int = 0
    nz: int = 0
    arrays: dict = field(default_factory=dict)

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


def _box_index(box, nx, ny, tops=False):
    i0, i1, j0, j1, k0, k1 = box
    if tops:
        k0 = k1 = 0
    if min(i0, j0, k0) < 0:
        raise ValueError(f"box {box} out of range")
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
        elif key in REAL_ARRAYS or key in INT_ARRAYS:
            cast = int if key in INT_ARRAYS else float
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
                idx = _box_index(_box(t[2:], deck.nx, deck.ny, deck.nz), deck.nx, deck.ny, name == "TOPS")
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
                idx = _box_index(_box(t[2:], deck.nx, deck.ny, deck.nz), deck.nx, deck.ny)
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
