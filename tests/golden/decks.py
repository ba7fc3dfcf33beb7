"""Seeded synthetic input decks (ECL-style keywords, METRIC units) for the
reference simulator, used to generate the golden fixtures under tests/golden/.

Every deck is written from seeded random numbers only; no public benchmark
data is reproduced.  The same generator also returns the model description in
plain numpy form so CPU tests can rebuild the synthetic fluid without running
the reference.

Keyword formats follow the reference's parsers: grid keywords
(``src/PreParamGridWell.cpp:28-160``, ``INITPTN0``/``PRESSURE``/``COMPM-*``/
``PHASEP-*`` at ``:700-735``), fluid and rock tables
(``src/ParamReservoir.cpp``), component keywords (``TCRIT``/``PCRIT``/
``ZCRIT``/``MW``/``ACF``/``BIC``), and the flash-control keywords
``RR``/``SSMSTA``/``NRSTA``/``SSMSP``/``NRSP`` that the reference requires
without defaults (``src/OCPPhaseEquilibrium.cpp:45-64``).
"""
from __future__ import annotations

import numpy as np

# Flash controls: max iterations and tolerances of the stability SSM/NR,
# split SSM/NR and Rachford-Rice solves (same as the reference's SPE5 fluid).
FLASH_CONTROL = """RR
30 1e-12
/

SSMSTA
100 1e-12 1e-8
/

NRSTA
55 1e-12
/

SSMSP
100 1E-6
/

NRSP
55 1e-12
/
"""


def _fmt(vals, per_line=8):
    vals = list(vals)
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append(" ".join(f"{v:.17g}" for v in vals[i:i + per_line]))
    return "\n".join(lines)


def corey_tables(nrow=12, swc=0.2, sor=0.2, n=2.0):
    """SWOF and SGOF tables (columns S, kr_phase, kr_oil, Pc) tabulated from
    Corey curves with exponent ``n``; Pc is zero."""
    span = 1.0 - swc - sor
    sw = np.linspace(swc, 1.0, nrow)
    krw = np.clip((sw - swc) / span, 0, 1) ** n
    krow = np.clip((1.0 - sw - sor) / span, 0, 1) ** n
    swof = np.stack([sw, krw, krow, np.zeros(nrow)], axis=1)
    sg = np.linspace(0.0, 1.0 - swc, nrow)
    krg = np.clip(sg / span, 0, 1) ** n
    krog = np.clip((1.0 - swc - sor - sg) / span, 0, 1) ** n
    sgof = np.stack([sg, krg, krog, np.zeros(nrow)], axis=1)
    return swof, sgof


def blackoil_tables(nrow=12, pmin=10.0, pmax=400.0):
    """Monotone live-oil (PVCO: Pb, Rs, Bo, mu_o, Co, Cmu) and dry-gas (PVDG:
    P, Bg, mu_g) tables over ``pmin..pmax`` bar (1-40 MPa)."""
    p = np.linspace(pmin, pmax, nrow)
    rs = 2.0 + 0.45 * p                      # sm3/sm3
    bo = 1.02 + 0.0011 * rs                  # rm3/sm3
    muo = 1.6 / (1.0 + 0.004 * rs)           # cP
    co = np.full(nrow, 1.5e-4)               # 1/bar
    cmu = np.full(nrow, 4.0e-4)
    pvco = np.stack([p, rs, bo, muo, co, cmu], axis=1)
    bg = 1.01325 / p * (0.95 - 0.0006 * p) * 1.2
    mug = 0.012 + 5.0e-5 * p
    pvdg = np.stack([p, bg, mug], axis=1)
    return pvco, pvdg


def _grid_block(nx, ny, nz, dx, dy, dz_layers, tops, poro, kx, kz):
    n = nx * ny * nz
    dz = np.repeat(np.asarray(dz_layers, float), nx * ny)
    return f"""DIMENS
{nx} {ny} {nz} /

DX
{n}*{dx}
/
DY
{n}*{dy}
/
DZ
{_fmt(dz)}
/
TOPS
{nx * ny}*{tops}
/
PORO
{_fmt(poro)}
/
PERMX
{_fmt(kx)}
/
PERMY
{_fmt(kx)}
/
PERMZ
{_fmt(kz)}
/
"""


def blackoil_deck(seed=1, nx=10, ny=10, nz=3, tsteps=(1.0, 1.0, 2.0, 5.0, 10.0)):
    """Three-phase black-oil (live oil + dry gas + water) FIM deck: 10x10x3,
    dx=dy=300 m, dz=6/9/15 m, phi~U(0.15,0.30), lognormal kx (median 100 mD,
    sigma_ln 1), kz=0.1 kx, 12-row PVCO/PVDG over 1-40 MPa, Bw=1.01, Corey
    n=2 with Swc=Sor=0.2, gas injector at (1,1) on rate, BHP producer at
    (nx,ny), hydrostatic 20 MPa with Sw=0.2 (equilibration)."""
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    poro = rng.uniform(0.15, 0.30, n)
    kx = 100.0 * np.exp(rng.normal(0.0, 1.0, n))
    swof, sgof = corey_tables()
    pvco, pvdg = blackoil_tables()
    grid = _grid_block(nx, ny, nz, 300.0, 300.0, [6.0, 9.0, 15.0][:nz] if nz <= 3 else [10.0] * nz,
                       2000.0, poro, kx, 0.1 * kx)
    tstep = "\n".join(f"{t:g}" for t in tsteps)
    return f"""RUNSPEC
TITLE
 synthetic black-oil
MODEL
ISOTHERMAL
BLACKOIL
OIL
WATER
GAS
DISGAS
METRIC
TABDIMS
1 1 1
WELLDIMS
2 2 /

GRID
{grid}
PROPS

SWOF
{_fmt(swof.ravel(), 4)}
/

SGOF
{_fmt(sgof.ravel(), 4)}
/

PVCO
{_fmt(pvco.ravel(), 6)}
/

PVDG
{_fmt(pvdg.ravel(), 3)}
/

PVTW
200.0 1.01 4.5E-5 0.5 0.0 /
/

ROCK
LINEAR01 200.0 4.5E-5
/

DENSITY
850.0 1000.0 0.9 /

SOLUTION

EQUIL
2000.0 200.0 2500.0 0 1500.0 0 1 /

PBVD
1500.0 199.0
2500.0 199.0
/

SCHEDULE

TUNING
-- Init     max    min   incre   chop    cut
   1       10    0.1      5    0.3    0.3 /
--  dPlim  dSlim   dNlim   dVerrlim
   300     0.2    0.3    0.001 /
-- itNRmax  NRtol  dPmax  dSmax  dPmin   dSmin   dVerrmax
   20    1E-3   200    0.2    1E-0      1E-2    0.01 /
/

METHOD
FIM  dense
/

WELSPECS
'INJE1'   'G'   1   1     1*    'GAS'   /
'PROD1'   'G'   {nx}  {ny}    1*    'OIL'   /
/

COMPDAT
'INJE1'   2*   1   1     1*   0.2   3*   /
'PROD1'   2*   {nz}   {nz}     1*   0.2   3*   /
/

WCONINJE
'INJE1'   'GAS'   'OPEN'   'RATE'   200000.0      400.0    /
/

WCONPROD
'PROD1'   'OPEN'    'BHP'   DEFAULT     120.0    /
/

TSTEP
{tstep}
/

END
"""


def seeded_components(ncomp, seed):
    """Light-to-heavy pseudo-components with seeded Tc [K], Pc [bar], omega,
    MW, Zc and a symmetric BIC matrix in [0, 0.15] with zero diagonal."""
    rng = np.random.default_rng(seed)
    f = np.sort(rng.uniform(0.0, 1.0, ncomp))
    f[0] = 0.0
    tc = 190.0 + f * 610.0 + rng.uniform(-10, 10, ncomp)
    pc = 46.0 - f * 32.0 + rng.uniform(-1.5, 1.5, ncomp)
    acf = 0.01 + f * 0.9 + rng.uniform(0.0, 0.02, ncomp)
    mw = 16.0 + f * 300.0 + rng.uniform(0.0, 4.0, ncomp)
    zc = rng.uniform(0.24, 0.29, ncomp)
    bic = np.zeros((ncomp, ncomp))
    for i in range(ncomp):
        for j in range(i):
            bic[i, j] = bic[j, i] = rng.uniform(0.0, 0.15)
    return dict(Tc=tc, Pc=pc, acf=acf, MW=mw, Zc=zc, BIC=bic)


def _component_block(comp):
    nc = len(comp["Tc"])
    tri = []
    for i in range(1, nc):
        tri.append(" ".join(f"{comp['BIC'][i, j]:.17g}" for j in range(i)))
    return f"""NCOMPS
{nc}
/
CNAMES
{chr(10).join(f'C{i + 1}' for i in range(nc))}
/
TCRIT
{_fmt(comp['Tc'], 1)}
/
PCRIT
{_fmt(comp['Pc'], 1)}
/
ZCRIT
{_fmt(comp['Zc'], 1)}
/
MW
{_fmt(comp['MW'], 1)}
/
ACF
{_fmt(comp['acf'], 1)}
/
BIC
{chr(10).join(tri)} /

{FLASH_CONTROL}"""


def comp_cells(nx, ny, nz, ncomp, seed, porosity=0.2, dxy=20.0, dz=5.0,
               p_range=(100.0, 300.0), alpha=2.0, temp_k=345.0, smooth=False):
    """Per-cell pressure [bar] and component moles (hydrocarbons then water)
    for a PTN initialisation: z ~ Dirichlet(alpha), P ~ U(p_range) per cell
    (or, with ``smooth``, a linear ramp over x across p_range plus +-1 bar of
    noise, which keeps multi-step Newton runs well posed), Sw ~ 0.2;
    hydrocarbon moles fill 80 % of the pore volume at an assumed Z = 0.6."""
    rng = np.random.default_rng(seed + 1000)
    n = nx * ny * nz
    p = rng.uniform(*p_range, n)
    if smooth:
        ix = np.arange(n) % nx
        p = p_range[0] + (p_range[1] - p_range[0]) * ix / max(nx - 1, 1) + rng.uniform(-1, 1, n)
    z = rng.dirichlet(np.full(ncomp, alpha), n)
    vp = dxy * dxy * dz * porosity
    vm = 0.6 * 0.083143 * temp_k / p          # m3/kmol
    nt = 0.8 * vp / vm
    ni = z * nt[:, None]
    nw = np.full(n, 0.2 * vp / 1.01)          # water "moles" = std m3 for METRIC PVTW
    return p, np.concatenate([ni, nw[:, None]], axis=1)


def corner_grid_block(nx, ny, nz, coord, zcorn, poro, kx, ky, kz):
    """DIMENS + COORD/ZCORN (Eclipse order) + rock arrays of a corner-point grid."""
    return f"""DIMENS
{nx} {ny} {nz} /

COORD
{_fmt(coord)}
/
ZCORN
{_fmt(zcorn)}
/
PORO
{_fmt(poro)}
/
PERMX
{_fmt(kx)}
/
PERMY
{_fmt(ky)}
/
PERMZ
{_fmt(kz)}
/
"""


def comp_deck(nx, ny, nz, ncomp, seed, perm=50.0, porosity=0.2, dxy=20.0, dz=5.0,
              temp_k=345.0, p_range=(100.0, 300.0), alpha=2.0, tsteps=(0.01, 0.01),
              wells=True, smooth=False, grid_text=None):
    """Compositional PR-EoS FIM deck with a PTN (pressure + moles) start.

    Returns ``(deck_text, ni)``: the per-cell moles ``ni`` (cells x (ncomp+1),
    water last) go into the side file ``<deck>.ptn_ni`` (raw float64) because
    the reference's grid distributor accepts at most 30 per-cell arrays
    (``src/Reservoir.cpp:38-66``), too few for ``COMPM-*`` with more than four
    hydrocarbon components."""
    comp = seeded_components(ncomp, seed)
    n = nx * ny * nz
    p, ni = comp_cells(nx, ny, nz, ncomp, seed, porosity, dxy, dz, p_range, alpha, temp_k, smooth)
    swof, sgof = corey_tables()
    grid = grid_text or _grid_block(nx, ny, nz, dxy, dxy, [dz] * nz, 2000.0, np.full(n, porosity),
                                    np.full(n, perm), np.full(n, perm))
    init = ["INITPTN0", "PRESSURE", _fmt(p), "/"]
    for j in range(3):
        init += [f"PHASEP-{j}", _fmt(p), "/"]
    # the deck reader insists on at least one COMPM-* array; the harness
    # replaces the whole set with the side file
    init += ["COMPM-0", _fmt(ni[:, 0]), "/"]
    inj = " ".join(["0.0"] * ncomp)
    inj = " ".join(["1.0"] + ["0.0"] * (ncomp - 1))
    well_text = f"""WELSPECS
'INJE1'   'G'   1   1     1*    'GAS'   /
'PROD1'   'G'   {nx}  {ny}    1*    'OIL'   /
/

COMPDAT
'INJE1'   2*   1   {nz}     1*   0.2   3*   /
'PROD1'   2*   1   {nz}     1*   0.2   3*   /
/

WELLSTRE
Solvent {inj} /
/

WCONINJE
'INJE1'   'Solvent'   'OPEN'   'RATE'   1000.0      400.0    /
/

WCONPROD
'PROD1'   'OPEN'    'BHP'   DEFAULT     90.0    /
/
""" if wells else ""
    tstep = "\n".join(f"{t:g}" for t in tsteps)
    return ni, f"""RUNSPEC
TITLE
 synthetic compositional
MODEL
ISOTHERMAL
COMPS
{ncomp}
/
OIL
WATER
GAS
METRIC
TABDIMS
1 1 1
WELLDIMS
2 2 /

GRID
{grid}
{chr(10).join(init)}

PROPS
{_component_block(comp)}
RTEMP
{temp_k - 273.15:.17g}
/

SWOF
{_fmt(swof.ravel(), 4)}
/

SGOF
{_fmt(sgof.ravel(), 4)}
/

PVTW
200.0 1.01 4.5E-5 0.5 0.0 /
/

ROCK
LINEAR01 200.0 4.5E-5
/

DENSITY
850.0 1000.0 0.9 /

SCHEDULE

TUNING
-- Init     max    min   incre   chop    cut
   0.01       10    0.001      5    0.3    0.3 /
--  dPlim  dSlim   dNlim   dVerrlim
   300     0.2    0.3    0.001 /
-- itNRmax  NRtol  dPmax  dSmax  dPmin   dSmin   dVerrmax
   20    1E-3   200    0.2    1E-0      1E-2    0.01 /
/

METHOD
FIM  dense
/

{well_text}
TSTEP
{tstep}
/

END
"""
