"""Seeded synthetic workloads (fluids, grids, initial states) for the bench
and the large-size tests, built without the reference.

The fluid description is what the reference's setup produces from an
ECL-style deck in METRIC units with TCRIT/PCRIT/ZCRIT/MW/ACF/BIC and the
flash-control keywords (ComponentParam, src/ParamReservoir.cpp:710-719;
EoS_PR, src/OCPEoS.cpp:19-66; OCPPhaseEquilibrium::Setup,
src/OCPPhaseEquilibrium.cpp:15-69; ViscosityMethod03,
src/OCPFuncPVT.cpp:415-460; OCPMixtureMethodComp01,
src/OCPMixtureMethodComp.cpp:650-668), including two of its quirks:
Vc = GAS_CONSTANT * Zc * Tc / Pc for the phase test, but the LBC critical
volume falls back to 10.73159 * Zc * Tc / Pc (the FIELD gas constant), and the
standard water density is RHOW_STD whenever DENSITY is given.
tests/test_synthetic.py checks these arrays against the reference's own dump.
"""
from __future__ import annotations

import numpy as np

from .fim import Model
from .grid import orthogonal_grid

# METRIC unit constants (src/OCPUnits.cpp:37-55, include/OCPUnits.hpp:80-101)
METRIC = dict(GRAVITY_FACTOR=0.0000980665, CONV_DARCY=0.008527, GAS_CONSTANT=0.083143, CONV1=1.0, CONV3=1.0,
              CONV4=273.15)
RHOW_STD_METRIC = 999.014
# flash controls used by the synthetic decks: SSMsta (maxIt, tol, eYt, Ktol, dYtol), NRsta (maxIt, tol),
# SSMsp (maxIt, tol), NRsp (maxIt, tol), RR (maxIt, tol); Ktol and dYtol are the reference's fixed values
FLASH_CTRL = [100, 1e-12, 1e-8, 1e-4, 1e-6, 55, 1e-12, 100, 1e-6, 55, 1e-12, 30, 1e-12]
LBC_DEFAULT = [0.1023, 0.023364, 0.058533, -0.040758, 0.0093324]


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


def corey_tables(nrow=12, swc=0.2, sor=0.2, n=2.0):
    """SWOF and SGOF (S, kr_phase, kr_oil, Pc) tabulated from Corey curves."""
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


def comp_model(ncomp, seed, pvtw=(200.0, 1.01, 4.5e-5, 0.5, 0.0), rock=(200.0, 4.5e-5, 0.0)) -> Model:
    """PR-EoS fluid + water + Corey kr, as the reference sets it up."""
    c = seeded_components(ncomp, seed)
    R = METRIC["GAS_CONSTANT"]
    swof, sgof = corey_tables()
    a = dict(METRIC)
    a.update(mixture_comp=np.array([1]), nc=np.array([ncomp + 1]), NC=np.array([ncomp]),
             Tc=c["Tc"], Pc=c["Pc"], MWC=c["MW"], acf=c["acf"],
             Vc=R * c["Zc"] * c["Tc"] / c["Pc"], Vcvis=10.73159 * c["Zc"] * c["Tc"] / c["Pc"],
             OmegaA=np.full(ncomp, 0.457235529), OmegaB=np.full(ncomp, 0.077796074), Vshift=np.zeros(ncomp),
             BIC=c["BIC"].ravel(), LBCcoef=np.array(LBC_DEFAULT) * 10, flash_ctrl=np.array(FLASH_CTRL, float),
             PVTW=np.array(pvtw, float), PVTW_nrow=np.array([1]), stdRhoW=np.array([RHOW_STD_METRIC]),
             stdVw=np.array([1.0]), SWOF=swof.T.ravel().copy(), SWOF_nrow=np.array([swof.shape[0]]),
             SGOF=sgof.T.ravel().copy(), SGOF_nrow=np.array([sgof.shape[0]]), rock_Pref=np.array([rock[0]]),
             rock_cp1=np.array([rock[1]]), rock_cp2=np.array([rock[2]]), skipPSA=np.array([1]))
    for k in METRIC:
        a[k] = np.array([METRIC[k]])
    return Model(a)


def comp_initial_state(grid, ncomp, seed, p_range=(100.0, 300.0), alpha=2.0, temp_c=71.85, smooth=False, nx=None,
                       n_total=None, first=0):
    """PTN start: per-cell pressure and moles (hydrocarbons then water) with
    z ~ Dirichlet(alpha), P ~ U(p_range); hydrocarbons fill 80 % of the pore
    volume at an assumed Z = 0.6 and water 20 % (Bw ~ 1.01).  Phase state is
    empty, as BulkInitializer::InitPTNi leaves it (src/BulkInitializer.cpp:104-143).
    With n_total, grid holds the cells [first, first + grid.nb) of a grid of
    n_total cells, and gets the values those cells have there."""
    rng = np.random.default_rng(seed + 1000)
    n = grid.nb
    nd = n if n_total is None else n_total
    p = rng.uniform(*p_range, nd)
    if smooth:
        ix = np.arange(nd) % nx
        p = p_range[0] + (p_range[1] - p_range[0]) * ix / max(nx - 1, 1) + rng.uniform(-1, 1, nd)
    z = rng.dirichlet(np.full(ncomp, alpha), nd)
    p, z = p[first:first + n], z[first:first + n]
    vp = grid.v * grid.poro_init
    vm = 0.6 * METRIC["GAS_CONSTANT"] * (temp_c + 273.15) / p
    ni = z * (0.8 * vp / vm)[:, None]
    nw = 0.2 * vp / 1.01
    Ni = np.concatenate([ni, nw[:, None]], axis=1)
    return dict(P=p, T=np.full(n, temp_c), Ni=Ni.ravel(), Pj=np.repeat(p, 3), phaseExist=np.zeros(3 * n, np.uint8),
                S=np.zeros(3 * n), xij=np.zeros(3 * n * (ncomp + 1)), lNi=Ni.ravel().copy(),
                Nt=Ni.sum(axis=1))


def comp_grid(nx, ny, nz, dxy=20.0, dz=5.0, perm=50.0, poro=0.2, tops=2000.0):
    n = nx * ny * nz
    return orthogonal_grid(nx, ny, nz, dxy, dxy, dz, tops, np.full(n, perm), np.full(n, perm), np.full(n, perm),
                           np.full(n, poro), conv_darcy=METRIC["CONV_DARCY"])


def layered_lognormal_perm(nx, ny, nz, median, sigma_ln, corr_cells, seed):
    """Layered lognormal permeability [mD]: a seeded standard-normal field
    smoothed in x and y by a Gaussian filter of standard deviation
    corr_cells / 2 (cells), rescaled to unit variance per layer, then
    k = median * exp(sigma_ln * g).  Cell order (k, j, i), x fastest."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((nz, ny, nx))
    for k in range(nz):
        layer = gaussian_filter(g[k], sigma=corr_cells / 2.0, mode="wrap")
        g[k] = (layer - layer.mean()) / max(layer.std(), 1e-12)
    return (median * np.exp(sigma_ln * g)).ravel()


def comp_grid_lognormal(nx, ny, nz, median=200.0, sigma_ln=1.5, corr_cells=10, seed=0, dxy=20.0, dz=5.0,
                        poro=0.2, tops=2000.0, kz_ratio=0.1):
    """Orthogonal grid with layered lognormal permeability (kz = kz_ratio kx)."""
    k = layered_lognormal_perm(nx, ny, nz, median, sigma_ln, corr_cells, seed)
    n = nx * ny * nz
    return orthogonal_grid(nx, ny, nz, dxy, dxy, dz, tops, k, k, kz_ratio * k, np.full(n, poro),
                           conv_darcy=METRIC["CONV_DARCY"])


def ptn_workload(ctx, grid, ncomp, seed, dt=0.1, dsmax=0.2, p_range=(100.0, 300.0), slot_before_last=None):
    """Drive a context to the input of the second Newton iteration of a time
    step from a seeded PTN start (pores filled by scaling the moles), as the
    bench does; returns the two seeded Newton updates (u1 applied, u2 the one
    that produced the returned state).  slot_before_last: a checkpoint slot
    that receives the state just before u2 is applied (the input of a whole
    Newton iteration, update included), or None."""
    st = comp_initial_state(grid, ncomp, seed, p_range=p_range)
    ctx.load_state(st)
    ctx.update_property()
    scale = ctx.get("ROCKVP") / ctx.get("VF")
    Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    ctx.load_state(st)
    ctx.set("SKIP_FLAG", np.zeros(grid.nb, np.uint8))
    ctx.update_property()
    ctx.cal_res(dt)
    ctx.update_last_time_step()
    us = ptn_updates(Ni, grid.nb, ncomp, seed)
    ctx.get_solution(us[0], dsmax)
    ctx.update_property()
    ctx.cal_res(dt)
    if slot_before_last is not None:
        ctx.checkpoint(slot_before_last)
    ctx.get_solution(us[1], dsmax)
    return us


def ptn_updates(Ni, nb, ncomp, seed, n_total=None, first=0):
    """The two seeded Newton updates of ptn_workload (dP ~ N(0, 2) bar, dNi =
    Ni N(0, 2e-3)) for cells with moles Ni; with n_total, the cells are
    [first, first + nb) of a grid of n_total cells and get the draws those
    cells have there."""
    nd = nb if n_total is None else n_total
    us = []
    for k in range(2):
        rng = np.random.default_rng(seed + 77 + k)
        dp = rng.normal(0.0, 2.0, nd)[first:first + nb]
        dn = rng.normal(0.0, 2e-3, (nd, ncomp + 1))[first:first + nb]
        u = np.zeros((nb, ncomp + 2))
        u[:, 0] = dp
        u[:, 1:] = np.asarray(Ni).reshape(nb, -1) * dn
        us.append(u.ravel())
    return us


def flash_grid(n, poro=0.2):
    """n independent unit-volume cells without connections (flash-only runs)."""
    from .fim import Grid
    return Grid(np.ones(n), np.zeros(n), np.full(n, poro), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                np.zeros(0))


def flash_state(P, Ni, temp_c):
    """State of independent cells flashed with no phase history (only the water
    phase flagged, so lNP = 0 and the phase equilibrium starts with the full
    four-start stability test, as the reference's InitFlash does)."""
    n = P.size
    nct = Ni.shape[1]
    return dict(P=P.copy(), T=np.full(n, temp_c), Ni=Ni.ravel().copy(), lNi=Ni.ravel().copy(),
                Nt=Ni.sum(axis=1), phaseExist=np.tile(np.array([0, 0, 1], np.uint8), n),
                S=np.tile([0.0, 0.0, 1.0], n), xij=np.zeros(n * 3 * nct), Pj=np.repeat(P, 3),
                skip_flag=np.zeros(n, np.uint8))


def flash_stress_cells(ctx_factory, n, ncomp, seed, near_frac=0.2, p_range=(50.0, 400.0), near_band=0.05,
                       temp_c=71.85, bisections=30):
    """Inputs of the batched-flash stress case: n independent cells with
    ncomp seeded components.  A fraction near_frac of the cells lie within
    +-near_band of their saturation pressure, found by bisection between a
    two-phase and a single-phase pressure of the seeded fluid's envelope
    (evaluated with the GPU flash itself); the others have P ~ U(p_range)
    and z ~ Dirichlet(1.5).  Returns (P [bar], Ni [n, ncomp+1])."""
    rng = np.random.default_rng(seed + 2000)
    z = rng.dirichlet(np.full(ncomp, 1.5), n)
    Ni = np.concatenate([z * 10.0, np.ones((n, 1))], axis=1)
    P = rng.uniform(*p_range, n)
    near = rng.random(n) < near_frac
    idx = np.nonzero(near)[0]
    if idx.size:
        sub = Ni[idx]
        ctx = ctx_factory(flash_grid(idx.size))
        try:
            def two_phase(p):
                ctx.load_state(flash_state(p, sub, temp_c))
                ctx.update_property()
                pe = ctx.get("PHASE_EXIST").reshape(-1, 3)
                return (pe[:, 0] != 0) & (pe[:, 1] != 0)
            lo = np.full(idx.size, p_range[0])
            hi = np.full(idx.size, p_range[1])
            tl, th = two_phase(lo), two_phase(hi)
            ok = tl != th           # a phase boundary inside the range
            for _ in range(bisections):
                mid = 0.5 * (lo + hi)
                tm = two_phase(mid)
                same = tm == tl
                lo = np.where(same, mid, lo)
                hi = np.where(same, hi, mid)
            psat = 0.5 * (lo + hi)
            band = rng.uniform(-near_band, near_band, idx.size)
            P[idx] = np.where(ok, psat * (1 + band), P[idx])
        finally:
            ctx.close()
    return P, Ni


def dipping_corner_point(nx, ny, nz, dxy, dz, top, dip_x_deg, dip_y_deg, pillar_tilt=0.0, seed=0,
                         pillar_jitter=0.0):
    """A corner-point grid (Eclipse COORD and ZCORN arrays) of nz layers of
    thickness dz over an nx x ny plan with spacing dxy, its top dipping by
    dip_x_deg / dip_y_deg.  Each pillar leans by a seeded slope within
    +-pillar_tilt in x and y (non-vertical pillars), and its top and bottom
    points are moved, independently, by seeded offsets within
    +-pillar_jitter * dxy in x and y, so every point of a pillar lies within
    that distance of its unperturbed place when pillar_tilt is 0.  Layer
    boundaries are shared by neighbouring cells, so faces match (no faults)."""
    rng = np.random.default_rng(seed)
    X = np.arange(nx + 1) * float(dxy)
    Y = np.arange(ny + 1) * float(dxy)
    XX, YY = np.meshgrid(X, Y)                     # [J][I]
    ztop = top + np.tan(np.deg2rad(dip_x_deg)) * XX + np.tan(np.deg2rad(dip_y_deg)) * YY
    zbot = ztop + nz * dz + 10.0
    sx = rng.uniform(-pillar_tilt, pillar_tilt, XX.shape)
    sy = rng.uniform(-pillar_tilt, pillar_tilt, XX.shape)
    coord = np.empty((ny + 1, nx + 1, 2, 3))
    coord[:, :, 0, 0], coord[:, :, 0, 1], coord[:, :, 0, 2] = XX, YY, ztop
    coord[:, :, 1, 0] = XX + sx * (zbot - ztop)
    coord[:, :, 1, 1] = YY + sy * (zbot - ztop)
    coord[:, :, 1, 2] = zbot
    if pillar_jitter:
        j = rng.uniform(-pillar_jitter, pillar_jitter, (2, 2) + XX.shape) * float(dxy)
        coord[:, :, 0, 0] += j[0, 0]
        coord[:, :, 0, 1] += j[0, 1]
        coord[:, :, 1, 0] += j[1, 0]
        coord[:, :, 1, 1] += j[1, 1]
    zb = ztop[None, :, :] + dz * np.arange(nz + 1)[:, None, None]   # [K][J][I] layer boundaries
    zc = np.empty((nz, 2, ny, 2, nx, 2))
    for tb in range(2):
        for fb in range(2):
            for lr in range(2):
                zc[:, tb, :, fb, :, lr] = zb[tb:nz + tb, fb:ny + fb, lr:nx + lr]
    return coord.ravel(), zc.ravel()


def faulted_corner_point(nx, ny, nz, dxy, dz, top, dip_x_deg, dip_y_deg, faults, pillar_tilt=0.0, seed=0):
    """The grid of dipping_corner_point cut by vertical faults on its pillar
    lines.  Each fault is (axis, index, throw_start, throw_end[, stretch]):
    for axis "x" the cells with I > index move down by a throw that varies
    linearly along the fault, from throw_start at its first pillar (J = 0) to
    throw_end at its last (J = ny), and their layers are `stretch` times as
    thick (default 1); for axis "y" the cells with J > index, the throw
    varying along I.  A throw that changes sign along the fault (a scissor
    fault) or a change of thickness across it makes the faces on it overlap
    in shapes other than quadrilaterals; a throw larger than dz makes
    non-neighbour connections."""
    coord, zc = dipping_corner_point(nx, ny, nz, dxy, dz, top, dip_x_deg, dip_y_deg, pillar_tilt, seed)
    z = zc.reshape(nz, 2, ny, 2, nx, 2)              # [K][top/bottom][J][y-/y+][I][x-/x+]
    for fault in faults:
        axis, index, t0, t1 = fault[:4]
        stretch = fault[4] if len(fault) > 4 else 1.0
        if axis == "x":
            pj = np.arange(ny)[:, None] + np.arange(2)[None, :]          # pillar J of each corner
            side = (slice(None), slice(None), slice(None), slice(None), slice(index + 1, None), slice(None))
            throw = (t0 + (t1 - t0) * pj / ny)[None, None, :, :, None, None]
        elif axis == "y":
            pi = np.arange(nx)[:, None] + np.arange(2)[None, :]
            side = (slice(None), slice(None), slice(index + 1, None), slice(None), slice(None), slice(None))
            throw = (t0 + (t1 - t0) * pi / nx)[None, None, None, None, :, :]
        else:
            raise ValueError("fault axis must be 'x' or 'y'")
        zs = z[side]
        z[side] = zs[:1, :1] + stretch * (zs - zs[:1, :1]) + throw
    return coord, z.ravel()
