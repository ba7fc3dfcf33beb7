"""Host-side set-up of Peaceman wells for the device step (ocpx_set_wells).

The reference computes each perforation's well index once, at well set-up
(PeacemanWell::CalWI, src/WellPeaceman.cpp:277-361): Peaceman's equivalent
radius of the perforated cell,

    r_o = 0.28 sqrt(l1^2 sqrt(b/a) + l2^2 sqrt(a/b)) / ((a/b)^(1/4) + (b/a)^(1/4)),
    WI  = 2 pi k h / (ln(r_o / r_w) + skin) * CONV_DARCY,

with (a, b, l1, l2) the permeabilities and sizes across the perforation's
direction and k h = length * sqrt(a b).  ``peaceman_wi`` evaluates it for
arrays of perforations.

``vertical_wells`` lays out the wells of the seeded synthetic workloads:
vertical wells through every layer of a structured grid, injectors of the
lightest hydrocarbon component under bottom-hole-pressure control and
producers under bottom-hole-pressure or total-hydrocarbon-rate control.
Two quantities the reference derives from its PVT at run time are set by a
stated rule instead: the wellbore's hydrostatic head dG = rho g (depth -
depth of the top perforation) with a fixed wellbore density per well type,
and the injected fluid's molar density P / (Z R T) at the bottom-hole
pressure with Z = 0.9.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.141592653  # include/OCPConst.hpp:32: the reference's pi, which its well index uses


def peaceman_index(direction, dx, dy, dz, ntg, kx, ky, kz, radius, skin=0.0, kh=-1.0, conv_darcy=0.008527):
    """Well index and kh of one perforation along x (0), y (1) or z (2) whose
    WI is not given, as PeacemanWell::CalWI forms them
    (src/WellPeaceman.cpp:277-361): the layer thickness dz * NTG, kh from the
    cell when kh < 0, pow and log from the C library (math), in the
    reference's order of operations.  Returns (WI, kh)."""
    dz = dz * ntg
    if direction == 0:
        a, b, l1, l2, length = ky, kz, dy, dz, dx
    elif direction == 1:
        a, b, l1, l2, length = kz, kx, dz, dx, dy
    elif direction == 2:
        a, b, l1, l2, length = kx, ky, dx, dy, dz
    else:
        raise ValueError("direction must be 0, 1 or 2")
    ab, a_b = a * b, a / b
    ro = 0.28 * math.pow(l1 * l1 * math.pow(1 / a_b, 0.5) + l2 * l2 * math.pow(a_b, 0.5), 0.5)
    ro /= math.pow(a_b, 0.25) + math.pow(1 / a_b, 0.25)
    if kh < 0:
        kh = length * math.pow(ab, 0.5)
    wi = (2 * PI) * kh / (math.log(ro / radius) + skin)
    return wi * conv_darcy, kh


def peaceman_wi(direction, dx, dy, dz, kx, ky, kz, ntg=1.0, radius=0.1, skin=0.0, conv_darcy=0.008527):
    """Well index of perforations along x (0), y (1) or z (2) (arrays or
    scalars; kh derived from the cell), perforation by perforation with
    peaceman_index."""
    if direction not in (0, 1, 2):
        raise ValueError("direction must be 0, 1 or 2")
    args = np.broadcast_arrays(*(np.asarray(v, np.float64) for v in (dx, dy, dz, ntg, kx, ky, kz, radius, skin)))
    out = np.empty(args[0].shape)
    for i in np.ndindex(out.shape):
        v = [float(a[i]) for a in args]
        out[i] = peaceman_index(direction, *v[:8], skin=v[8], conv_darcy=conv_darcy)[0]
    return out[()] if out.ndim == 0 else out


def vertical_wells(nx, ny, nz, n_inj, n_prod, dxy, dz, perm_x, perm_z, depth, ncomp, seed, temp_c=71.85,
                   bhp_inj=320.0, bhp_prod=90.0, n_rate=0, rate=50.0, gravity_factor=0.0000980665,
                   gas_constant=0.083143, corners=False):
    """Wells of a synthetic nx * ny * nz grid (cells (k, j, i), i fastest;
    perm_x, perm_z and depth per cell): n_inj injectors and n_prod producers
    through every layer at seeded distinct columns (corners=True: the first
    injector at column (0, 0) and the first producer at (nx-1, ny-1)).
    Injectors inject the lightest component at bhp_inj; the last n_rate
    producers hold a total hydrocarbon rate `rate` (mol/day), the others
    bhp_prod.  Returns dicts for FimContext.set_wells (ncomp hydrocarbon
    components plus water)."""
    rng = np.random.default_rng(seed + 4000)
    n = n_inj + n_prod
    if corners:
        rest = np.setdiff1d(rng.permutation(nx * ny), [0, nx * ny - 1])
        cols = np.r_[0, rest[:n_inj - 1], nx * ny - 1, rest[n_inj - 1:n - 2]]
    else:
        cols = rng.choice(nx * ny, size=n, replace=False)
    nc = ncomp + 1
    wells = []
    for w, col in enumerate(cols):
        cells = col + nx * ny * np.arange(nz)
        kx, kz = np.asarray(perm_x)[cells], np.asarray(perm_z)[cells]
        WI = peaceman_wi(2, dxy, dxy, dz, kx, kx, kz)
        d = np.asarray(depth)[cells]
        inj = w < n_inj
        rho = 200.0 if inj else 700.0   # wellbore density of the hydrostatic head (kg/m3)
        dG = rho * gravity_factor * (d - d[0])
        bhp = bhp_inj if inj else bhp_prod
        zi = np.zeros(nc)
        zi[0] = 1.0
        factor = np.r_[np.ones(ncomp), 0.0]
        xi = (bhp + dG) / (0.9 * gas_constant * (temp_c + 273.15))
        rate_w = (not inj) and (w >= n - n_rate)
        wells.append(dict(type=0 if inj else 1, mode=1 if rate_w else 0, bhp=bhp, tar_bhp=bhp,
                          tar_rate=rate if rate_w else 0.0, cell=cells.astype(np.int32), WI=WI, dG=dG,
                          xi_inj=xi if inj else np.zeros(nz), inj_zi=zi, factor=factor))
    return wells
