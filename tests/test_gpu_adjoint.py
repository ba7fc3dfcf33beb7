"""Adjoint vector-Jacobian products (ocpx_adjoint) on the GPU.

* J^T lambda against the transpose of the reference's own assembled Jacobian
  (golden fixtures) and of the library's Jacobian;
* (dR/dT)^T lambda and (dR/dporoInit)^T lambda against central finite
  differences of the GPU residual, relative step 1e-6, on seeded entries.
  The residual is linear in both parameters, so the differences are exact up
  to rounding; the bar is 1e-6 relative.
"""
import numpy as np
import pytest

import parity as P
from opencaeporox_gb300 import fim

pytestmark = pytest.mark.gpu

FD_STEP = 1e-6
FD_TOL = 1e-6


def bcsr_transpose_product(rowptr, col, val, lam, nb, dim):
    """y_c = sum_r B_rc^T lam_r for a block-CSR matrix with (dim x dim) row-major blocks."""
    y = np.zeros((nb, dim))
    L = lam.reshape(nb, dim)
    B = val.reshape(-1, dim, dim)
    for r in range(nb):
        for k in range(rowptr[r], rowptr[r + 1]):
            y[col[k]] += B[k].T @ L[r]
    return y.ravel()


@pytest.mark.parametrize("name", ["bo_10x10x3", "comp6_8x8x3", "comp8_6x6x4"])
def test_jt_lambda_against_transposed_jacobians(gpu_lib, name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    dim = model.nc + 1
    rng = np.random.default_rng(11)
    with fim.FimContext(model, grid) as ctx:
        for it in P.iterations(fx)[:2]:
            js = P.jac_state(fx, it)
            dt = float(js["dt"][0])
            ctx.load_state(js)
            ctx.cal_res(dt)
            ctx.assemble_mat(dt)
            lam = rng.normal(size=grid.nb * dim)
            jt, _, _ = ctx.adjoint(lam, trans=False, poro=False)
            rp, col, val = ctx.jacobian()
            own = bcsr_transpose_product(rp, col, val, lam, grid.nb, dim)
            ref = bcsr_transpose_product(js["jac_rowptr"], js["jac_col"], js["jac_val"], lam, grid.nb, dim)
            scale = np.linalg.norm(ref)
            assert np.linalg.norm(jt - own) <= 1e-13 * np.linalg.norm(own), it
            assert np.linalg.norm(jt - ref) <= P.REL_TOL * scale, (it, np.linalg.norm(jt - ref) / scale)


def _residual(ctx, dt):
    ctx.cal_res(dt)
    return ctx.get("RES")


@pytest.mark.parametrize("name", ["comp6_8x8x3", "bo_10x10x3"])
def test_dr_dtrans_against_central_differences(gpu_lib, name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    dim = model.nc + 1
    it = P.iterations(fx)[0]
    js = P.jac_state(fx, it)
    dt = float(js["dt"][0])
    rng = np.random.default_rng(12)
    lam = rng.normal(size=grid.nb * dim)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(js)
        ctx.cal_res(dt)
        ctx.assemble_mat(dt)
        _, g, _ = ctx.adjoint(lam, jt=False, poro=False)
        T0 = ctx.get("TRANS").copy()
        picks = rng.choice(grid.nconn, size=min(256, grid.nconn), replace=False)
        errs = []
        for c in picks:
            h = FD_STEP * T0[c]
            T = T0.copy()
            T[c] = T0[c] + h
            ctx.set("TRANS", T)
            rp = _residual(ctx, dt)
            T[c] = T0[c] - h
            ctx.set("TRANS", T)
            rm = _residual(ctx, dt)
            fd = lam @ (rp - rm) / (2 * h)
            errs.append(abs(fd - g[c]) / max(abs(g[c]), abs(fd), 1e-9 * np.max(np.abs(g))))
        ctx.set("TRANS", T0)
    assert max(errs) <= FD_TOL, max(errs)


@pytest.mark.parametrize("name", ["comp6_8x8x3", "bo_10x10x3"])
def test_dr_dporo_against_central_differences(gpu_lib, name):
    fx = P.load_fixture(name)
    model, grid = fim.model_and_grid_from_dump(fx)
    dim = model.nc + 1
    it = P.iterations(fx)[0]
    js = P.jac_state(fx, it)
    dt = float(js["dt"][0])
    rng = np.random.default_rng(13)
    lam = rng.normal(size=grid.nb * dim)
    with fim.FimContext(model, grid) as ctx:
        ctx.load_state(js)
        ctx.cal_res(dt)
        ctx.assemble_mat(dt)
        _, _, g = ctx.adjoint(lam, jt=False, trans=False)
        phi0 = ctx.get("PORO_INIT").copy()
        errs = []
        for n in rng.choice(grid.nb, size=min(64, grid.nb), replace=False):
            h = FD_STEP * phi0[n]
            r = []
            for sgn in (1, -1):
                phi = phi0.copy()
                phi[n] = phi0[n] + sgn * h
                ctx.set("PORO_INIT", phi)
                ctx.load_state(js)          # same state for both evaluations
                ctx.update_property()       # CalRock recomputes the pore volume
                r.append(_residual(ctx, dt))
            fd = lam @ (r[0] - r[1]) / (2 * h)
            errs.append(abs(fd - g[n]) / max(abs(g[n]), abs(fd), 1e-9 * np.max(np.abs(g))))
        ctx.set("PORO_INIT", phi0)
    assert max(errs) <= FD_TOL, max(errs)
