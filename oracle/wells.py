"""CPU restatement of the wells' part of the FIM residual (test
infrastructure only: the tests compare it with the reference's own values,
dumped by the reference harness into the wells_* golden fixtures).

Peaceman wells as the reference computes them for the residual of a Newton
iteration:

* perforation pressure: P_perf = bhp + dG (include/WellPeaceman.hpp:86,
  CalPerfP);
* phase transmissibilities: transj = WI*multiplier*kr/mu for each present
  phase, and for an injector transINJ = sum_j transj
  (PeacemanWell::CalTrans, src/WellPeaceman.cpp:365-400; the unweighted-
  permeability option is not restated);
* component mole rates (PeacemanWell::CalFlux, src/WellPeaceman.cpp:409-466):
  injector qi = transINJ*(P_cell - P_perf)*xi_inj*zi_inj, producer
  qi = sum_j transj*(Pj - P_perf)*xi_j*x_ij over present phases;
* residual (PeacemanWellIsoT::CalResFIM, src/WellPeaceman.cpp:1226-1265):
  each perforation adds qi*dt to its cell's component rows; the well's own
  row is bhp - tarBHP under BHP control, or +-tarRate + sum_i qi*factor_i
  under rate control, which also updates maxWellRelRes_mol; the caller then
  negates the whole residual (src/IsoThermalMethod.cpp:1170).

The perforations' WI is restated too (PeacemanWell::CalWI, Peaceman's
equivalent radius for x, y or z perforations, from the cell's size, net to
gross and permeabilities, the well radius and skin; well_index below).
Inputs not restated here and taken from the reference's dump: the
perforations' multiplier and dG (well setup), the injected fluid's molar
density xi_inj (the reference's PVT at the perforation pressure, computed at
the first flux of a time step) and the rate-control factors (CalFactor,
src/WellPeaceman.cpp:654-712: the mixture at surface conditions).

Arrays are in the reference's BulkVarSet layout: per cell P; per cell and
phase (cell-major) Pj, phaseExist, kr, mu, xi; xij as [nb * np * nc].
Plain loops in the reference's order, so sums accumulate exactly as there.
"""
from __future__ import annotations

import numpy as np


def split_wells(fx: dict) -> list[dict]:
    """Wells of one dumped iteration (the harness's dump_wells arrays) as a
    list of dicts with their perforations."""
    nc = len(fx["well_qi"]) // len(fx["well_type"])
    np_ = len(fx["perf_transj"]) // len(fx["perf_loc"])
    wells, p0 = [], 0
    for w, n in enumerate(np.asarray(fx["well_nperf"]).tolist()):
        sl = slice(p0, p0 + n)
        wells.append(dict(type=int(fx["well_type"][w]), mode=int(fx["well_mode"][w]),
                          bhp=float(fx["well_bhp"][w]), tar_bhp=float(fx["well_tar_bhp"][w]),
                          tar_rate=float(fx["well_tar_rate"][w]),
                          factor=np.asarray(fx["well_factor"][w * nc:(w + 1) * nc], dtype=float),
                          inj_zi=np.asarray(fx["well_inj_zi"][w * nc:(w + 1) * nc], dtype=float),
                          loc=np.asarray(fx["perf_loc"][sl]).astype(int), WI=np.asarray(fx["perf_WI"][sl]),
                          mult=np.asarray(fx["perf_mult"][sl]), dG=np.asarray(fx["perf_dG"][sl]),
                          xi_inj=np.asarray(fx["perf_xi"][sl])))
        p0 += n
    return wells, nc, np_


def perf_pressure(w: dict) -> list[float]:
    """CalPerfP (include/WellPeaceman.hpp:86)."""
    return [w["bhp"] + float(g) for g in w["dG"]]


def perf_trans(w: dict, phase_exist, kr, mu, np_: int):
    """PeacemanWell::CalTrans (src/WellPeaceman.cpp:365-400): per perforation
    the phase transmissibilities and, for an injector, their sum."""
    transj, trans_inj = [], []
    for p, k in enumerate(w["loc"]):
        temp = float(w["WI"][p]) * float(w["mult"][p])
        tj = [0.0] * np_
        tinj = 0.0
        for j in range(np_):
            idx = k * np_ + j
            if phase_exist[idx]:
                tj[j] = temp * float(kr[idx]) / float(mu[idx])
                tinj += tj[j]
        transj.append(tj)
        trans_inj.append(tinj if w["type"] == 0 else 0.0)
    return transj, trans_inj


def perf_flux(w: dict, state: dict, nc: int, np_: int):
    """PeacemanWell::CalFlux (src/WellPeaceman.cpp:409-466): per perforation
    and component the mole rate, and the well's totals."""
    P_perf = perf_pressure(w)
    transj, trans_inj = perf_trans(w, state["phaseExist"], state["kr"], state["mu"], np_)
    perf_qi = []
    qi = [0.0] * nc
    for p, k in enumerate(w["loc"]):
        q = [0.0] * nc
        if w["type"] == 0:
            dP = float(state["P"][k]) - P_perf[p]
            qt = trans_inj[p] * dP
            for i in range(nc):
                q[i] = qt * float(w["xi_inj"][p]) * float(w["inj_zi"][i])
                qi[i] += q[i]
        else:
            for j in range(np_):
                idx = k * np_ + j
                if state["phaseExist"][idx]:
                    dP = float(state["Pj"][idx]) - P_perf[p]
                    qj = transj[p][j] * dP
                    xi = float(state["xi"][idx])
                    for i in range(nc):
                        q[i] += qj * xi * float(state["xij"][idx * nc + i])
            for i in range(nc):
                qi[i] += q[i]
        perf_qi.append(q)
    return dict(P=P_perf, transj=transj, trans_inj=trans_inj, perf_qi=perf_qi, qi=qi)


def residual_with_wells(res_bulk, wells: list[dict], state: dict, dt: float, nc: int, np_: int):
    """PeacemanWellIsoT::CalResFIM (src/WellPeaceman.cpp:1226-1265) for every
    open well in order, on top of the bulk residual: returns the full residual
    (bulk rows, then nc + 1 rows per well) and maxWellRelRes_mol.

    res_bulk and the result are in the reference's returned sign: IsoT_FIM::
    CalRes negates the whole residual after the wells' terms
    (src/IsoThermalMethod.cpp:1170), and negation is exact, so the bulk rows
    are negated back, the terms added as there, and the sum negated."""
    length = nc + 1
    res = [-float(v) for v in res_bulk] + [0.0] * (length * len(wells))
    wid = len(res_bulk)
    max_rel = 0.0
    for w in wells:
        fl = perf_flux(w, state, nc, np_)
        for p, k in enumerate(w["loc"]):
            for i in range(nc):
                res[k * length + 1 + i] += fl["perf_qi"][p][i] * dt
        if w["mode"] == 0:
            res[wid] = w["bhp"] - w["tar_bhp"]
        else:
            r = w["tar_rate"] if w["type"] == 0 else -w["tar_rate"]
            for i in range(nc):
                r += fl["qi"][i] * float(w["factor"][i])
            res[wid] = r
            max_rel = max(max_rel, abs(r / w["tar_rate"]))
        wid += length
    return -np.array(res), max_rel


def _matmul_add(alpha, A, B, beta, C):
    """alpha*A*B + beta*C of row-major dense blocks (DaABpbC,
    src/DenseMat.cpp:61-85, which the reference hands to BLAS dgemm; the
    summation order of a BLAS is not the reference's to fix, so this product is
    compared within a tolerance)."""
    return alpha * (np.asarray(A) @ np.asarray(B)) + beta * np.asarray(C)


def well_jacobian(wells: list[dict], state: dict, dt: float, nb: int, nc: int, np_: int):
    """PeacemanWellIsoT::AssembleMatInjFIM / AssembleMatProdFIM
    (src/WellPeaceman.cpp:1268-1361, 1488-1613) for every open well in order.

    Returns the blocks the wells add to the system, as (ncol x ncol) arrays:
    ``bulk_add[n]`` summed into cell n's diagonal block, ``bulk_well[(n, w)]``
    inserted in cell n's row at well w's column, ``well_diag[w]`` (the well's
    diagonal block), and ``well_bulk[(w, n)]`` in the well's row at cell n's
    column, w counted from nb.  state holds the bulk arrays the assembly reads
    (BulkVarSet layout, dSec_dPri as [nb][ncol2][ncol])."""
    ncol = nc + 1
    ncol2 = np_ * nc + np_
    dsec = np.asarray(state["dSec_dPri"]).reshape(-1, ncol2, ncol)
    bulk_add, bulk_well, well_diag, well_bulk = {}, {}, {}, {}
    for wi, w in enumerate(wells):
        wid = nb + wi
        transj, _ = perf_trans(w, state["phaseExist"], state["kr"], state["mu"], np_)
        diag = np.zeros((ncol, ncol))
        for p, n in enumerate(w["loc"]):
            dQdXpB = np.zeros((ncol, ncol))
            dQdXpW = np.zeros((ncol, ncol))
            dQdXsB = np.zeros((ncol, ncol2))
            wi_m = float(w["WI"][p]) * float(w["mult"][p])
            for j in range(np_):
                idx = n * np_ + j
                if not state["phaseExist"][idx]:
                    continue
                mu, muP = float(state["mu"][idx]), float(state["muP"][idx])
                tj = transj[p][j]
                if w["type"] == 0:
                    dP = float(state["P"][n]) - w["bhp"] - float(w["dG"][p])
                    xi_inj = float(w["xi_inj"][p])
                    for i in range(nc):
                        zi = float(w["inj_zi"][i])
                        transIJ = tj * xi_inj * zi
                        dQdXpB[i + 1, 0] += transIJ * (1 - dP * muP / mu)
                        dQdXpW[i + 1, 0] += -transIJ
                        for k in range(np_):
                            dQdXsB[i + 1, k] += (wi_m * xi_inj * zi * float(state["dKrdS"][idx * np_ + k])
                                                 * dP / mu)
                        for k in range(nc):
                            dQdXsB[i + 1, np_ + j * nc + k] += -transIJ * dP / mu * float(
                                state["mux"][idx * nc + k])
                else:
                    dP = float(state["Pj"][idx]) - w["bhp"] - float(w["dG"][p])
                    xi, xiP = float(state["xi"][idx]), float(state["xiP"][idx])
                    for i in range(nc):
                        xij = float(state["xij"][idx * nc + i])
                        transIJ = tj * xi * xij
                        dQdXpB[i + 1, 0] += transIJ * (1 - dP * muP / mu) + dP * tj * xij * xiP
                        dQdXpW[i + 1, 0] += -transIJ
                        for k in range(np_):
                            tmp = wi_m * dP / mu * xi * xij * float(state["dKrdS"][idx * np_ + k])
                            tmp += transIJ * float(state["dPcdS"][idx * np_ + k])
                            dQdXsB[i + 1, k] += tmp
                        for k in range(nc):
                            tmp = dP * tj * xij * (float(state["xix"][idx * nc + k])
                                                   - xi / mu * float(state["mux"][idx * nc + k]))
                            dQdXsB[i + 1, np_ + j * nc + k] += tmp
                        dQdXsB[i + 1, np_ + j * nc + i] += tj * xi * dP
            bb = _matmul_add(dt, dQdXsB, dsec[n], dt, dQdXpB)
            bulk_add[n] = bulk_add.get(n, np.zeros((ncol, ncol))) + bb
            bulk_well[(n, wid)] = dQdXpW * dt
            if w["mode"] == 1:
                ww = np.zeros((ncol, ncol))
                for i in range(nc):
                    ww[0, 0] += dQdXpW[i + 1, 0] * float(w["factor"][i])
                    ww[i + 1, i + 1] = 1.0
                diag = diag + ww
                m = _matmul_add(1.0, dQdXsB, dsec[n], 1.0, dQdXpB)
                wb = np.zeros((ncol, ncol))
                for i in range(nc):
                    wb[0, :] += float(w["factor"][i]) * m[i + 1, :]
                well_bulk[(wid, n)] = wb
            else:
                diag = diag + np.eye(ncol)
                well_bulk[(wid, n)] = np.zeros((ncol, ncol))
        well_diag[wid] = diag
    return dict(bulk_add=bulk_add, bulk_well=bulk_well, well_diag=well_diag, well_bulk=well_bulk)


PI = 3.141592653  # include/OCPConst.hpp:32, the reference's value


def well_index(direction: int, dx: float, dy: float, dz: float, ntg: float, kx: float, ky: float, kz: float,
               radius: float, skin: float, conv_darcy: float, kh: float = -1.0):
    """PeacemanWell::CalWI (src/WellPeaceman.cpp:277-361) for a perforation
    whose WI is not given: Peaceman's equivalent radius for a perforation
    along x (0), y (1) or z (2); kh < 0 means derived from the cell.  Returns
    (WI, kh).  math.pow and math.log are the C library's, as the reference's."""
    import math
    dz = dz * ntg
    if direction == 0:
        a, b, l1, l2, length = ky, kz, dy, dz, dx
    elif direction == 1:
        a, b, l1, l2, length = kz, kx, dz, dx, dy
    elif direction == 2:
        a, b, l1, l2, length = kx, ky, dx, dy, dz
    else:
        raise ValueError("unstructured perforations are not restated")
    ab = a * b
    a_b = a / b
    ro = 0.28 * math.pow((l1 * l1 * math.pow(1 / a_b, 0.5) + l2 * l2 * math.pow(a_b, 0.5)), 0.5)
    ro /= (math.pow(a_b, 0.25) + math.pow(1 / a_b, 0.25))
    if kh < 0:
        kh = length * math.pow(ab, 0.5)
    wi = (2 * PI) * kh / (math.log(ro / radius) + skin)
    return wi * conv_darcy, kh
