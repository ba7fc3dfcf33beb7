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

Inputs not restated here and taken from the reference's dump: the
perforations' WI, multiplier and dG (well setup), the injected fluid's molar
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
