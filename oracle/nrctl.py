"""CPU restatement of the reference's Newton-iteration and time-step control,
bulk part (test infrastructure only: the tests compare the device's results
with these and with the reference's own values in the golden fixtures).

Arrays are in the reference's BulkVarSet layout: P, T per cell; Ni as
[nb * nc] cell-major; S as [nb * np] cell-major; vf, rockVp per cell.
Plain Python loops in the reference's order, so each maximum is the
reference's value exactly (the fixtures are a few hundred cells).
"""
from __future__ import annotations

TINY = 1e-8  # include/OCPConst.hpp:30


def _upd(cur, x):
    """`if (fabs(cur) < fabs(x)) cur = x;` of the reference's loops."""
    return x if abs(cur) < abs(x) else cur


def max_change_nr(now: dict, last: dict, nc: int, np_: int = 3) -> dict:
    """OCPNRsuite::CalMaxChangeNR, bulk loop (src/OCPNRsuite.cpp:86-133):
    `last` is the previous Newton iterate (lP, lT, lN, lS)."""
    nb = len(now["P"])
    dP = dT = dN = dS = eV = 0.0
    for n in range(nb):
        dP = _upd(dP, now["P"][n] - last["P"][n])
        dT = _upd(dT, now["T"][n] - last["T"][n])
        Nt = 0.0
        for i in range(nc):
            Nt += last["Ni"][n * nc + i]
        for i in range(nc):
            dN = _upd(dN, (now["Ni"][n * nc + i] - last["Ni"][n * nc + i]) / Nt)
        for j in range(np_):
            dS = _upd(dS, now["S"][n * np_ + j] - last["S"][n * np_ + j])
        eV = _upd(eV, (now["vf"][n] - now["rockVp"][n]) / now["rockVp"][n])
    return dict(dP=dP, dT=dT, dN=dN, dS=dS, eV=eV)


def max_change_time(now: dict, last: dict, nc: int, np_: int = 3) -> dict:
    """OCPNRsuite::CalMaxChangeTime, bulk loop (src/OCPNRsuite.cpp:163-214):
    `last` is the last time step's state (lP, lT, lS, lNi)."""
    nb = len(now["P"])
    dP = dT = dN = dS = eV = 0.0
    for n in range(nb):
        dP = _upd(dP, now["P"][n] - last["P"][n])
        dT = _upd(dT, now["T"][n] - last["T"][n])
        for j in range(np_):
            dS = _upd(dS, now["S"][n * np_ + j] - last["S"][n * np_ + j])
        for i in range(nc):
            a, b = now["Ni"][n * nc + i], last["Ni"][n * nc + i]
            tmp = abs(b if a < b else a)  # fabs(std::max(Ni, lNi))
            if tmp > TINY:
                dN = _upd(dN, (a - b) / tmp)
        eV = _upd(eV, (now["vf"][n] - now["rockVp"][n]) / now["rockVp"][n])
    return dict(dP=dP, dT=dT, dN=dN, dS=dS, eV=eV)


def check_converge(maxRelRes_V, maxRelRes0_V, maxRelRes_N, maxWellRelRes_mol, dPBmax, dSmax, iterNR, tol, dPmin,
                   dSmin, maxIter, tmpfac=1.0) -> int:
    """ControlNR::CheckConverge with {"res", "d"} (src/OCPControlNR.cpp:27-77):
    0 converge, 1 continue, 2 not converged (OCPNRStateC values)."""
    conv = False
    if ((maxRelRes_V <= maxRelRes0_V * tol * tmpfac or maxRelRes_V <= tol * tmpfac or
         maxRelRes_N <= tol * tmpfac) and maxWellRelRes_mol <= tol * tmpfac):
        conv = True
    if abs(dPBmax) <= dPmin and abs(dSmax) <= dSmin:
        conv = True
    if conv:
        return 0
    return 2 if iterNR >= maxIter else 1


def next_time_step(current_dt, current_time, dPBmaxT, dPWmaxT, dSmaxT, iterNR, maxIncreFac, minChopFac, dPlim,
                   dSlim, timeMax, timeMin, end_time):
    """ControlTime::CalNextTimeStep with {"dP", "dS", "iter"}
    (src/OCPControlTime.cpp:128-178) after CalMaxChangeTime's well/bulk
    choice of dPmaxT (src/OCPNRsuite.cpp:223-228); returns (next dt,
    predicted dt)."""
    current_time = current_time + current_dt
    factor = maxIncreFac
    dPmaxT = dPWmaxT if abs(dPBmaxT) < abs(dPWmaxT) else dPBmaxT
    dPmax, dSmax = abs(dPmaxT), abs(dSmaxT)
    if dPmax > TINY:
        factor = min(factor, dPlim / dPmax)
    if dSmax > TINY:
        factor = min(factor, dSlim / dSmax)
    if iterNR < 5:
        factor = min(factor, 2.0)
    elif iterNR > 10:
        factor = min(factor, 0.5)
    else:
        factor = min(factor, 1.5)
    factor = max(minChopFac, factor)
    dt = current_dt * factor
    if dt > timeMax:
        dt = timeMax
    if dt < timeMin:
        dt = timeMin
    predict = dt
    if dt > end_time - current_time:
        dt = end_time - current_time
    return dt, predict

