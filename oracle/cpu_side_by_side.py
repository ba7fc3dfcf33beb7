"""The reference's own build and the C restatement of the oracle, timed side
by side on this host, one thread each, on the same Newton iterations of the
same deck.

Test infrastructure (nothing on the library's path runs it).  It needs the
reference's own build (oracle/_ref/ocp_ref_dump, made by oracle/build.py where
the reference's sources are present) and the deck writer of the golden
fixtures (tests/golden/decks.py).

- The reference: the dump harness runs the deck and times, per Newton
  iteration, IsoT_FIM's property update (the flash of every cell, kr/Pc,
  rock, the wells' fluxes and CalRes: t_update) and AssembleMatBulks
  (t_assemble), the timers that stand for OCPTIME_UPDATE_GRID and
  OCPTIME_ASSEMBLE_MAT.
- The restatement (oracle/ocpx_oracle.c): update_property + cal_res from the
  state the reference's update started from, and assemble from the state its
  assembly started from, timed the same way.

Both are C/C++ built with -ffp-contract=off (the reference at -O2 with its
dense products in OpenBLAS, the restatement at -O3).  Run it with
OMP_NUM_THREADS=1 so that the restatement uses one thread, as the harness
does:

    OMP_NUM_THREADS=1 python oracle/cpu_side_by_side.py --dims 30 30 10 --ncomp 9
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[30, 30, 10])
    ap.add_argument("--ncomp", type=int, default=9)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    if os.environ.get("OMP_NUM_THREADS") != "1":
        print("note: OMP_NUM_THREADS is not 1; the restatement may use several threads")
    import decks
    import gen_fixtures as gf
    import parity as P
    from opencaeporox_gb300 import fim
    from oracle.pyoracle import OracleBulk

    nx, ny, nz = args.dims
    ni, text = decks.comp_deck(nx, ny, nz, args.ncomp, seed=args.seed, tsteps=(0.02, 0.05), smooth=True)
    data = gf.run_fim(text, "side", args.iters, ni=ni, calibrate=True)
    model, grid = fim.model_and_grid_from_dump(data)
    log = np.asarray(data["log"])            # step, iter, dt, event, t_update, t_assemble
    its = P.iterations(data)
    nb = grid.nb
    rows = []
    for k, it in enumerate(its):
        js = P.jac_state(data, it)
        pre = P.group(data, it + "/pre")
        if not pre or log[k, 3] != 0:
            continue
        dt = float(js["dt"][0])
        ob = OracleBulk(model, grid)
        t_asm, t_upd = [], []
        for _ in range(args.reps):
            ob.load(js)
            ob.cal_res(dt)
            t0 = time.perf_counter()
            ob.assemble(dt)
            t_asm.append(time.perf_counter() - t0)
            ob.load(js)
            ob.load(pre)
            t0 = time.perf_counter()
            ob.update_property()
            ob.cal_res(dt)
            t_upd.append(time.perf_counter() - t0)
        rows.append((it, log[k, 4], log[k, 5], min(t_upd), min(t_asm)))
    print(f"deck: {nx} x {ny} x {nz} = {nb} cells, {args.ncomp} components, {len(rows)} Newton iterations; "
          f"restatement: best of {args.reps}")
    print("iteration | reference update, assemble (s) | restatement update, assemble (s) | "
          "reference cells/s | restatement cells/s | restatement / reference")
    tot_r = tot_o = 0.0
    for it, ru, ra, ou, oa in rows:
        tot_r += ru + ra
        tot_o += ou + oa
        print(f"{it} | {ru:.3f}, {ra:.3f} | {ou:.3f}, {oa:.3f} | {nb / (ru + ra):,.0f} | {nb / (ou + oa):,.0f} | "
              f"{(ru + ra) / (ou + oa):.2f}x")
    n = len(rows)
    print(f"all | | | {n * nb / tot_r:,.0f} | {n * nb / tot_o:,.0f} | {tot_r / tot_o:.2f}x")


if __name__ == "__main__":
    main()
