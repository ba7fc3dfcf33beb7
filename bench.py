#!/usr/bin/env python3
"""FIM Newton-step throughput on GB300: cells/s of one Newton iteration of
the compositional PR-EoS path (property update with flash and FlashDer,
kr/Pc, rock, flux, residual and block-CSR Jacobian), batched GPU form vs the
plain per-kernel form, beside the reference algorithm on the host cores.

Workload (the compositional single-Newton-step case): 60 x 60 x 10 = 36,000
cells, 6 seeded pseudo-components, per-cell feed z ~ Dirichlet(2), P ~
U(10, 30) MPa, T = 345 K, 50 mD, porosity 0.2, PTN start; the timed step is
the second Newton iteration of the time step (two seeded Newton updates).  Wells are
host-side in the reference design and not part of the GPU step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  value = device-resident cells/s of the
batched form (CUDA events on the library's stream, L2 flushed between
steps); e2e = the same metric through the C ABI with host buffers (pinned
Newton update in, residual and Jacobian values out) inside the timed region.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ, NCOMP, SEED = 60, 60, 10, 6, 2
DT, DSMAX = 0.1, 0.2
METRIC = "FIM Newton-step cells/s (flash+assembly), batched vs plain GPU, <=1e-10 rel err"
WORKLOAD = "compositional PR-EoS FIM, 6 components, 60x60x10 = 36000 cells, single Newton step"


# ------------------------------------------------------------ CUDA runtime --
class Cudart:
    def __init__(self):
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        else:
            raise RuntimeError("libcudart not found")
        rt = self.rt
        rt.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
        rt.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
        rt.cudaEventSynchronize.argtypes = [C.c_void_p]
        rt.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaMemsetAsync.argtypes = [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p]
        rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        rt.cudaSetDevice.argtypes = [C.c_int]

    def event(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def elapsed_ms(self, a, b):
        self.rt.cudaEventSynchronize(b)
        ms = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(ms), a, b) == 0
        return ms.value

    def malloc(self, nbytes):
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), nbytes) == 0
        return p

    def pinned(self, n, dtype=np.float64):
        p = C.c_void_p()
        nbytes = int(n * np.dtype(dtype).itemsize)
        assert self.rt.cudaMallocHost(C.byref(p), nbytes) == 0
        buf = (C.c_char * nbytes).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype, count=n)


# ----------------------------------------------------------------- clocks ---
class ClockSampler:
    """nvidia-smi samples every 50 ms, of which those stamped inside the
    window [start(), end()] (the timed loop) are kept; all samples when none
    falls inside it."""
    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu=0, interval_ms=50):
        self.p = None
        self.t0 = self.t1 = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", str(interval_ms)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def start(self, t=None):
        self.t0 = time.time() if t is None else t

    def end(self, t=None):
        self.t1 = time.time() if t is None else t

    @staticmethod
    def _stamp(s):
        from datetime import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.strptime(s, fmt).timestamp()
            except ValueError:
                pass
        return None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm, mx = float(f[1]), float(f[2])
            except ValueError:
                continue
            rows.append((self._stamp(f[0]), sm, mx, [nm for nm, v in zip(self.NAMES, f[5:9])
                                                     if v.lower().startswith("active")]))
        inside = [r for r in rows if r[0] is not None and self.t0 is not None and self.t1 is not None
                  and self.t0 <= r[0] <= self.t1]
        use = inside or rows
        sm = [r[1] for r in use]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(r[2] for r in use) if use else None,
                "reasons": sorted({nm for r in use for nm in r[3]}), "samples": len(use),
                "window": "timed loop" if inside else "whole sampler run (no sample inside the timed loop)"}


# ---------------------------------------------------------------- workload --
def newton_updates(grid, Ni):
    """Two seeded Newton updates (dP ~ N(0, 2) bar, dNi = Ni N(0, 2e-3))."""
    out = []
    for k in range(2):
        rng = np.random.default_rng(SEED + 77 + k)
        u = np.zeros((grid.nb, NCOMP + 2))
        u[:, 0] = rng.normal(0.0, 2.0, grid.nb)
        u[:, 1:] = Ni.reshape(grid.nb, -1) * rng.normal(0.0, 2e-3, (grid.nb, NCOMP + 1))
        out.append(u.ravel())
    return out


def build_workload(variant, device=0):
    """PTN start, pores filled; first Newton iteration of the time step; the
    timed step is the second Newton iteration (the flash then starts from the
    phase state and iteration history of the first, as in a simulation)."""
    from opencaeporox_gb300 import synthetic
    from opencaeporox_gb300.fim import FimContext
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid(NX, NY, NZ)
    st = synthetic.comp_initial_state(grid, NCOMP, SEED)
    ctx = FimContext(model, grid, device=device, variant=variant)
    ctx.load_state(st)
    ctx.update_property()  # PTN start: FlashDer with no phase history (MixtureUnit::InitFlashFIM)
    # scale the moles so the fluid fills the pores, then flash again from scratch
    scale = ctx.get("ROCKVP") / ctx.get("VF")
    Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    ctx.load_state(st)
    ctx.set("SKIP_FLAG", np.zeros(grid.nb, np.uint8))
    ctx.update_property()
    ctx.cal_res(DT)
    ctx.update_last_time_step()
    u1, u2 = newton_updates(grid, Ni)
    ctx.get_solution(u1, DSMAX)  # Newton iteration 1
    ctx.update_property()
    ctx.cal_res(DT)
    ctx.checkpoint(1)  # before the second Newton update
    ctx.get_solution(u2, DSMAX)
    ctx.checkpoint(0)  # input of the timed Newton iteration
    return ctx, model, grid, u2


def time_device(ctx, rt, steps, warmup, flush):
    """Device time per step (ms), CUDA events on the library's stream."""
    stream = C.c_void_p(ctx.stream)
    e0, e1 = rt.event(), rt.event()
    times = []
    launches0 = None
    for k in range(warmup + steps):
        ctx.checkpoint(0, restore=True)
        rt.rt.cudaMemsetAsync(flush[0], k & 0xff, flush[1], stream)
        if k == warmup:
            launches0 = ctx.launch_count
        rt.rt.cudaEventRecord(e0, stream)
        ctx.enqueue_step(DT)
        rt.rt.cudaEventRecord(e1, stream)
        ms = rt.elapsed_ms(e0, e1)
        rep = ctx.step_report()
        if rep.status_or & ((1 << 4) | (1 << 5)):
            raise RuntimeError("physical check failed in the timed step")
        if k >= warmup:
            times.append(ms)
    return times, ctx.launch_count - launches0


def time_e2e(ctx, rt, steps, warmup, flush, u):
    """End to end through the C ABI: pinned u in, residual + Jacobian values out."""
    stream = C.c_void_p(ctx.stream)
    nb, nc = ctx.nb, ctx.nc
    _, nnz_col, _ = None, None, None
    rp, col, val = ctx.jacobian()
    u_pin = rt.pinned(u.size)
    u_pin[:] = u
    res_pin = rt.pinned(nb * (nc + 1))
    jac_pin = rt.pinned(val.size)
    times = []
    for k in range(warmup + steps):
        ctx.checkpoint(1, restore=True)
        rt.rt.cudaMemsetAsync(flush[0], k & 0xff, flush[1], stream)
        rt.rt.cudaStreamSynchronize(stream)
        t0 = time.perf_counter()
        ctx.step(u=u_pin, dSmax=DSMAX, dt=DT, res_out=res_pin, jac_out=jac_pin)
        t1 = time.perf_counter()
        if k >= warmup:
            times.append((t1 - t0) * 1e3)
    return times, u.nbytes, res_pin.nbytes + jac_pin.nbytes


def stage_profile(ctx, rt, flush, reps=3):
    stream = C.c_void_p(ctx.stream)
    ctx.profile(True)
    for k in range(reps):
        ctx.checkpoint(0, restore=True)
        rt.rt.cudaMemsetAsync(flush[0], k & 0xff, flush[1], stream)
        ctx.enqueue_step(DT)
        ctx.step_report()
    prof = ctx.profile_read()
    ctx.profile(False)
    return {k: (v[0] / max(v[1], 1), v[1] // reps) for k, v in prof.items() if v[1]}


def cpu_baseline(threads=None):
    """The reference algorithm (oracle port, C, OpenMP over cells) on the host
    cores: the same workload and Newton iteration, timed on the host."""
    from opencaeporox_gb300 import synthetic
    from oracle.pyoracle import OracleBulk
    model = synthetic.comp_model(NCOMP, SEED)
    grid = synthetic.comp_grid(NX, NY, NZ)
    st = synthetic.comp_initial_state(grid, NCOMP, SEED)
    ob = OracleBulk(model, grid)
    ob.load(st)
    ob.update_property()
    scale = ob.a["rockVp"] / ob.a["vf"]
    Ni = (st["Ni"].reshape(grid.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(grid.nb, -1).sum(axis=1))
    ob.load(st)
    ob.a["skip_flag"][:] = 0
    ob.update_property()
    ob.cal_res(DT)
    ob.a["lNi"][:] = ob.a["Ni"]
    u1, u2 = newton_updates(grid, Ni)
    ob.newton_update(u1, DSMAX)
    ob.update_property()
    ob.cal_res(DT)
    ob.newton_update(u2, DSMAX)
    saved = {k: v.copy() for k, v in ob.a.items()}
    times = []
    t_end = time.perf_counter() + 12.0
    while time.perf_counter() < t_end or len(times) < 2:
        for k, v in saved.items():
            ob.a[k][:] = v
        t0 = time.perf_counter()
        ob.update_property()
        ob.cal_res(DT)
        ob.assemble(DT)
        times.append(time.perf_counter() - t0)
        if len(times) >= 50:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return grid.nb / statistics.median(times), cores, len(times)


def fp64_peak(device=0):
    """FP64 peak of this GPU (TFLOP/s), measured by the library's DFMA-chain
    probe: the measured-peaks file carries HBM and bf16 figures only."""
    from opencaeporox_gb300.fim import measure_fp64_tflops
    return max(measure_fp64_tflops(device, 20000) for _ in range(3))


# FP64 operations of the flash on this workload, per cell: 2 x DFMA + DADD + DMUL
# thread-level instructions of the plain one-thread-per-cell kernel (k_flash_comp)
# for the timed Newton iteration (ncu smsp__sass_thread_inst_executed_op_
# {dfma,dadd,dmul}_pred_on.sum: 223.4 M, 121.7 M, 142.7 M = 711.2 MFLOP), divided by
# the 36,000 cells; libm internals included.  The batched form does the same
# algorithmic work in another order (profiles/k_flash_comp_comp6_36k.md).
FLASH_FP64_FLOP_PER_CELL = (2 * 223408633 + 121682495 + 142721273) / 36000
# DRAM bytes (read + write) of that launch, from the same capture.
FLASH_DRAM_BYTES = 107259392 + 173581568        # two-stream form: budgeted + cooperative kernels (ncu)
FLASH_DRAM_BYTES_FUSED = 155323904 + 250230016  # k_flash_fused<6> on this step (ncu, one launch)


def assembly_bytes(nb, nconn, nc, nnzb):
    """Algorithmic HBM bytes of the Jacobian assembly (k_jac_conn + k_jac_rows):
    every input it reads, once, and the block-CSR values it writes.
    Per cell (np = 3 phases, nct = nc components incl. water): kr, mu, muP,
    xi, xiP, rhoP (6 np), xij, rhox, xix, mux (4 np nct), dKrdS, dPcdS (2 np^2),
    dSec_dPri ((np nct + np) (nct + 1)), v, poroP, vfP (3), vfi (nct) -- doubles;
    per connection: bId, eId (2 x u32), trans (f64), upblock (np x u32),
    dP (np x f64); out: nnzb blocks of (nct + 1)^2 doubles."""
    np_, nct = 3, nc
    per_cell = 8 * (6 * np_ + 4 * np_ * nct + 2 * np_ * np_ + (np_ * nct + np_) * (nct + 1) + 3 + nct)
    per_conn = 4 * 2 + 8 + 4 * np_ + 8 * np_
    return nb * per_cell + nconn * per_conn + nnzb * (nct + 1) ** 2 * 8


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


# ------------------------------------------------- batched-flash stress ---
FS_CELLS, FS_NCOMP, FS_SEED, FS_TEMP = 1 << 20, 10, 3, 71.85
FS_METRIC = "batched-flash stress: flash cells/s, 10 components, 20% of cells near saturation"


def flash_stress(args, rt, local):
    """1,048,576 independent 10-component cells; 20 % placed within 5 % of their
    saturation pressure by bisection on the seeded fluid's envelope, the rest
    at P ~ U(5, 40) MPa, z ~ Dirichlet(1.5), T = 345 K.  Each timed flash starts
    from no phase history (full stability test) with the iteration counters
    of the previous flash of the same cells.  Plain one-thread-per-cell kernel
    vs the batched form (cost order, work budget, warp-cooperative tail)."""
    from opencaeporox_gb300 import synthetic
    from opencaeporox_gb300.fim import FimContext
    model = synthetic.comp_model(FS_NCOMP, FS_SEED)
    t0 = time.perf_counter()
    P, Ni = synthetic.flash_stress_cells(lambda g: FimContext(model, g, device=local, variant=1), FS_CELLS,
                                         FS_NCOMP, FS_SEED, temp_c=FS_TEMP)
    t_setup = time.perf_counter() - t0
    print(f"flash-stress: inputs ready in {t_setup:.1f} s", file=sys.stderr, flush=True)
    grid = synthetic.flash_grid(FS_CELLS)
    st = synthetic.flash_state(P, Ni, FS_TEMP)
    out = {}
    for variant in (0, 1):
        ctx = FimContext(model, grid, device=local, variant=variant)
        ctx.load_state(st)
        ctx.update_property()  # iteration history
        ctx.load_state(st)
        ctx.checkpoint(0)
        if variant == 1 and not args.no_tune:
            # tune on the flash stage (the step has no connections)
            from opencaeporox_gb300 import autotune
            # each flash of this workload takes seconds: a small candidate set, one round
            space = {"fused_blocks": ("sms", 0, 1, 2), "fused_coop_blocks": (0,), "flash_budget": (48, 192),
                     "predefer": (0, 192),
                     "coop_cells": (608, 1216, 4864), "coop_blocks": (608,), "block_cell": (128,), "pre_blocks": (0,)}
            out["autotune"] = {k: v for k, v in autotune.tune(ctx, DT, slot=0, space=space, rounds=1,
                                                              reps=1).items() if k != "trials"}
        times = []
        for k in range(args.warmup + args.steps):
            ctx.checkpoint(0, restore=True)
            ctx.profile(True)
            ctx.update_property()
            ms, n = ctx.profile_read()["flash"]
            ctx.profile(False)
            if k >= args.warmup:
                times.append(ms)
        print(f"flash-stress: variant {variant} flash {statistics.median(times):.1f} ms", file=sys.stderr, flush=True)
        pe = ctx.get("PHASE_EXIST").reshape(-1, 3)
        out[variant] = dict(ms=statistics.median(times), two_phase=int(np.sum((pe[:, 0] != 0) & (pe[:, 1] != 0))),
                            iters=ctx.get("FLASH_ITERS").reshape(-1, 5),
                            deferred=ctx.get_param("deferred") if variant == 1 else 0,
                            predeferred=ctx.get_param("predeferred") if variant == 1 else 0,
                            level=ctx.get_param("level") if variant == 1 else 0)
        ctx.close()
    it = out[0]["iters"].sum(axis=1)
    line = {"metric": FS_METRIC, "value": FS_CELLS / (out[1]["ms"] * 1e-3), "unit": "cells/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out[1]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "1,048,576 independent cells, 10 seeded components, 20% within 5% of "
                                   "saturation (bisection), rest P~U(5,40) MPa, z~Dirichlet(1.5), T=345 K"},
            "plain_value": FS_CELLS / (out[0]["ms"] * 1e-3), "plain_ms": out[0]["ms"],
            "batched_over_plain": out[0]["ms"] / out[1]["ms"], "two_phase_cells": out[0]["two_phase"],
            "iterations_per_cell": {"mean": float(it.mean()), "p99": float(np.percentile(it, 99)),
                                    "max": int(it.max())},
            "deferred_cells": out[1]["deferred"], "predeferred_cells": out[1]["predeferred"],
            "level": out[1]["level"], "autotune": out.get("autotune"), "setup_s": t_setup,
            "timing": "flash stage, CUDA events on the library stream"}
    return line


# ------------------------------------------------------ large Newton step ---
LG_NX, LG_NY, LG_NZ, LG_NCOMP, LG_SEED = 200, 200, 100, 9, 5
LG_METRIC = "FIM Newton-step cells/s, 4,000,000-cell compositional grid, 9 components"


def large_step(args, rt, local):
    """200 x 200 x 100 = 4,000,000 cells, 9 seeded components, lognormal
    permeability (median 100 mD, sigma_ln 2.0, correlation 10 cells), on a
    corner-point grid (COORD / ZCORN) whose layers dip by seeded angles within
    +-5 degrees and whose pillars lean by seeded slopes within +-0.02, read by
    the corner-point ingest.  PTN start, the second Newton iteration timed as
    in the default workload; plain vs batched form, library defaults."""
    from opencaeporox_gb300 import synthetic
    from opencaeporox_gb300.fim import FimContext
    from opencaeporox_gb300.grid import corner_point_grid
    nx, ny, nz = args.large_dims
    rng = np.random.default_rng(LG_SEED)
    dxy, dz = 20.0, 2.0
    dip_x, dip_y = rng.uniform(-5, 5, 2)
    n = nx * ny * nz
    t0 = time.perf_counter()
    coord, zcorn = synthetic.dipping_corner_point(nx, ny, nz, dxy, dz, 2000.0, dip_x, dip_y, 0.02, seed=LG_SEED)
    k = synthetic.layered_lognormal_perm(nx, ny, nz, 100.0, 2.0, 10, LG_SEED)
    grid = corner_point_grid(nx, ny, nz, coord, zcorn, k, k, 0.1 * k, np.full(n, 0.2),
                             conv_darcy=synthetic.METRIC["CONV_DARCY"])
    print(f"large: corner-point ingest {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    model = synthetic.comp_model(LG_NCOMP, LG_SEED)
    out = {}
    flush = (rt.malloc(512 << 20), 512 << 20)
    for variant in args.large_variants:
        t0 = time.perf_counter()
        ctx = FimContext(model, grid, device=local, variant=variant)
        synthetic.ptn_workload(ctx, grid, LG_NCOMP, LG_SEED, dt=DT, dsmax=DSMAX)
        ctx.checkpoint(0)
        print(f"large: variant {variant} set up in {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
        times, _ = time_device(ctx, rt, args.steps, args.warmup, flush)
        prof = stage_profile(ctx, rt, flush, reps=1)
        out[variant] = dict(ms=statistics.median(times), stages={st: round(v[0], 3) for st, v in prof.items()},
                            deferred=ctx.get_param("deferred") if variant == 1 else 0,
                            predeferred=ctx.get_param("predeferred") if variant == 1 else 0,
                            level=ctx.get_param("level") if variant == 1 else 0,
                            params={k: ctx.get_param(k) for k in ("fused_blocks", "fused_coop_blocks", "flash_budget", "predefer",
                                                                 "coop_cells", "coop_blocks", "pre_blocks",
                                                                 "cell_blocks", "block_cell")} if variant == 1 else None)
        print(f"large: variant {variant} step {out[variant]['ms']:.1f} ms", file=sys.stderr, flush=True)
        ctx.close()
    if 0 not in out or 1 not in out:  # one form only (profiling runs): its times
        return {"large_dims": [nx, ny, nz], **{f"variant{v}": o for v, o in out.items()}}
    metric = LG_METRIC if n == LG_NX * LG_NY * LG_NZ else LG_METRIC.replace("4,000,000", f"{n:,}")
    return {"metric": metric, "value": n / (out[1]["ms"] * 1e-3), "unit": "cells/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out[1]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{nx}x{ny}x{nz} = {n:,} cells, 9 components, lognormal k (median 100 mD, "
                                   "sigma_ln 2.0), corner-point grid (COORD/ZCORN: layers dipping within "
                                   "+-5 degrees, leaning pillars), second Newton iteration",
                       "connections": int(grid.nconn)},
            "plain_value": n / (out[0]["ms"] * 1e-3), "plain_ms": out[0]["ms"],
            "batched_over_plain": out[0]["ms"] / out[1]["ms"], "stages_ms": out[1]["stages"],
            "plain_stages_ms": out[0]["stages"], "deferred_cells": out[1]["deferred"],
            "predeferred_cells": out[1]["predeferred"], "level": out[1]["level"], "params": out[1]["params"],
            "timing": "CUDA events on the library stream around the step (the batched form's graph), "
                      "L2 flushed between steps; stage times from one eager profiled step (library defaults)"}


class Ranks:
    """torchrun ranks: one replica of the workload per GPU (the path has no
    cross-rank exchange inside a Newton step here); host barrier and max over
    ranks through torch.distributed (gloo)."""

    def __init__(self, world):
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self, rt=None):
        if rt is not None:
            rt.rt.cudaDeviceSynchronize()
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner (library defaults)")
    ap.add_argument("--workload", default="fim", choices=["fim", "flash-stress", "large"],
                    help="fim: the compositional Newton step (default); flash-stress: 1M independent flashes; "
                         "large: the 4M-cell Newton step")
    ap.add_argument("--large-dims", type=lambda v: tuple(int(x) for x in v.split(",")), default=(LG_NX, LG_NY, LG_NZ),
                    help="grid of the large workload, NX,NY,NZ (default 200,200,100)")
    ap.add_argument("--large-variants", type=lambda v: tuple(int(x) for x in v.split(",")), default=(0, 1),
                    help="forms the large workload runs: 0 plain, 1 batched (default 0,1)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import build as ob
        ob.build()
        v, cores, n = cpu_baseline()
        line = {"metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": NX * NY * NZ / v * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD}, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "cells/s", "cores": cores, "kind": "port",
                                 "sample": f"full 36000-cell second Newton iteration, {n} repetitions, median"},
                "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from opencaeporox_gb300 import build as gb
    gb.build()
    rt = Cudart()
    rt.rt.cudaSetDevice(local)
    if args.workload != "fim":
        if rank == 0:
            fn = {"flash-stress": flash_stress, "large": large_step}[args.workload]
            print(json.dumps(fn(args, rt, local)))
        return
    ranks = Ranks(world)
    flush_bytes = 512 << 20
    flush = (rt.malloc(flush_bytes), flush_bytes)
    results = {}
    tuned = None
    for variant in (0, 1):
        ctx, model, grid, u = build_workload(variant, device=local)
        if variant == 1 and not args.no_tune:
            from opencaeporox_gb300 import autotune
            tuned = autotune.tune(ctx, DT, slot=0)
        ranks.barrier(rt)
        t, launches = time_device(ctx, rt, args.steps, args.warmup, flush)
        ranks.barrier(rt)
        prof = stage_profile(ctx, rt, flush)
        results[variant] = dict(ms=ranks.max(statistics.median(t)), mean=statistics.fmean(t),
                                launches=launches / args.steps, prof=prof, ctx=ctx, u=u)
    clocks = ClockSampler(local)
    time.sleep(0.5)  # the sampler's first samples come after its start-up
    ranks.barrier(rt)
    clocks.start()
    tb, launches = time_device(results[1]["ctx"], rt, args.steps, args.warmup, flush)
    clocks.end()
    ranks.barrier(rt)
    ck = clocks.stop()
    ranks.barrier(rt)
    e2e_t, h2d, d2h = time_e2e(results[1]["ctx"], rt, args.steps, args.warmup, flush, results[1]["u"])
    ranks.barrier(rt)
    nb = NX * NY * NZ
    ms = ranks.max(statistics.median(tb))
    value = nb / (ms * 1e-3) * world
    plain = nb / (results[0]["ms"] * 1e-3) * world
    e2e_ms = ranks.max(statistics.median(e2e_t))
    prof = results[1]["prof"]
    dom = max(prof, key=lambda k: prof[k][0])
    fp64 = fp64_peak(local)
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    flash_ms = prof["flash"][0]
    fused = results[1]["ctx"].get_param("fused_blocks") > 0
    roof = {"kernel": ("k_flash_fused + k_flash_post" if fused else "k_flash_budget + k_flash_pe_coop + k_flash_post")
                      + " (flash stage of the batched step)", "bound": "fp64", "unit": "TFLOP/s",
            "peak": fp64, "peak_source": "measured (DFMA-chain probe of this library, best of 3)",
            "achieved": None, "frac": None, "traffic": FLASH_DRAM_BYTES_FUSED if fused else FLASH_DRAM_BYTES}
    if FLASH_FP64_FLOP_PER_CELL:
        roof["achieved"] = FLASH_FP64_FLOP_PER_CELL * nb / (flash_ms * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / fp64
    ctx1 = results[1]["ctx"]
    rp, _, _ = ctx1.jacobian()
    asm_ms = prof["jac_conn"][0] + prof["jac_rows"][0]
    abytes = assembly_bytes(nb, ctx1.nconn, ctx1.nc, int(rp[-1]))
    roof_asm = {"kernel": "k_jac_conn + k_jac_rows (Jacobian assembly)", "bound": "hbm", "unit": "GB/s",
                "algorithmic_bytes": abytes, "achieved": abytes / (asm_ms * 1e-3) / 1e9, "peak": hbm,
                "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "of fallback 6800",
                "traffic": None}
    roof_asm["frac"] = roof_asm["achieved"] / (hbm or 6800.0)
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "l2": "flushed between steps (512 MiB memset)", "variant": "batched",
                       "parallelism": f"replicas x{world} (one 36000-cell grid per GPU)"},
            "plain_value": plain, "plain_ms_per_step": results[0]["ms"], "batched_over_plain": value / plain,
            "plain_stages_ms": {k: round(v[0], 4) for k, v in results[0]["prof"].items()},
            "stages_ms": {k: round(v[0], 4) for k, v in prof.items()}, "dominant_stage": dom,
            "roofline": roof, "roofline_assembly": roof_asm, "fp64_peak_tflops": fp64,
            "batched": {"flash_budget": ctx1.get_param("flash_budget"), "coop_blocks": ctx1.get_param("coop_blocks"),
                        "deferred_cells": ctx1.get_param("deferred"),
                        "predeferred_cells": ctx1.get_param("predeferred"), "level": ctx1.get_param("level"),
                        "block_cell": ctx1.get_param("block_cell"), "predefer": ctx1.get_param("predefer"),
                        "coop_cells": ctx1.get_param("coop_cells"), "pre_blocks": ctx1.get_param("pre_blocks"),
                        "cell_blocks": ctx1.get_param("cell_blocks"), "fused_blocks": ctx1.get_param("fused_blocks"),
                        "fused_coop_blocks": ctx1.get_param("fused_coop_blocks"),
                        "autotune": None if tuned is None else {k: v for k, v in tuned.items() if k != "trials"}},
            "clocks": ck, "gpu_launches": launches,
            "e2e": {"value": nb / (e2e_ms * 1e-3) * world, "unit": "cells/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h}}
    if rank == 0 and world == 1 and os.environ.get("OCPX_BENCH_NO_CPU") != "1":
        v, cores, n = cpu_baseline()
        line["cpu_baseline"] = {"value": v, "unit": "cells/s", "cores": cores, "kind": "port",
                                "sample": f"full 36000-cell second Newton iteration, {n} repetitions, median"}
    if rank == 0:
        print(json.dumps(line))
    ranks.close()


if __name__ == "__main__":
    main()
