#!/usr/bin/env python3
"""FIM Newton-step throughput on GB300: cells/s of one Newton iteration of
the compositional PR-EoS path (property update with flash and FlashDer,
kr/Pc, rock, flux, residual, block-CSR Jacobian and the adjoint products),
batched GPU form vs the plain per-kernel form, beside the reference
algorithm on the host cores.

Workloads (--workload):
  large (default)  200 x 200 x 100 = 4,000,000 cells, 9 seeded components,
                   corner-point grid (COORD / ZCORN) whose layers dip by
                   seeded angles within +-5 degrees and whose pillars are
                   moved by seeded offsets within 10 % of the cell size,
                   lognormal permeability (median 100 mD, sigma_ln 2.0,
                   correlation 10 cells); every step also computes J^T lambda,
                   (dR/dT)^T lambda and (dR/dporo)^T lambda (lambda ~ N(0, 1)).
  fim              60 x 60 x 10 = 36,000 cells, 6 seeded components, 50 mD.
  flash-stress     1,048,576 independent 10-component flashes.
Both FIM workloads start from a seeded PTN start (P ~ U(10, 30) MPa,
z ~ Dirichlet(2), T = 345 K, pores filled) and time the second Newton
iteration of the time step (two seeded Newton updates), so the flash starts
from the phase state and iteration history of the first.  Their Peaceman
wells are part of every step, on the device (large: 10 injectors and 10
producers, 5 of them rate-controlled, through all 100 layers; fim: one
injector and one producer at opposite corners).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

Prints one JSON line (rank 0).  value = device-resident cells/s of the
batched form (its CUDA graph replayed on the library's stream, timed with
CUDA events, L2 flushed between steps); e2e = the same metric through the C
ABI with host buffers (the pinned Newton update in, the residual, Jacobian
values and adjoint products out) inside the timed region; parity = the timed
step against the oracle run from the same inputs on a window of the grid
(the large workload: two whole layers with their ghost layers).
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

DT, DSMAX = 0.1, 0.2
METRIC = "FIM Newton-step cells/s (flash+assembly), batched vs plain GPU, <=1e-10 rel err"
REL_TOL = 1e-10
LIBM_FACTOR = 4.0  # CUDA and glibc transcendentals differ by up to about 2 ulp per call; margin 2


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
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaFreeHost.argtypes = [C.c_void_p]
        rt.cudaMemsetAsync.argtypes = [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p]
        rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        rt.cudaSetDevice.argtypes = [C.c_int]
        self.pinned_ptrs = []

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
        nbytes = int(max(n, 1) * np.dtype(dtype).itemsize)
        assert self.rt.cudaMallocHost(C.byref(p), nbytes) == 0, f"cudaMallocHost({nbytes}) failed"
        self.pinned_ptrs.append(p)
        buf = (C.c_char * nbytes).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype, count=n)

    def free_pinned(self):
        for p in self.pinned_ptrs:
            self.rt.cudaFreeHost(p)
        self.pinned_ptrs = []


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


# -------------------------------------------------------------- workloads ---
class FimWorkload:
    """The compositional Newton step on 60 x 60 x 10 = 36,000 cells."""
    key = "fim"
    ncomp, seed = 6, 2
    dims = (60, 60, 10)
    adjoint = False

    def __init__(self, args):
        self.args = args

    @property
    def description(self):
        nx, ny, nz = self.dims
        return (f"compositional PR-EoS FIM, {self.ncomp} components, {nx}x{ny}x{nz} = {nx * ny * nz} cells, "
                "single Newton step")

    def model(self):
        from opencaeporox_gb300 import synthetic
        return synthetic.comp_model(self.ncomp, self.seed)

    def grid(self):
        from opencaeporox_gb300 import synthetic
        return synthetic.comp_grid(*self.dims)

    def wells(self, grid):
        """One injector at column (0, 0) and one producer at the opposite
        corner, through every layer, both under bottom-hole-pressure control."""
        from opencaeporox_gb300 import wells as W
        nx, ny, nz = self.dims
        k = np.full(grid.nb, 50.0)
        return W.vertical_wells(nx, ny, nz, 1, 1, 20.0, 5.0, k, k, grid.depth, self.ncomp, self.seed, corners=True)

    def parity_cells(self):
        """(owned cells, ghost cells) of the parity window: the whole grid."""
        nb = int(np.prod(self.dims))
        return np.arange(nb), np.zeros(0, np.int64)

    def cpu_sample(self):
        """(grid, cells of the whole grid it holds, description) of the CPU
        baseline's sample: the whole grid."""
        g = self.grid()
        return g, np.arange(g.nb), f"the whole {g.nb}-cell grid"


class LargeWorkload(FimWorkload):
    """200 x 200 x 100 = 4,000,000 cells, 9 components, dipping corner-point
    grid with moved pillars, lognormal permeability; the adjoint products in
    every step."""
    key = "large"
    ncomp, seed = 9, 5
    dxy, dz, top = 20.0, 2.0, 2000.0
    adjoint = True
    _grid = None

    def __init__(self, args):
        super().__init__(args)
        self.dims = tuple(args.large_dims)

    @property
    def description(self):
        nx, ny, nz = self.dims
        return (f"{nx}x{ny}x{nz} = {nx * ny * nz:,} cells, {self.ncomp} components, lognormal k (median 100 mD, "
                "sigma_ln 2.0, correlation 10 cells), corner-point grid (COORD/ZCORN: layers dipping within +-5 "
                "degrees, pillars moved within 10% of the cell size), second Newton iteration with the adjoint "
                "products J^T lambda, (dR/dT)^T lambda, (dR/dporo)^T lambda")

    def geometry(self):
        from opencaeporox_gb300 import synthetic
        nx, ny, nz = self.dims
        rng = np.random.default_rng(self.seed)
        dip_x, dip_y = rng.uniform(-5, 5, 2)
        coord, zcorn = synthetic.dipping_corner_point(nx, ny, nz, self.dxy, self.dz, self.top, dip_x, dip_y, 0.0,
                                                      seed=self.seed, pillar_jitter=0.1)
        k = synthetic.layered_lognormal_perm(nx, ny, nz, 100.0, 2.0, 10, self.seed)
        return coord, zcorn, k

    def _ingest(self, k0, k1):
        """The layers [k0, k1) as a grid of their own (the same cells and, among
        them, the same connections as in the whole grid)."""
        from opencaeporox_gb300 import synthetic
        from opencaeporox_gb300.grid import corner_point_grid
        nx, ny, nz = self.dims
        coord, zcorn, k = self.geometry()
        zc = zcorn.reshape(nz, -1)[k0:k1].ravel()
        ks = k.reshape(nz, -1)[k0:k1].ravel()
        n = ks.size
        return corner_point_grid(nx, ny, k1 - k0, coord, zc, ks, ks, 0.1 * ks, np.full(n, 0.2),
                                 conv_darcy=synthetic.METRIC["CONV_DARCY"])

    def grid(self):
        if LargeWorkload._grid is None or LargeWorkload._grid[0] != self.dims:
            t0 = time.perf_counter()
            g = self._ingest(0, self.dims[2])
            print(f"large: corner-point ingest {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
            LargeWorkload._grid = (self.dims, g)
        return LargeWorkload._grid[1]

    def wells(self, grid):
        """20 wells at seeded columns through every layer: 10 injectors and 10
        producers, 5 of them under a total hydrocarbon rate target."""
        from opencaeporox_gb300 import wells as W
        nx, ny, nz = self.dims
        _, _, k = self.geometry()
        return W.vertical_wells(nx, ny, nz, 10, 10, self.dxy, self.dz, k, 0.1 * k, grid.depth, self.ncomp,
                                self.seed, n_rate=5)

    def parity_cells(self):
        nx, ny, nz = self.dims
        layer = nx * ny
        k0 = max(1, nz // 2 - 1)
        k1 = min(nz - 1, k0 + 2)
        owned = np.arange(k0 * layer, k1 * layer)
        ghost = np.concatenate([np.arange((k0 - 1) * layer, k0 * layer), np.arange(k1 * layer, (k1 + 1) * layer)])
        return owned, ghost

    def cpu_sample(self):
        nx, ny, nz = self.dims
        layers = min(nz, max(1, int(self.args.cpu_layers)))
        k0 = max(0, nz // 2 - layers // 2)
        g = self._ingest(k0, k0 + layers)
        first = k0 * nx * ny
        return g, np.arange(first, first + g.nb), (f"layers {k0}..{k0 + layers - 1} of the grid ({g.nb:,} cells, "
                                                   "their state from the same seeds) as a grid of their own")


# -------------------------------------------------------------- GPU legs ---
def prepare(wl, model, grid, variant, device, recompute=False):
    """A context at the input of the timed Newton iteration: checkpoint 0 =
    the state after the second Newton update, checkpoint 1 = the state just
    before it.  Returns (ctx, u2)."""
    from opencaeporox_gb300 import synthetic
    from opencaeporox_gb300.fim import FimContext
    ctx = FimContext(model, grid, device=device, variant=variant, recompute=recompute)
    ctx.set_wells(wl.wells(grid))
    us = synthetic.ptn_workload(ctx, grid, wl.ncomp, wl.seed, dt=DT, dsmax=DSMAX, slot_before_last=1)
    ctx.checkpoint(0)
    if wl.adjoint:
        ctx.set_adjoint_seed(np.random.default_rng(wl.seed + 500).normal(size=ctx.nv))
    # the last update does not move the wells' bhp
    return ctx, np.r_[us[1], np.zeros(ctx.nv - us[1].size)]


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


def time_e2e(ctx, rt, steps, warmup, flush, u, adjoint):
    """End to end through the C ABI: the pinned Newton update in, residual,
    Jacobian values (and the adjoint products) out to pinned host buffers."""
    stream = C.c_void_p(ctx.stream)
    nb, nc = ctx.nb, ctx.nc
    nnz = ctx_nnz(ctx)
    u_pin = rt.pinned(u.size)
    u_pin[:] = u
    res_pin = rt.pinned(ctx.nv)
    jac_pin = rt.pinned(nnz * (nc + 1) ** 2)
    adj = (rt.pinned(ctx.nv), rt.pinned(ctx.nconn), rt.pinned(nb)) if adjoint else None
    times = []
    for k in range(warmup + steps):
        ctx.checkpoint(1, restore=True)
        rt.rt.cudaMemsetAsync(flush[0], k & 0xff, flush[1], stream)
        rt.rt.cudaStreamSynchronize(stream)
        t0 = time.perf_counter()
        ctx.step(u=u_pin, dSmax=DSMAX, dt=DT, res_out=res_pin, jac_out=jac_pin)
        if adjoint:
            ctx.get_adjoint(out=adj)
        t1 = time.perf_counter()
        if k >= warmup:
            times.append((t1 - t0) * 1e3)
    d2h = res_pin.nbytes + jac_pin.nbytes + (sum(a.nbytes for a in adj) if adjoint else 0)
    return times, u.nbytes, d2h


def ctx_nnz(ctx):
    nrow, nnz, bd = C.c_size_t(), C.c_size_t(), C.c_int()
    ctx.lib.ocpx_jacobian_dims(ctx.h, C.byref(nrow), C.byref(nnz), C.byref(bd))
    return nnz.value


def stage_profile(ctx, rt, flush, reps=1):
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


# --------------------------------------------------------------- parity ---
ORACLE_FIELDS = ["P", "T", "PB", "NI", "LNI", "NT", "VF", "VFP", "VFI", "PJ", "PC", "S", "PHASE_EXIST", "XIJ", "RHO",
                 "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "KR", "DKRDS", "DPCDS", "DSEC_DPRI", "PORO",
                 "POROP", "ROCKVP", "SKIP_FLAG", "SKIP_MINEIG", "SKIP_P", "SKIP_T", "SKIP_ZI"]
FLASH_KEYS = {"S": "S", "XIJ": "xij", "RHO": "rho", "XI": "xi", "MU": "mu", "RHOX": "rhox", "XIX": "xix",
              "MUX": "mux", "RHOP": "rhoP", "XIP": "xiP", "MUP": "muP", "VF": "vf", "VFP": "vfP", "VFI": "vfi",
              "NT": "Nt", "DSEC_DPRI": "dSec_dPri"}
PHASE_KEYS = ("RHO", "XI", "MU", "RHOP", "XIP", "MUP")
PHASE_COMP_KEYS = ("XIJ", "RHOX", "XIX", "MUX")
CELLWISE_KEYS = ("VFI", "VFP", "DSEC_DPRI")   # outputs of the NC x NC derivative solve: normwise per cell


def cells_ranges(cells):
    """Runs of consecutive cell numbers: [(first, count)]."""
    cells = np.asarray(cells, np.int64)
    if cells.size == 0:
        return []
    cut = np.nonzero(np.diff(cells) != 1)[0] + 1
    starts = np.concatenate([[0], cut])
    ends = np.concatenate([cut, [cells.size]])
    return [(int(cells[s]), int(e - s)) for s, e in zip(starts, ends)]


def get_cells(ctx, name, cells):
    return np.concatenate([ctx.get_range(name, f, n) for f, n in cells_ranges(cells)])


def flash_errors(got, ref, pe, nc):
    """Max relative error per flash output (floor 1e-12 x the array's
    scale); phase quantities where the phase exists; derivative-solve outputs
    normwise per cell."""
    out = {}
    n = pe.shape[0]
    for k in FLASH_KEYS:
        a = np.asarray(got[k], np.float64).reshape(n, -1)
        b = np.asarray(ref[k], np.float64).reshape(n, -1)
        if k in CELLWISE_KEYS:
            out[k] = float(np.max(np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)))
            continue
        if k in PHASE_KEYS:
            m = pe
        elif k in PHASE_COMP_KEYS:
            m = np.repeat(pe, nc, axis=1)
        else:
            m = np.ones_like(a, bool)
        a, b = a[m], b[m]
        if a.size == 0:
            out[k] = 0.0
            continue
        floor = max(np.max(np.abs(b)) * 1e-12, 1e-300)
        out[k] = float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))
    return out


def cell_errors(got, ref, pe, nc):
    """Per cell, the largest relative error over its flash outputs (floor
    1e-12 x each array's scale; phase quantities where the phase exists; the
    derivative-solve outputs normwise)."""
    n = pe.shape[0]
    out = np.zeros(n)
    for k in FLASH_KEYS:
        a = np.asarray(got[k], np.float64).reshape(n, -1)
        b = np.asarray(ref[k], np.float64).reshape(n, -1)
        if k in CELLWISE_KEYS:
            e = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
        else:
            if k in PHASE_KEYS:
                m = pe
            elif k in PHASE_COMP_KEYS:
                m = np.repeat(pe, nc, axis=1)
            else:
                m = np.ones_like(a, bool)
            floor = max(np.max(np.abs(b[m])) * 1e-12, 1e-300) if np.any(m) else 1e-300
            e = np.max(np.where(m, np.abs(a - b) / np.maximum(np.abs(b), floor), 0.0), axis=1)
        out = np.maximum(out, e)
    return out


NUDGES = ((1, 1), (2, 1), (3, 1), (4, 2), (5, 2), (6, 2))  # (seed, ulps) of the oracle's libm-sensitivity runs
RECHECK = tuple((s, 1) for s in range(7, 47)) + tuple((s, 2) for s in range(47, 87))


def recheck_cells(model, geometry, inputs, got, nudges=RECHECK):
    """Cells of a flash comparison left unexplained by the first sensitivity
    runs, rechecked alone: the oracle's sensitivity on them from more
    perturbation patterns (a cell's flash depends on its own inputs only, and
    a rare branch of its equilibrium -- an iteration more or less near a
    tolerance -- shows in a few patterns only).  geometry: (v, depth,
    poro_init) of the cells; inputs: oracle arrays of the cells; got: the
    flash outputs compared, rows per cell.  Returns how many cells stay above
    max(1e-10, 4 x that sensitivity)."""
    from opencaeporox_gb300.fim import Grid
    from oracle.pyoracle import OracleBulk
    n = geometry[0].size
    z = np.zeros(0, np.uint32)
    g1 = Grid(geometry[0], geometry[1], geometry[2], z, z, np.zeros(0))

    def run(variant="exact", seed=None, ulps=1):
        o = OracleBulk(model, g1, variant=variant)
        if seed is not None:
            o.set_nudge_seed(seed, ulps)
        o.load(inputs)
        o.update_property()
        return ({k: o.a[v].reshape(n, -1).copy() for k, v in FLASH_KEYS.items()},
                o.a["phaseExist"].reshape(-1, 3).astype(bool))

    ref, pe = run()
    e = cell_errors(got, ref, pe, model.nc)
    s = np.zeros(n)
    for seed, ulps in nudges:
        nz, pn = run("ulp", seed, ulps)
        sk = cell_errors(nz, ref, pe, model.nc)
        sk[np.any(pn != pe, axis=1)] = np.inf   # labels change under the perturbation: libm-sensitive
        s = np.maximum(s, sk)
    return int(np.sum(e > np.maximum(REL_TOL, LIBM_FACTOR * s)))


def parity(ctx, wl, model, grid, dump=None):
    """The timed step (the replayed graph) against the oracle from the same
    inputs on a window: owned cells with their ghost cells.  Upwind choices
    exact; phase labels exact except in cells whose labels the oracle itself
    changes when its transcendentals round one or two ulp differently
    (counted); flash outputs of the other cells, per cell, within max(1e-10,
    4 x the oracle's own libm sensitivity on that cell); residual rows on each
    equation's scale and Jacobian rows normwise within 1e-10, from the GPU's
    post-flash state.  dump: a .npz path that receives the inputs and outputs
    of the cells above 1e-10, for a closer look."""
    from opencaeporox_gb300 import halo
    from opencaeporox_gb300.fim import REF_NAMES
    from oracle.pyoracle import OracleBulk
    t0 = time.perf_counter()
    owned, ghost = wl.parity_cells()
    sub_grid, cells, conns = halo.subdomain(grid, owned, ghost)
    no = owned.size
    nc = model.nc
    inv = {v: k for k, v in REF_NAMES.items()}
    ctx.checkpoint(0, restore=True)
    inputs = {f: get_cells(ctx, f, cells) for f in ORACLE_FIELDS}
    ctx.enqueue_step(DT)
    ctx.step_report()
    got = {f: get_cells(ctx, f, owned) for f in list(FLASH_KEYS) + ["PHASE_EXIST"]}
    res_g = get_cells(ctx, "RES", owned).reshape(no, -1)
    c0, c1 = int(conns.min()), int(conns.max()) + 1
    up_g = ctx.get_range("UPBLOCK", c0, c1 - c0).reshape(-1, 3)[conns - c0]
    runs = cells_ranges(owned)
    jac_g = [ctx.jacobian_rows(f, f + n) for f, n in runs]

    def oracle(variant="exact", seed=None, ulps=1):
        ob = OracleBulk(model, sub_grid, variant=variant)
        if seed is not None:
            ob.set_nudge_seed(seed, ulps)
        ob.load({inv[f]: v for f, v in inputs.items()})
        ob.update_property()
        return ob

    ob = oracle()
    pe_o = ob.a["phaseExist"].reshape(-1, 3)[:no].astype(bool)
    pe_g = got["PHASE_EXIST"].reshape(-1, 3).astype(bool)
    # cells whose phase labels the reference algorithm itself changes when its
    # transcendentals round one ulp differently (near a phase boundary): there
    # the GPU's libm may decide either way
    nudged = []
    sensitive = np.zeros(no, bool)
    for seed, ulps in NUDGES:
        nb_ = oracle("ulp", seed, ulps)
        pe_n = nb_.a["phaseExist"].reshape(-1, 3)[:no].astype(bool)
        sensitive |= np.any(pe_n != pe_o, axis=1)
        nudged.append({k: nb_.a[v].reshape(cells.size, -1)[:no].copy() for k, v in FLASH_KEYS.items()})
        del nb_
    mismatch = np.any(pe_o != pe_g, axis=1)
    label_mismatch = int(mismatch.sum())
    unexplained = int(np.sum(mismatch & ~sensitive))
    keep = ~(mismatch | sensitive)
    ref = {k: ob.a[v].reshape(cells.size, -1)[:no][keep] for k, v in FLASH_KEYS.items()}
    errs = flash_errors({k: np.asarray(got[k]).reshape(no, -1)[keep] for k in FLASH_KEYS}, ref, pe_o[keep], nc)
    sens = {}
    for nz in nudged:
        for k, v in flash_errors({k: nz[k][keep] for k in FLASH_KEYS}, ref, pe_o[keep], nc).items():
            sens[k] = max(sens.get(k, 0.0), v)
    tol = {k: max(REL_TOL, LIBM_FACTOR * sens.get(k, 0.0)) for k in FLASH_KEYS}
    # per cell: the GPU's error against the oracle's own one-ulp sensitivity
    got_k = {k: np.asarray(got[k]).reshape(no, -1)[keep] for k in FLASH_KEYS}
    e_cell = cell_errors(got_k, ref, pe_o[keep], nc)
    s_cell = np.zeros_like(e_cell)
    for nz in nudged:
        s_cell = np.maximum(s_cell, cell_errors({k: nz[k][keep] for k in FLASH_KEYS}, ref, pe_o[keep], nc))
    above = e_cell > REL_TOL
    explained = above & (e_cell <= LIBM_FACTOR * s_cell)
    # cells the six runs leave unexplained: their sensitivity from 80 more
    # perturbation patterns (40 seeds at one ulp, 40 at two), the oracle run on
    # those cells alone (a cell's flash depends on its own inputs only).  A
    # rare branch of the equilibrium (an iteration more or less near a
    # tolerance) shows in a few of those runs only.
    cand = np.nonzero(above & ~explained)[0]
    unexplained_cells = 0
    if cand.size:
        w = np.nonzero(keep)[0][cand]
        unexplained_cells = recheck_cells(
            model, (sub_grid.v[w], sub_grid.depth[w], sub_grid.poro_init[w]),
            {inv[f]: np.asarray(v).reshape(cells.size, -1)[w].ravel() for f, v in inputs.items()},
            {k: v[cand] for k, v in got_k.items()})
    if dump:
        idx = np.nonzero(keep)[0][above]
        np.savez_compressed(dump, cells=owned[idx], e_cell=e_cell[above], s_cell=s_cell[above],
                            **{"in/" + f: np.asarray(v).reshape(cells.size, -1)[idx] for f, v in inputs.items()},
                            **{"gpu/" + k: np.asarray(got[k]).reshape(no, -1)[idx] for k in FLASH_KEYS},
                            **{"oracle/" + k: ob.a[v].reshape(cells.size, -1)[idx] for k, v in FLASH_KEYS.items()})
    # residual and Jacobian of the oracle from the GPU's post-flash state
    post = {f: get_cells(ctx, f, cells) for f in ORACLE_FIELDS}
    oc = OracleBulk(model, sub_grid)
    oc.load({inv[f]: v for f, v in post.items()})
    oc.cal_res(DT)
    rp, col, val = oc.assemble(DT)
    up_mismatch = int(np.sum(cells[oc.conn["upblock"].reshape(-1, 3)] != up_g))
    # rows of perforated cells also hold their wells' terms, which the oracle
    # window leaves out (tests/test_gpu_wells_step.py checks those against the
    # reference): they are left out here
    perforated = np.zeros(grid.nb, bool)
    for w in wl.wells(grid):
        perforated[np.asarray(w["cell"])] = True
    plain_rows = ~perforated[owned]
    r_o = oc.res.reshape(cells.size, -1)[:no]
    scale = np.empty_like(r_o)
    scale[:, 0] = post["ROCKVP"][:no]
    scale[:, 1:] = post["NT"][:no, None]
    res_err = float(np.max((np.abs(res_g - r_o) / scale)[plain_rows]))
    bs = (nc + 1) ** 2
    jac_err, pattern_mismatch, row = 0.0, 0, 0
    for (f, n), (grp, gcol, gval) in zip(runs, jac_g):
        for q in range(n):
            if plain_rows[row]:
                a = gval[grp[q] * bs:grp[q + 1] * bs]
                b = val[rp[row] * bs:rp[row + 1] * bs]
                if not np.array_equal(gcol[grp[q]:grp[q + 1]], cells[col[rp[row]:rp[row + 1]]]):
                    pattern_mismatch += 1
                jac_err = max(jac_err, float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)))
            row += 1
    flash_ok = all(errs[k] <= tol[k] for k in errs)
    ok = (unexplained == 0 and up_mismatch == 0 and pattern_mismatch == 0 and flash_ok and res_err <= REL_TOL
          and jac_err <= REL_TOL and unexplained_cells == 0)
    return {"window": f"{no:,} owned cells with {ghost.size:,} ghost cells, {conns.size:,} connections",
            "against": "oracle (CPU restatement pinned to the reference) from the timed step's own inputs",
            "label_mismatch_cells": label_mismatch,
            "libm_sensitive_cells": int(sensitive.sum()),
            "label_mismatch_outside_libm_sensitive_cells": unexplained,
            "flash_values_compared_on": f"{int(keep.sum()):,} cells (the others' labels differ or are libm-sensitive)",
            "upwind_mismatches": up_mismatch,
            "residual_and_jacobian_rows_compared": int(plain_rows.sum()),
            "perforated_rows_left_out": int((~plain_rows).sum()),
            "jacobian_pattern_mismatch_rows": pattern_mismatch,
            "flash_cells_above_1e-10": int(above.sum()),
            "libm_sensitivity_runs": [f"seed {sd}, {u} ulp" for sd, u in NUDGES],
            "flash_cells_above_1e-10_within_4x_their_libm_sensitivity": int(explained.sum()),
            "flash_cells_rechecked_with_80_more_runs": int(cand.size),
            "flash_cells_unexplained": unexplained_cells,
            "flash_max_rel_err": {k: float(f"{v:.3g}") for k, v in errs.items()},
            "flash_tolerance": {k: float(f"{v:.3g}") for k, v in tol.items()},
            "residual_max_rel_err": res_err, "jacobian_max_rowwise_rel_err": jac_err, "tolerance": REL_TOL,
            "pass": bool(ok), "seconds": round(time.perf_counter() - t0, 1)}


# ------------------------------------------------------------ CPU legs ---
def cpu_state(wl):
    """The CPU sample at the input of the timed Newton iteration, built on the
    host by the oracle from the same seeds: (OracleBulk, saved state, cells)."""
    from opencaeporox_gb300 import synthetic
    from oracle.pyoracle import OracleBulk
    g, cells, desc = wl.cpu_sample()
    n_total = int(np.prod(wl.dims))
    first = int(cells[0])
    st = synthetic.comp_initial_state(g, wl.ncomp, wl.seed, n_total=n_total, first=first)
    ob = OracleBulk(wl.model(), g)
    ob.load(st)
    ob.update_property()
    scale = ob.a["rockVp"] / ob.a["vf"]
    Ni = (st["Ni"].reshape(g.nb, -1) * scale[:, None]).ravel()
    st.update(Ni=Ni, lNi=Ni, Nt=Ni.reshape(g.nb, -1).sum(axis=1))
    ob.load(st)
    ob.a["skip_flag"][:] = 0
    ob.update_property()
    ob.cal_res(DT)
    ob.a["lNi"][:] = ob.a["Ni"]
    u1, u2 = synthetic.ptn_updates(Ni, g.nb, wl.ncomp, wl.seed, n_total=n_total, first=first)
    ob.newton_update(u1, DSMAX)
    ob.update_property()
    ob.cal_res(DT)
    ob.newton_update(u2, DSMAX)
    return ob, {k: v.copy() for k, v in ob.a.items()}, g.nb, desc


def cpu_step(ob, saved):
    for k, v in saved.items():
        ob.a[k][:] = v
    t0 = time.perf_counter()
    ob.update_property()
    ob.cal_res(DT)
    ob.assemble(DT)
    return time.perf_counter() - t0


def cpu_baseline(wl, seconds=12.0, max_reps=50):
    """The reference algorithm (oracle port, C, OpenMP over cells) on the host
    cores: the timed Newton iteration on the workload's CPU sample."""
    ob, saved, n, desc = cpu_state(wl)
    times = []
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end or len(times) < 2:
        times.append(cpu_step(ob, saved))
        if len(times) >= max_reps:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return n / statistics.median(times), cores, (f"{desc}: the timed Newton iteration, {len(times)} repetitions, "
                                                 "median; the port runs at 0.96x the reference's own build per core "
                                                 "(oracle/cpu_side_by_side.py, one thread each, x86)")


def fp64_peak(device=0):
    """FP64 peak of this GPU (TFLOP/s), measured by the library's DFMA-chain
    probe: the measured-peaks file carries HBM and bf16 figures only."""
    from opencaeporox_gb300.fim import measure_fp64_tflops
    return max(measure_fp64_tflops(device, 20000) for _ in range(3))


# FP64 operations of the flash per cell of each workload's timed Newton
# iteration: 2 x DFMA + DADD + DMUL thread-level instructions of the plain
# one-thread-per-cell kernel (ncu smsp__sass_thread_inst_executed_op_{dfma,
# dadd,dmul}_pred_on.sum over one launch, libm internals included) divided by
# the cells of that launch; the batched form does the same algorithmic work in
# another order.  fim: 223.4 M DFMA, 121.7 M DADD, 142.7 M DMUL over 36,000
# cells (profiles/k_flash_comp_comp6_36k.md).  large: the same counts on the
# workload's generator at 200 x 200 x 25 = 1,000,000 cells
# (profiles/k_flash_comp_large_1m.md).
FLASH_FP64_FLOP_PER_CELL = {"fim": (2 * 223408633 + 121682495 + 142721273) / 36000,
                            "large": (2 * 12605259882 + 6716773959 + 8614568226) / 1000000}
# DRAM bytes (read + write) per cell of one fused-flash launch on the workload
# (ncu dram__bytes_read.sum + dram__bytes_write.sum of k_flash_fused); the large
# workload's from its generator at 250,000 cells (the traffic, almost all of it
# the thread frames' local memory, grows with the cells processed)
FLASH_DRAM_BYTES_PER_CELL = {"fim": (155323904 + 250230016) / 36000,
                             "large": (2463918000 + 3046760000) / 250000}


def conn_jac_flops(nconn, nc):
    """Algorithmic FP64 flops of k_jac_conn: per side of a connection, for
    every phase, the np saturation and nc composition rows of dSec_dPri
    scaled into W_j (np (np + nc) (nc + 1) FMA), the nc component rows
    summed over phases (np nc (nc + 1)) and the upwind phase's own
    composition rows (nc (nc + 1)); 2 flops an FMA, two sides (all phases
    flowing: an upper bound of the branches taken)."""
    np_, ncol = 3, nc + 1
    per_side = ncol * (np_ * (np_ + nc) + np_ * nc + nc)
    return 2 * 2 * per_side * nconn


def rows_bytes(nb, nconn, nc, nnzb):
    """Algorithmic HBM bytes of k_jac_rows: the connection blocks read once
    (2 per connection), the accumulation inputs of the diagonal (v, poroP,
    vfP, vfi), the row-incidence lists, and the block-CSR values written."""
    bs = (nc + 1) ** 2
    return 2 * nconn * bs * 8 + nb * 8 * (3 + nc) + (nb + 1 + 2 * nconn) * 4 + nnzb * bs * 8


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


class Ranks:
    """torchrun ranks: one replica of the workload per GPU (each rank runs the
    whole Newton step of its own grid); host barrier and max over ranks
    through torch.distributed (gloo)."""

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


TUNE_SPACE_LARGE = {"fused_blocks": ("sms", 2, 4), "fused_coop_blocks": (0,), "flash_budget": (32, 48, 64),
                    "predefer": (96, 192), "coop_cells": (1216, 4864), "coop_blocks": (608,), "block_cell": (128,),
                    "pre_blocks": (0,)}


def log(msg):
    print(msg, file=sys.stderr, flush=True)


def run_fim(args, wl, rt, local, rank, world):
    """The FIM Newton-step bench of one workload: plain form, then the
    batched form (autotuned, graph-replayed), e2e, parity, rooflines, CPU
    baseline."""
    ranks = Ranks(world)
    model = wl.model()
    grid = wl.grid()
    nb = grid.nb
    large = wl.key == "large"
    flush_bytes = 512 << 20
    flush = (rt.malloc(flush_bytes), flush_bytes)
    # plain form: fewer steps on the large grid, where one takes seconds
    # the 4,000,000-cell configuration recomputes the flash derivatives where
    # they are used instead of storing them; the others store them
    recompute = args.flash_der == "recompute" or (args.flash_der is None and large)
    p_steps, p_warm = (min(args.steps, 3), 1) if large else (args.steps, args.warmup)
    plain_ms, plain_prof = float("nan"), {}
    if not args.no_plain:
        t0 = time.perf_counter()
        ctx0, _ = prepare(wl, model, grid, 0, local, recompute)
        log(f"{wl.key}: plain form set up in {time.perf_counter() - t0:.1f} s")
        ranks.barrier(rt)
        t_plain, _ = time_device(ctx0, rt, p_steps, p_warm, flush)
        ranks.barrier(rt)
        plain_ms = ranks.max(statistics.median(t_plain))
        plain_prof = stage_profile(ctx0, rt, flush)
        log(f"{wl.key}: plain step {plain_ms:.1f} ms")
        ctx0.close()
        del ctx0
    # batched form
    t0 = time.perf_counter()
    ctx, u2 = prepare(wl, model, grid, 1, local, recompute)
    log(f"{wl.key}: batched form set up in {time.perf_counter() - t0:.1f} s")
    for kv in args.param:
        k, v = kv.split("=")
        ctx.set_param(k, int(v))
    tuned = None
    if not args.no_tune:
        from opencaeporox_gb300 import autotune
        tuned = autotune.tune(ctx, DT, slot=0, space=TUNE_SPACE_LARGE if large else None, rounds=1 if large else 2,
                              reps=1 if large else 2)
        log(f"{wl.key}: tuned {({k: v for k, v in tuned.items() if k != 'trials'})}")
    clocks = ClockSampler(local)
    time.sleep(0.5)  # the sampler's first samples come after its start-up
    ranks.barrier(rt)
    clocks.start()
    tb, launches = time_device(ctx, rt, args.steps, args.warmup, flush)
    clocks.end()
    ranks.barrier(rt)
    ck = clocks.stop()
    ms = ranks.max(statistics.median(tb))
    log(f"{wl.key}: batched step {ms:.1f} ms")
    prof = stage_profile(ctx, rt, flush)
    ranks.barrier(rt)
    e2e_t, h2d, d2h = time_e2e(ctx, rt, args.steps, args.warmup, flush, u2, wl.adjoint)
    ranks.barrier(rt)
    e2e_ms = ranks.max(statistics.median(e2e_t))
    rt.free_pinned()
    log(f"{wl.key}: e2e step {e2e_ms:.1f} ms")
    par = None
    if rank == 0 and not args.no_parity:
        par = parity(ctx, wl, model, grid, dump=args.parity_dump)
        log(f"{wl.key}: parity {par}")
    value = nb / (ms * 1e-3) * world
    plain = nb / (plain_ms * 1e-3) * world
    fp64 = fp64_peak(local)
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    flash_ms = prof["flash"][0]
    fused = ctx.get_param("fused_blocks") > 0
    flop_cell = FLASH_FP64_FLOP_PER_CELL.get(wl.key)
    dram_cell = FLASH_DRAM_BYTES_PER_CELL.get(wl.key)
    roof = {"kernel": ("k_flash_fused + k_flash_post" if fused else "k_flash_budget + k_flash_pe_coop + k_flash_post")
                      + " (flash stage of the batched step)", "bound": "fp64", "unit": "TFLOP/s",
            "peak": fp64, "peak_source": "measured (DFMA-chain probe of this library, best of 3)",
            "flop_per_cell": flop_cell, "achieved": None, "frac": None,
            "traffic": dram_cell * nb if dram_cell else None}
    if flop_cell:
        roof["achieved"] = flop_cell * nb / (flash_ms * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / fp64
    # the assembly's two kernels, each against its own bound
    cflop = conn_jac_flops(ctx.nconn, ctx.nc)
    conn_ms = prof["jac_conn"][0]
    roof_conn = {"kernel": ("k_dsec_slab + k_jac_side (connection blocks, dSec_dPri recomputed per slab; the "
                            "recomputation's flops not counted)") if recompute else "k_jac_conn (connection blocks)",
                 "bound": "fp64", "unit": "TFLOP/s",
                 "algorithmic_flops": cflop, "achieved": cflop / (conn_ms * 1e-3) / 1e12, "peak": fp64,
                 "peak_source": "measured (DFMA-chain probe of this library, best of 3)"}
    roof_conn["frac"] = roof_conn["achieved"] / fp64
    rbytes = rows_bytes(nb, ctx.nconn, ctx.nc, ctx_nnz(ctx))
    rows_ms = prof["jac_rows"][0]
    roof_rows = {"kernel": "k_jac_rows (block rows from the connection blocks)", "bound": "hbm", "unit": "GB/s",
                 "algorithmic_bytes": rbytes, "achieved": rbytes / (rows_ms * 1e-3) / 1e9, "peak": hbm,
                 "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "of fallback 6800"}
    roof_rows["frac"] = roof_rows["achieved"] / (hbm or 6800.0)
    dom = max(prof, key=lambda k: prof[k][0] if k not in ("flash_budget", "flash_post", "flash_order") else -1)
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": wl.description, "cells": nb, "connections": int(grid.nconn),
                       "l2": "flushed between steps (512 MiB memset); inputs larger than L2" if large
                       else "flushed between steps (512 MiB memset)", "variant": "batched",
                       "flash_derivatives": "recomputed where used (dSec_dPri not stored)" if recompute
                       else "stored (dSec_dPri)", "device_bytes": ctx.get_param("device_bytes"),
                       "parallelism": f"replicas x{world} (one grid per GPU)"},
            "plain_value": plain, "plain_ms_per_step": plain_ms, "plain_steps": p_steps,
            "batched_over_plain": value / plain,
            "plain_stages_ms": {k: round(v[0], 4) for k, v in plain_prof.items()},
            "stages_ms": {k: round(v[0], 4) for k, v in prof.items()}, "dominant_stage": dom,
            "roofline": roof, "roofline_conn_jacobian": roof_conn, "roofline_rows": roof_rows,
            "fp64_peak_tflops": fp64,
            "batched": {k: ctx.get_param(k) for k in ("flash_budget", "coop_blocks", "block_cell", "predefer",
                                                      "coop_cells", "pre_blocks", "cell_blocks", "fused_blocks",
                                                      "fused_coop_blocks", "split_refill")},
            "autotune": None if tuned is None else {k: v for k, v in tuned.items() if k != "trials"},
            "clocks": ck, "gpu_launches": launches,
            "e2e": {"value": nb / (e2e_ms * 1e-3) * world, "unit": "cells/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "parity": par}
    line["batched"].update(deferred_cells=ctx.get_param("deferred"), predeferred_cells=ctx.get_param("predeferred"),
                           level=ctx.get_param("level"))
    ctx.close()
    if rank == 0 and world == 1 and os.environ.get("OCPX_BENCH_NO_CPU") != "1":
        v, cores, sample = cpu_baseline(wl)
        line["cpu_baseline"] = {"value": v, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line))
    ranks.close()


def reference_arm(args, wl):
    """The reference algorithm on the host cores (the oracle port, OpenMP over
    cells; the reference's own sources are not on the GPU machine): each step
    the timed Newton iteration on the workload's CPU sample."""
    from oracle import build as ob_build
    ob_build.build()
    ob, saved, n, desc = cpu_state(wl)
    times = []
    for k in range(args.warmup + args.steps):
        t = cpu_step(ob, saved)
        if k >= args.warmup:
            times.append(t)
    v = n / statistics.median(times)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = (f"{desc}: the timed Newton iteration per step, median of {len(times)}; the port runs at 0.96x the "
              "reference's own build per core (oracle/cpu_side_by_side.py, one thread each, x86)")
    return {"metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": wl.description, "cells": int(np.prod(wl.dims))}, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner (library defaults)")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the timed step")
    ap.add_argument("--param", action="append", default=[],
                    help="name=value: a library parameter of the batched form, set before tuning (repeatable)")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain form's leg (to profile the batched step alone)")
    ap.add_argument("--parity-dump", default=None, help="write the cells above 1e-10 in the parity check to this .npz")
    ap.add_argument("--flash-der", default=None, choices=["store", "recompute"],
                    help="keep dSec_dPri, or recompute it where it is used (ocpx_options); default: "
                         "recompute on the large workload, store on the others")
    ap.add_argument("--workload", default="large", choices=["large", "fim", "flash-stress"],
                    help="large: the 4,000,000-cell Newton step with the adjoint (default); fim: the 36,000-cell "
                         "Newton step; flash-stress: 1M independent flashes")
    ap.add_argument("--large-dims", type=lambda v: tuple(int(x) for x in v.split(",")), default=(200, 200, 100),
                    help="grid of the large workload, NX,NY,NZ (default 200,200,100)")
    ap.add_argument("--cpu-layers", type=int, default=5,
                    help="layers of the large workload's grid in the CPU baseline's sample (default 5)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    wl = {"large": LargeWorkload, "fim": FimWorkload}.get(args.workload, FimWorkload)(args)

    if args.impl == "reference":
        if rank != 0:
            return
        if args.workload == "flash-stress":
            print(json.dumps({"impl": "reference", "unavailable": "the flash-stress workload has no CPU arm"}))
            return
        print(json.dumps(reference_arm(args, wl)))
        return

    from opencaeporox_gb300 import build as gb
    gb.build()
    rt = Cudart()
    rt.rt.cudaSetDevice(local)
    if args.workload == "flash-stress":
        if rank == 0:
            print(json.dumps(flash_stress(args, rt, local)))
        return
    run_fim(args, wl, rt, local, rank, world)


if __name__ == "__main__":
    main()
