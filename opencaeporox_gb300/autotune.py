"""Launch-shape autotuner of the batched FIM step.

The batched flash has knobs that change only how the work is laid out on
the GPU, never the results:

- the fused single-kernel form against the two-stream one, the fused
  kernel's grid, and how many of its blocks run only cooperative work;
- the per-cell work budget after which a cell's phase equilibrium moves to
  the warp-cooperative kernel;
- the pre-deferral threshold (cells that were expensive in their last flash
  go there at once, concurrently with the per-cell kernel);
- the adaptive cap on how many cells the cooperative kernel gets;
- the number of blocks of that kernel, and whether the pre-deferred cells
  run on SM-exclusive blocks instead (and how many);
- the block size of the per-cell kernels.

The tuner times whole Newton iterations as they run in production: the
step's CUDA graph replayed on the context stream (captured once per trial
point, untimed), from the same device checkpoint every time, bracketed by
stream synchronisations.  The stage profiler is not used for this because
it runs the step eagerly, and the two streams of the batched flash then
overlap differently from the graph.  The tuner searches one parameter at a
time from the current best point (coordinate descent, two rounds by
default) and leaves the context set to the fastest point found.
"""
from __future__ import annotations

import time

DEFAULT_SPACE = {
    "fused_blocks": ("sms", 0, 1, 2, 4),   # multiples of the SM count ("sms" marks the form)
    "fused_coop_blocks": ("sms/8", 0, 2, 3, 4),   # eighths of the SM count
    "flash_budget": (24, 32, 48, 64, 96, 128, 192),
    "predefer": (0, 48, 96, 192, 384),
    "coop_cells": (0, 1216, 4864),
    "coop_blocks": (152, 304, 608),
    "block_cell": (64, 128),
    "pre_blocks": (0, 38, 76),
}


def _step_ms(ctx, dt: float, slot: int, reps: int) -> float:
    from .fim import OcpxError
    ctx.checkpoint(slot, restore=True)
    try:
        ctx.enqueue_step(dt)      # captures the graph of this point
        ctx.synchronize()
    except OcpxError:
        # a point the device cannot run (for instance a cooperative grid that
        # does not fit on it at once): not a candidate
        return float("inf")
    best = float("inf")
    for _ in range(reps):
        ctx.checkpoint(slot, restore=True)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.enqueue_step(dt)
        ctx.synchronize()
        best = min(best, (time.perf_counter() - t0) * 1e3)
    return best


def tune(ctx, dt: float, slot: int = 0, space: dict | None = None, rounds: int = 2, reps: int = 2) -> dict:
    """Tune on the state saved in checkpoint `slot` (the caller saves it).
    `space` maps parameter names to candidate values (DEFAULT_SPACE entries
    for the names it omits; a one-value tuple fixes a parameter).  Returns
    the best point with its step time (ms) and the list of trials.  The context
    must use the batched variant."""
    sp = dict(DEFAULT_SPACE)
    sp.update(space or {})
    n = ctx.get_param("sms")
    for key, unit in (("fused_blocks", "sms"), ("fused_coop_blocks", "sms/8")):
        if key in sp and sp[key] and sp[key][0] == unit:
            # the context's current value first, so it stays unless another point is faster
            cur = ctx.get_param(key)
            scale = n if unit == "sms" else n / 8
            sp[key] = tuple(sorted({int(v * scale) for v in sp[key][1:]} | {cur}, key=lambda v: (v != cur, v)))
    point = {k: ctx.get_param(k) for k in sp}
    for k, cands in sp.items():
        if point[k] not in cands:
            point[k] = cands[0]
    trials = []
    cache = {}

    def run(p):
        key = tuple(sorted(p.items()))
        if key not in cache:
            for k, v in p.items():
                ctx.set_param(k, v)
            cache[key] = _step_ms(ctx, dt, slot, reps)
            trials.append(dict(p, step_ms=cache[key]))
        return cache[key]

    best = run(point)
    for _ in range(rounds):
        for k, cands in sp.items():
            for v in cands:
                p = dict(point, **{k: v})
                t = run(p)
                if t < best:
                    best, point = t, p
    for k, v in point.items():
        ctx.set_param(k, v)
    ctx.checkpoint(slot, restore=True)
    return dict(point, step_ms=best, trials=trials)
