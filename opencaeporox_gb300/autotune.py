"""Launch-shape autotuner of the batched FIM step.

The batched flash has knobs that change only how the work is laid out on
the GPU, never the results:

- the per-cell work budget after which a cell's phase equilibrium moves to
  the warp-cooperative kernel;
- the pre-deferral threshold (cells that were expensive in their last flash
  go there at once, concurrently with the per-cell kernel);
- the adaptive cap on how many cells the cooperative kernel gets;
- the number of blocks of that kernel;
- the block size of the per-cell kernels.

The tuner times the flash stage of real Newton iterations.  The times are
CUDA events recorded on the context stream by the library's stage profiler,
and the same device checkpoint is restored before every trial.  It searches
one parameter at a time from the current best point (coordinate descent,
two rounds by default) and leaves the context set to the fastest point found.
"""
from __future__ import annotations

DEFAULT_SPACE = {
    "flash_budget": (24, 32, 48, 64, 96, 128, 192),
    "predefer": (0, 48, 96, 192, 384),
    "coop_cells": (0, 608, 1216, 2432),
    "coop_blocks": (152, 304, 608),
    "block_cell": (64, 128),
}


def _flash_ms(ctx, dt: float, slot: int, reps: int) -> float:
    best = float("inf")
    for _ in range(reps):
        ctx.checkpoint(slot, restore=True)
        ctx.profile(True)
        ctx.enqueue_step(dt)
        ctx.step_report()
        ms, n = ctx.profile_read()["flash"]
        ctx.profile(False)
        if n:
            best = min(best, ms / n)
    return best


def tune(ctx, dt: float, slot: int = 0, space: dict | None = None, rounds: int = 2, reps: int = 2) -> dict:
    """Tune on the state saved in checkpoint `slot` (the caller saves it).
    `space` maps parameter names to candidate values (DEFAULT_SPACE entries
    for the names it omits; a one-value tuple fixes a parameter).  Returns
    the best point with its flash time and the list of trials.  The context
    must use the batched variant."""
    sp = dict(DEFAULT_SPACE)
    sp.update(space or {})
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
            cache[key] = _flash_ms(ctx, dt, slot, reps)
            trials.append(dict(p, flash_ms=cache[key]))
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
    return dict(point, flash_ms=best, trials=trials)
