"""Launch-shape autotuner of the batched FIM step.

The batched flash has knobs that change only how the work is laid out on
the GPU, never the results: the per-cell work budget after which a cell's
phase equilibrium moves to the warp-cooperative kernel, whether cells that
were expensive in their last flash go there at once (concurrently with the
per-cell kernel), the number of blocks of that kernel, and the block size of
the per-cell kernels.  The
tuner times the flash stage of real Newton iterations (CUDA events recorded
on the context stream by the library's stage profiler), restoring the same
device checkpoint before every trial, and keeps the fastest setting.
"""
from __future__ import annotations

import itertools

DEFAULT_BUDGETS = (24, 32, 48, 64, 96, 128, 192)


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


def tune(ctx, dt: float, slot: int = 0, budgets=DEFAULT_BUDGETS, coop_blocks=None, block_cells=(128,),
         predefer=(0, 1, 2, 4, 8), reps: int = 2) -> dict:
    """Try every combination on the state saved in checkpoint `slot` (the
    caller saves it) and leave the context set to the fastest one.  Returns
    {"flash_budget", "coop_blocks", "block_cell", "predefer", "flash_ms", "trials"}.
    predefer: pre-deferral thresholds as multiples of the budget (0: off).
    The context must use the batched variant."""
    if coop_blocks is None:
        coop_blocks = (ctx.get_param("coop_blocks"),)
    trials = []
    for budget, blocks, bc, pre in itertools.product(budgets, coop_blocks, block_cells, predefer):
        ctx.set_param("flash_budget", budget)
        ctx.set_param("coop_blocks", blocks)
        ctx.set_param("block_cell", bc)
        ctx.set_param("predefer", pre * budget)
        trials.append((_flash_ms(ctx, dt, slot, reps), budget, blocks, bc, pre * budget))
    ms, budget, blocks, bc, pre = min(trials)
    ctx.set_param("flash_budget", budget)
    ctx.set_param("coop_blocks", blocks)
    ctx.set_param("block_cell", bc)
    ctx.set_param("predefer", pre)
    ctx.checkpoint(slot, restore=True)
    return {"flash_budget": budget, "coop_blocks": blocks, "block_cell": bc, "predefer": pre, "flash_ms": ms,
            "trials": [{"flash_ms": t[0], "flash_budget": t[1], "coop_blocks": t[2], "block_cell": t[3],
                        "predefer": t[4]} for t in trials]}
