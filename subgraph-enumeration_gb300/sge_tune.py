"""Autotuner for a batched launch.

Chooses, from short sampled runs of the batch itself:
  - per launch: whether to pin the root's lists in per-warp shared-memory
    tables (more shared memory per warp, fewer warps resident);
  - per plan (pattern) and degree bucket: the heavy-root threshold, i.e. the
    degree bucket of roots deferred to the split launch, and how finely each
    heavy root is split (level-3 parts per task), plus whether the plan probes
    through the hub bitmaps.
Per-plan costs come from sge_count_plan_times: the warp-milliseconds each
plan's roots took inside the batched launch, so a plan is judged where it
runs, beside the others.  Counts never depend on the choices; the tuner
checks that every run returned the same counts.

The reference has no counterpart: its OpenMP split is one task per root
(matching/parallel.cpp:1270-1273).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import sge

# candidate per-plan settings: (heavy threshold, level-3 parts, binary search only)
CANDIDATES = [(0, 0, 0), (64, 0, 0), (256, 0, 0), (256, 32, 0), (256, 0, 1)]


@dataclass
class Tuning:
    pin_tables: int
    plans: list = field(default_factory=list)   # sge.PlanTuning per plan
    choice: list = field(default_factory=list)  # index into CANDIDATES per plan
    tuning_ms: float = 0.0                     # kernel time spent tuning
    runs: int = 0


def tune(engine: "sge.Engine", plans, sample: dict, sub: int = 4) -> Tuning:
    """Tunes plans for runs on `sample` (Engine.count keyword arguments:
    root_stride, root_offset, root_max_degree).  The tuning runs use every
    sub-th root edge of the sample."""
    opts = dict(sample)
    opts["root_stride"] = sample.get("root_stride", 1) * sub
    spent, runs = 0.0, 0
    ref = None
    # launch level: shared-memory tables or more resident warps
    best_pin, best_ms = 0, None
    for pin in (0, 1, 2):
        c, _, st = engine.count(plans, pin_tables=pin, **opts)
        spent += st["kernel_ms"]
        runs += 1
        ref = ref if ref is not None else c
        assert c == ref, "counts changed with the shared-memory tables"
        if best_ms is None or st["kernel_ms"] < best_ms:
            best_pin, best_ms = pin, st["kernel_ms"]
    # per plan: every candidate setting once for the whole batch; each plan
    # keeps the setting under which its own roots took the least warp time
    busy = []
    for thr, p3, nohub in CANDIDATES:
        tun = [sge.PlanTuning(thr, p3, nohub) for _ in plans]
        c, _, st = engine.count(plans, pin_tables=best_pin, tuning=tun, plan_times=True, **opts)
        spent += st["kernel_ms"]
        runs += 1
        assert c == ref, "counts changed with the plan tuning"
        busy.append(st["plan_busy_ms"])
    choice = [min(range(len(CANDIDATES)), key=lambda k: busy[k][i]) for i in range(len(plans))]
    return Tuning(pin_tables=best_pin, plans=[sge.PlanTuning(*CANDIDATES[k]) for k in choice], choice=choice,
                  tuning_ms=spent, runs=runs)
