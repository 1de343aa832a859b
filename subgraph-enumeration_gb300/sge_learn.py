"""Learned planning: record per-plan GPU runtimes, train the MLP scorer, and
measure its regret against the cost model.

The scorer replaces the cost the reference's optimizer minimises over
candidate plans (computeOrderCost / optCostOrder, plan/optimizer.cpp:319-577).
The data it learns from is recorded by this engine itself: for each training
pattern, the cost model's shortlist of candidate plans is run on a sample of
the root edges (root_stride) and the kernel time is the label (log ms).
The cost model stays: it builds the shortlist, and it is the baseline the
learned choice is judged against (regret = time of the chosen plan ÷ time of
the best measured candidate).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

import sge

WEIGHTS = Path(__file__).resolve().parent / "scorer" / "mlp_weights.npz"


@dataclass
class Records:
    """One row per (pattern, candidate plan)."""
    pattern: list = field(default_factory=list)    # pattern id
    cand: list = field(default_factory=list)       # rank of the candidate in the cost model's shortlist
    x: list = field(default_factory=list)          # features (SGE_FEATURES floats)
    ms: list = field(default_factory=list)         # kernel ms on the root sample
    count: list = field(default_factory=list)      # count on the root sample (for consistency checks)

    def arrays(self):
        return (np.array(self.pattern, np.int32), np.array(self.cand, np.int32),
                np.array(self.x, np.float32).reshape(-1, sge.SGE_FEATURES), np.array(self.ms, np.float64),
                np.array(self.count, np.uint64))

    def save(self, path):
        p, c, x, ms, cnt = self.arrays()
        np.savez_compressed(path, pattern=p, cand=c, x=x, ms=ms, count=cnt)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        r = cls()
        r.pattern, r.cand, r.x, r.ms, r.count = (d["pattern"].tolist(), d["cand"].tolist(), d["x"].tolist(),
                                                 d["ms"].tolist(), d["count"].tolist())
        return r


def record(engine: "sge.Engine", stats, patterns, shortlist: int = 12, stride: int = 8, pattern_offset: int = 0,
           time_budget_s: float = 5.0, iep: bool = True, rec: Records | None = None, candidates_fn=None,
           sample: dict | None = None) -> Records:
    """Runs the cost model's shortlist of every pattern on every stride-th root
    (the same roots for all candidates of a pattern) and records kernel times.
    candidates_fn(p, stats, shortlist) replaces the shortlist (e.g. candidates
    sharing one symmetry scheme and root edge); sample (Engine.count keyword
    arguments) replaces the stride sample."""
    rec = rec or Records()
    for pi, p in enumerate(patterns):
        cands = candidates_fn(p, stats, shortlist) if candidates_fn else sge.candidates(p, stats, iep=iep, cap=shortlist)
        off = (pattern_offset + pi) % stride
        opts = dict(sample) if sample is not None else dict(root_stride=stride, root_offset=off)
        counts = []
        for ci, b in enumerate(cands):
            try:
                c, _, st = engine.count([b], time_budget_s=time_budget_s, **opts)
                ms = st["kernel_ms"]
            except sge.SgeError as e:
                if e.status_name != "TIMEOUT":
                    raise
                c, ms = [0], time_budget_s * 1e3 * 2  # censored: slower than the budget
            counts.append(c[0])
            rec.pattern.append(pattern_offset + pi)
            rec.cand.append(ci)
            rec.x.append(sge.features(b, stats).tolist())
            rec.ms.append(ms)
            rec.count.append(c[0])
    return rec


def labels(ms: np.ndarray) -> np.ndarray:
    return np.log(np.maximum(ms, 1e-3)).astype(np.float32)


def train(rec: Records, hidden: int = 128, epochs: int = 300, lr: float = 2e-3, seed: int = 0,
          mlp: "sge.MLP | None" = None) -> "sge.MLP":
    _, _, x, ms, _ = rec.arrays()
    mlp = mlp or sge.MLP(sge.SGE_FEATURES, hidden, seed)
    mlp.train(x, labels(ms), epochs=epochs, batch=128, lr=lr, seed=seed)
    return mlp


def regret(rec: Records, mlp: "sge.MLP | None" = None, bf16: bool = True) -> dict:
    """Geometric-mean regret of the cost model's pick (shortlist rank 0) and of
    the MLP's pick, over the patterns in rec."""
    pid, cand, x, ms, _ = rec.arrays()
    pred = mlp.forward(x, bf16=bf16) if mlp is not None else None
    cm, ml = [], []
    for p in np.unique(pid):
        sel = np.nonzero(pid == p)[0]
        best = ms[sel].min()
        cm.append(ms[sel[np.argmin(cand[sel])]] / best)
        if pred is not None:
            ml.append(ms[sel[np.argmin(pred[sel])]] / best)
    g = lambda v: float(math.exp(np.mean(np.log(v)))) if v else None
    return {"patterns": int(len(np.unique(pid))), "cost_model": g(cm), "learned": g(ml),
            "cost_model_max": float(max(cm)) if cm else None, "learned_max": float(max(ml)) if ml else None}


def save_mlp(mlp: "sge.MLP", path: Path = WEIGHTS) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, params=mlp.get_params(), hidden=mlp.hidden, in_dim=mlp.in_dim)


def load_mlp(path: Path = WEIGHTS, device: int = 0) -> "sge.MLP":
    d = np.load(path)
    mlp = sge.MLP(int(d["in_dim"]), int(d["hidden"]), 0, device)
    mlp.set_params(d["params"])
    return mlp
