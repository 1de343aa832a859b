"""Plan blobs for bench.py's CPU reference arm (tests/golden/bench_plans.npz).

The reference arm times the CPU implementation of the hot path and must not
load the library, so the plans it runs are recorded here ahead of time, from
the library's planner on the same seeded graphs (their statistics are stored
beside them, and a test re-plans from those statistics and compares):
  chunglu7100_*: the 12 plans of the Chung-Lu n=7,100 workload (house, K5-e,
                 8-edge near-5-clique x WCOJ / WCOJ+IEP / exploration /
                 exploration+IEP), plus for the IEP modes the cheapest
                 multi-level-tail plan as an alternative the arm may prefer;
  rmat22_*:      the cost model's plans for the 78 seeded 7-vertex patterns on
                 R-MAT 2^22 / 64M edges, each with the canonical symmetry
                 sequence and root edge bench.py samples on.
Run:  python tests/golden/make_bench_plans.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "subgraph-enumeration_gb300"))
sys.path.insert(0, str(REPO))
import sge  # noqa: E402
import bench  # noqa: E402


def stats_array(st) -> np.ndarray:
    return np.frombuffer(bytes(memoryview(st)), np.uint8).copy()


def blobs(plans) -> np.ndarray:
    return np.stack([np.frombuffer(b.to_bytes(), np.uint8) for b in plans])


def main() -> None:
    out = {}
    g = sge.gen_chung_lu(**{k: bench.CL_GRAPH[k] for k in ("n", "m", "gamma", "max_deg", "seed")})
    st = g.stats()
    plans, alts, names = [], [], []
    for pname, (k, edges) in bench.CL_PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        for mname, expl, iep in bench.CL_MODES:
            b = sge.plan(p, st, iep=iep, exploration=expl)
            alt = b
            if iep:
                multi = [c for c in sge.candidates(p, st, iep=True, exploration=expl, cap=4096) if c.tail_len >= 2]
                if multi:
                    alt = min(multi, key=lambda c: c.est_cost)
            plans.append(b)
            alts.append(alt)
            names.append(f"{pname}/{mname}")
    out["chunglu7100_stats"] = stats_array(st)
    out["chunglu7100_plans"] = blobs(plans)
    out["chunglu7100_alt"] = blobs(alts)
    out["chunglu7100_names"] = np.array(names)
    gs = bench.RMAT22
    off, nb = bench.oracle_graph("rmat22")
    st = sge.DataGraph(off, nb).stats()
    pats = bench.rmat22_patterns(sge)
    out["rmat22_stats"] = stats_array(st)
    out["rmat22_plain"] = blobs([bench.plain_plan(sge, p, st) for p in pats])
    np.savez_compressed(HERE / "bench_plans.npz", **out)
    print("wrote", HERE / "bench_plans.npz", {k: v.shape for k, v in out.items()}, gs)


if __name__ == "__main__":
    main()
