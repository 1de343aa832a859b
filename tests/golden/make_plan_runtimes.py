"""Records the learned scorer's training data on a GPU and trains the shipped
weights.

  python tests/golden/make_plan_runtimes.py OUT_DIR [BUDGET_S]
  python tests/golden/make_plan_runtimes.py --rmat22 OUT_DIR [BUDGET_S]

The second form records the benchmark's own setting (see the end of this
docstring) and retrains the weights on the union of both recordings.

For seeded synthetic patterns (7-vertex, 16-19 edges, and 6-vertex, 11-13
edges; seeds disjoint from every benchmark batch) on seeded R-MAT graphs
(a=.57 b=.19 c=.19; scale 9 with 4,000 edges and scale 10 with 8,000 edges),
the cost model's 8-plan shortlist of each pattern is run over all root edges
and the kernel time recorded (sge_learn.record); every candidate of a pattern
must give the same count.  A candidate past 0.5 s is recorded as censored.
Recording stops after a wall-clock budget (argument 2, seconds).  Writes OUT_DIR/plan_runtimes.npz (the
fixture tests/golden/plan_runtimes.npz) and OUT_DIR/mlp_weights.npz (the
scorer checkpoint subgraph-enumeration_gb300/scorer/mlp_weights.npz), trained
on the patterns marked for training only.
"""
import json
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "subgraph-enumeration_gb300"))
import numpy as np  # noqa: E402

import sge  # noqa: E402
import sge_learn  # noqa: E402


def main(out: Path, budget_s: float):
    out.mkdir(parents=True, exist_ok=True)
    graphs = {"rmat_s9": sge.gen_rmat(9, 4000, seed=5), "rmat_s10": sge.gen_rmat(10, 8000, seed=5)}
    rec = sge_learn.Records()
    meta = {"graphs": {}, "patterns": []}
    pid = 0
    t0 = time.time()
    for gname, g in graphs.items():
        st = g.stats()
        meta["graphs"][gname] = g.fingerprint()
        pats = []
        for i in range(24):
            pats.append(("6v", sge.PatternGraph.random(6, 11 + i % 3, 8000 + i)))
            pats.append(("7v", sge.PatternGraph.random(7, 16 + i % 4, 9000 + i)))
        with sge.Engine(g) as eng:
            for kind, p in pats:
                if time.time() - t0 > budget_s * (0.5 if gname == "rmat_s9" else 1.0):
                    break
                n0 = len(rec.count)
                sge_learn.record(eng, st, [p], shortlist=8, stride=1, pattern_offset=pid, time_budget_s=0.5, rec=rec)
                done = [c for c, ms in zip(rec.count[n0:], rec.ms[n0:]) if ms < 1000.0]
                assert len(set(done)) <= 1, f"candidate plans disagree: {done}"
                meta["patterns"].append({"id": pid, "graph": gname, "kind": kind, "k": p.k,
                                         "edges": p.edges.tolist(), "train": pid % 4 != 3})
                pid += 1
                print(f"{gname} {kind} pattern {pid} recorded ({time.time() - t0:.0f}s)", flush=True)
    rec.save(out / "plan_runtimes.npz")
    (out / "plan_runtimes.json").write_text(json.dumps(meta))
    # shipped weights: trained on the training patterns only
    p, c, x, ms, cnt = rec.arrays()
    train_ids = {m["id"] for m in meta["patterns"] if m["train"]}
    tr = sge_learn.Records()
    for i in range(len(p)):
        if int(p[i]) in train_ids:
            tr.pattern.append(int(p[i])); tr.cand.append(int(c[i])); tr.x.append(x[i].tolist())
            tr.ms.append(float(ms[i])); tr.count.append(int(cnt[i]))
    mlp = sge_learn.train(tr, epochs=400, seed=0)
    sge_learn.save_mlp(mlp, out / "mlp_weights.npz")
    te = sge_learn.Records()
    for i in range(len(p)):
        if int(p[i]) not in train_ids:
            te.pattern.append(int(p[i])); te.cand.append(int(c[i])); te.x.append(x[i].tolist())
            te.ms.append(float(ms[i])); te.count.append(int(cnt[i]))
    print("held-out regret", sge_learn.regret(te, mlp), flush=True)


def split(rec, meta):
    p, c, x, ms, cnt = rec.arrays()
    train_ids = {m["id"] for m in meta["patterns"] if m["train"]}
    tr, te = sge_learn.Records(), sge_learn.Records()
    for i in range(len(p)):
        d = tr if int(p[i]) in train_ids else te
        d.pattern.append(int(p[i])); d.cand.append(int(c[i])); d.x.append(x[i].tolist())
        d.ms.append(float(ms[i])); d.count.append(int(cnt[i]))
    return tr, te


def merge(a, b):
    m = sge_learn.Records()
    for r in (a, b):
        m.pattern += list(r.pattern); m.cand += list(r.cand); m.x += list(r.x); m.ms += list(r.ms)
        m.count += list(r.count)
    return m


def main_rmat22(out: Path, budget_s: float):
    """The benchmark's setting: R-MAT 2^22 / 64M edges (seed 4) built on the
    GPU; 48 random 7-vertex patterns with 16-19 edges (seeds 3000+, disjoint
    from the benchmark's 2000+); per pattern the cost model's 12 cheapest
    candidates under the benchmark's canonical symmetry sequence and root
    edge, each counted on every 4th edge of the benchmark's root sample (the
    same roots and the same count for every candidate).  Pattern ids continue
    after the existing fixture's; every 4th pattern is held out.  Retrains the
    weights on the training patterns of both recordings."""
    sys.path.insert(0, str(REPO))
    import bench
    out.mkdir(parents=True, exist_ok=True)
    old = sge_learn.Records.load(HERE / "plan_runtimes.npz")
    old_meta = json.loads((HERE / "plan_runtimes.json").read_text())
    pid0 = max(old.pattern) + 1
    eng = sge.Engine.rmat_device(22, 64_000_000, seed=4)
    st = eng.graph.stats()
    sample = bench.sample_opts(1, 0, 4)

    def cands(p, stats, cap):
        seq, root = bench.canonical_symmetry(p.k, p.edges)
        return sge.candidates(p, stats, cap=cap, symmetry_seq=seq, root_edge=root)
    rec = sge_learn.Records()
    meta = {"graphs": {"rmat_s22": "R-MAT 2^22 / 64M, seed 4, built on the GPU"}, "patterns": [],
            "sample": {k: v for k, v in sample.items()}}
    t0 = time.time()
    for i in range(48):
        if time.time() - t0 > budget_s:
            break
        p = sge.PatternGraph.random(7, 16 + i % 4, 3000 + i)
        n0 = len(rec.count)
        sge_learn.record(eng, st, [p], shortlist=12, pattern_offset=pid0 + i, time_budget_s=1.0, rec=rec,
                         candidates_fn=cands, sample=sample)
        done = [c for c, ms in zip(rec.count[n0:], rec.ms[n0:]) if ms < 2000.0]
        assert len(set(done)) <= 1, f"candidate plans disagree: {done}"
        meta["patterns"].append({"id": pid0 + i, "graph": "rmat_s22", "kind": "7v", "k": p.k,
                                 "edges": p.edges.tolist(), "train": i % 4 != 3})
        print(f"rmat_s22 pattern {i} recorded ({time.time() - t0:.0f}s)", flush=True)
    eng.close()
    rec.save(out / "plan_runtimes_rmat22.npz")
    (out / "plan_runtimes_rmat22.json").write_text(json.dumps(meta))
    tr_old, te_old = split(old, old_meta)
    tr_new, te_new = split(rec, meta)
    mlp = sge_learn.train(merge(tr_old, tr_new), epochs=400, seed=0)
    sge_learn.save_mlp(mlp, out / "mlp_weights.npz")
    print("held-out regret, small R-MAT", sge_learn.regret(te_old, mlp), flush=True)
    print("held-out regret, R-MAT 2^22 sample", sge_learn.regret(te_new, mlp), flush=True)


if __name__ == "__main__":
    if sys.argv[1] == "--rmat22":
        main_rmat22(Path(sys.argv[2]), float(sys.argv[3]) if len(sys.argv) > 3 else 600.0)
    else:
        main(Path(sys.argv[1]), float(sys.argv[2]) if len(sys.argv) > 2 else 300.0)
