"""Generates the golden fixtures under tests/golden/ from the reference.

Run with SGE_REFERENCE naming a reference checkout, after
``__graft_entry__.build()`` (with the same variable set) has compiled
oracle/_ref/graph_mining_system from its sources.  The reference itself never runs in the tests: only its recorded
outputs do.

Outputs (all small):
  ca_netscience.el      – the reference's ca-netscience data graph as "u v" lines
  patterns.json         – every shipped query pattern (light_query, huge_query,
                          6vertex, 7vertex) + seeded random batches
  golden_counts.json    – reference "Number of matches" (and "num bags") per
                          (graph, pattern, mode), with the synthetic graphs'
                          generator parameters and fingerprints
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "subgraph-enumeration_gb300"))
import sge  # noqa: E402

if not os.environ.get("SGE_REFERENCE"):
    sys.exit("set SGE_REFERENCE to the reference checkout")
REF = Path(os.environ["SGE_REFERENCE"])
REF_BIN = REPO / "oracle" / "_ref" / "graph_mining_system"

# Synthetic data graphs with the shapes of the reference's fixtures.
SYNTH = {
    # configuration 1: stands in for ca-netscience (n=379, m=914, maxdeg 34)
    "chunglu_n380": dict(kind="chung_lu", n=380, m=915, gamma=2.3, max_deg=0, seed=1),
    # configuration 2: stands in for wiki-vote (n=7115, m=100762, maxdeg 1065)
    "chunglu_n7100": dict(kind="chung_lu", n=7100, m=100000, gamma=2.1, max_deg=1000, seed=2),
    # a down-scaled R-MAT with the batch configurations' generator parameters
    "rmat_s12": dict(kind="rmat", scale=12, m=40000, a=0.57, b=0.19, c=0.19, seed=3),
}


def make_graph(spec: dict) -> sge.DataGraph:
    if spec["kind"] == "chung_lu":
        return sge.gen_chung_lu(spec["n"], spec["m"], spec["gamma"], spec["max_deg"], spec["seed"])
    return sge.gen_rmat(spec["scale"], spec["m"], spec["a"], spec["b"], spec["c"], spec["seed"])


def run_ref(q: str, d: str, flags: list[str]) -> dict:
    r = subprocess.run([str(REF_BIN), "-q", q, "-d", d, *flags], capture_output=True, text=True, timeout=3600)
    out = r.stdout
    m = re.search(r"Number of matches: (\d+)", out)
    b = re.search(r"num bags: (\d+)", out)
    return {"count": int(m.group(1)) if m else None, "num_bags": int(b.group(1)) if b else None,
            "rc": r.returncode}


def main() -> None:
    if not REF_BIN.exists():
        sys.exit(f"{REF_BIN} missing: build it first (oracle/ref.mk)")
    patterns: dict[str, dict] = {}
    for sub in ("light_query", "huge_query", "6vertex", "7vertex"):
        for f in sorted((REF / "dataset" / sub).glob("*.txt"), key=lambda p: int(re.sub(r"\D", "", p.stem))):
            p = sge.PatternGraph.load(f)
            patterns[f"{sub}/{f.stem}"] = {"k": p.k, "edges": p.edges.tolist()}
    # extra shapes named by the benchmark configurations
    patterns["k5_minus_e"] = {"k": 5, "edges": [[a, b] for a in range(5) for b in range(a + 1, 5) if (a, b) != (3, 4)]}
    patterns["triangle"] = {"k": 3, "edges": [[0, 1], [0, 2], [1, 2]]}
    patterns["k4_pendant"] = {"k": 5, "edges": [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3], [3, 4]]}
    patterns["c6_two_chords"] = {"k": 6, "edges": [[0, 1], [1, 2], [2, 3], [3, 4], [4, 5], [0, 5], [0, 3], [1, 4]]}
    patterns["two_triangles_4cycle"] = {"k": 6, "edges": [[0, 1], [0, 2], [1, 2], [3, 4], [3, 5], [4, 5],
                                                          [1, 3], [2, 4]]}
    batch6, batch7, rnd = [], [], []
    for i in range(16):
        p = sge.PatternGraph.random(6, 11 + i % 3, 1000 + i)
        patterns[f"batch6/{i}"] = {"k": 6, "edges": p.edges.tolist()}
        batch6.append(f"batch6/{i}")
    for i in range(78):
        p = sge.PatternGraph.random(7, 16 + i % 4, 2000 + i)
        patterns[f"batch7/{i}"] = {"k": 7, "edges": p.edges.tolist()}
        batch7.append(f"batch7/{i}")
    for i in range(120):
        k = 4 + i % 4
        mmax = k * (k - 1) // 2
        m = k - 1 + (i * 7) % (mmax - k + 2)
        p = sge.PatternGraph.random(k, m, 5000 + i)
        patterns[f"random/{i}"] = {"k": k, "edges": p.edges.tolist()}
        rnd.append(f"random/{i}")
    (HERE / "patterns.json").write_text(json.dumps(patterns, separators=(",", ":")))

    tmp = Path(tempfile.mkdtemp())
    qpath = {}
    for name, p in patterns.items():
        f = tmp / (name.replace("/", "_") + ".txt")
        f.write_text(sge.PatternGraph.from_edges(p["k"], p["edges"]).text())
        qpath[name] = str(f)

    ca = sge.DataGraph.load(REF / "dataset" / "ca-netscience.txt")
    with open(HERE / "ca_netscience.el", "w") as f:
        f.write(f"{ca.num_vertices} {ca.num_edges}\n")
        for a, b in ca.edge_array():
            f.write(f"{a} {b}\n")
    graphs = {"ca_netscience": {"kind": "file", "path": "ca_netscience.el", "fingerprint": ca.fingerprint(),
                                "n": ca.num_vertices, "m": ca.num_edges}}
    gfiles = {"ca_netscience": str(HERE / "ca_netscience.el")}
    for name, spec in SYNTH.items():
        g = make_graph(spec)
        gf = tmp / f"{name}.txt"
        g.save_text(gf)
        gfiles[name] = str(gf)
        graphs[name] = dict(spec, fingerprint=g.fingerprint(), n=g.num_vertices, m=g.num_edges,
                            max_degree=g.max_degree)

    jobs = []  # (graph, pattern, mode)
    everything = [n for n in patterns]
    for pn in everything:
        jobs.append(("ca_netscience", pn, "default"))
    for pn in ["light_query/p1", "light_query/p2", "light_query/p4", "light_query/p6", "k5_minus_e", "triangle",
               "k4_pendant", "light_query/p3", "light_query/p7", "c6_two_chords", "two_triangles_4cycle"] + rnd[:60]:
        jobs.append(("chunglu_n380", pn, "default"))
    for pn in ["light_query/p2", "light_query/p4", "light_query/p6", "k5_minus_e", "light_query/p1"]:
        for mode in ("default", "u", "i", "iu"):
            jobs.append(("chunglu_n7100", pn, mode))
    for pn in ["light_query/p3", "light_query/p7", "triangle"]:
        jobs.append(("chunglu_n7100", pn, "default"))
    for pn in batch6 + ["c6_two_chords", "two_triangles_4cycle", "light_query/p7", "light_query/p4"]:
        jobs.append(("rmat_s12", pn, "default"))

    def do(job):
        gname, pn, mode = job
        single = sge.PatternGraph.from_edges(patterns[pn]["k"], patterns[pn]["edges"]).info()[1]
        flags = {"default": [], "u": ["-u"], "i": ["-i"], "iu": ["-i", "-u"]}[mode]
        # single-bag plans crash the reference's OpenMP path; run them serially
        flags = flags + (["-t", "1"] if single or gname == "ca_netscience" else ["-t", "4"])
        return job, run_ref(qpath[pn], gfiles[gname], flags)

    results = []
    with ThreadPoolExecutor(max_workers=2) as ex:
        for (gname, pn, mode), r in ex.map(do, jobs):
            results.append({"graph": gname, "pattern": pn, "mode": mode, **r})
            print(gname, pn, mode, r, flush=True)
    (HERE / "golden_counts.json").write_text(json.dumps(
        {"graphs": graphs, "results": results,
         "note": "reference graph_mining_system built from its sources by oracle/ref.mk; counts are its "
                 "'Number of matches'; mode i/iu counts are recorded but known to be wrong in the reference"},
        indent=0))


if __name__ == "__main__":
    main()
