"""Reference counts on down-scaled R-MAT graphs of the batch configurations'
generator (a=.57 b=.19 c=.19, edge factor 16, seed 4), for the patterns the
reference finishes there within two minutes.

Run with SGE_REFERENCE naming a reference checkout, after
``__graft_entry__.build()`` (same variable) has compiled
oracle/_ref/graph_mining_system from its sources.  Writes
tests/golden/golden_rmat.json: per (graph, pattern) the reference's
"Number of matches", its "num bags", the decomposition it printed
(the text sge_plan_from_order_text and sge_bags_create read) and run time.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "subgraph-enumeration_gb300"))
import sge  # noqa: E402

REF_BIN = REPO / "oracle" / "_ref" / "graph_mining_system"
GRAPHS = {"rmat_s14": dict(scale=14, m=1 << 18, seed=4), "rmat_s16": dict(scale=16, m=1 << 20, seed=4)}
PATTERNS = {
    "rmat_s14": ["light_query/p1", "light_query/p2", "light_query/p3", "light_query/p4", "light_query/p6",
                 "triangle", "k5_minus_e"],
    "rmat_s16": ["light_query/p1", "light_query/p2", "light_query/p6", "triangle", "k5_minus_e"],
}


def main() -> None:
    if not os.environ.get("SGE_REFERENCE"):
        sys.exit("set SGE_REFERENCE to the reference checkout")
    if not REF_BIN.exists():
        sys.exit(f"{REF_BIN} missing: build it first (oracle/ref.mk)")
    pats = json.loads((HERE / "patterns.json").read_text())
    tmp = Path(tempfile.mkdtemp())
    out = {"graphs": {}, "results": []}
    for gname, spec in GRAPHS.items():
        g = sge.gen_rmat(spec["scale"], spec["m"], 0.57, 0.19, 0.19, spec["seed"])
        gf = tmp / f"{gname}.bin"
        g.save_binary(gf)
        out["graphs"][gname] = dict(spec, a=0.57, b=0.19, c=0.19, kind="rmat", fingerprint=g.fingerprint(),
                                    n=g.num_vertices, max_degree=g.max_degree)
        for pn in PATTERNS[gname]:
            p = sge.PatternGraph.from_edges(pats[pn]["k"], pats[pn]["edges"])
            qf = tmp / "q.txt"
            qf.write_text(p.text())
            single = p.info()[1]
            t = time.time()
            r = subprocess.run([str(REF_BIN), "-q", str(qf), "-d", str(gf), "-t", "1" if single else "8"],
                               capture_output=True, text=True, timeout=600)
            m = re.search(r"Number of matches: (\d+)", r.stdout)
            b = re.search(r"num bags: (\d+)", r.stdout)
            plan = None
            if b:  # the printed decomposition: "num bags: N" and one order per bag
                lines = r.stdout[b.start():].splitlines()
                plan = "\n".join(lines[: 1 + int(b.group(1))]) + "\n"
            row = {"graph": gname, "pattern": pn, "count": int(m.group(1)) if m else None,
                   "num_bags": int(b.group(1)) if b else None, "plan": plan, "rc": r.returncode,
                   "seconds": round(time.time() - t, 1)}
            out["results"].append(row)
            print(row, flush=True)
    (HERE / "golden_rmat.json").write_text(json.dumps(out, indent=0))


if __name__ == "__main__":
    main()
