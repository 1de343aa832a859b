"""Records the reference planner's own plans for the plan-import tests.

Run with SGE_REFERENCE naming a reference checkout, after
``__graft_entry__.build()`` (with the same variable set) has compiled
oracle/_ref/graph_mining_system from its sources.  For every shipped query
pattern (light_query, huge_query, 6vertex, 7vertex) on the shipped
ca-netscience graph, in the default and the -u mode, it keeps the block
HyperTree::writeToStream prints after planning ("num bags: N" + one bag order
per line, global bag last; plan/decomposition.cpp:537-552, main.cpp:66) and
the run's "Number of matches".  The reference seeds its sampler from
std::random_device (utility/utils.h:24-25), so the recorded plans are one
draw; the counts do not depend on it.

Output: tests/golden/reference_plans.json
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF_BIN = REPO / "oracle" / "_ref" / "graph_mining_system"


def plan_block(out: str) -> str:
    lines = out.splitlines()
    for i, ln in enumerate(lines):
        m = re.match(r"num bags: (\d+)", ln)
        if m:
            return "\n".join(lines[i:i + 1 + int(m.group(1))]) + "\n"
    return ""


def main() -> None:
    if not os.environ.get("SGE_REFERENCE"):
        sys.exit("set SGE_REFERENCE to the reference checkout")
    ref = Path(os.environ["SGE_REFERENCE"])
    if not REF_BIN.exists():
        sys.exit(f"{REF_BIN} missing: build it first (oracle/ref.mk)")
    data = ref / "dataset" / "ca-netscience.txt"
    jobs = []
    for sub in ("light_query", "huge_query", "6vertex", "7vertex"):
        for f in sorted((ref / "dataset" / sub).glob("*.txt"), key=lambda p: int(re.sub(r"\D", "", p.stem))):
            for mode in ("default", "u"):
                jobs.append((f"{sub}/{f.stem}", str(f), mode))

    def run(job):
        name, q, mode = job
        flags = ["-u"] if mode == "u" else []
        r = subprocess.run([str(REF_BIN), "-q", q, "-d", str(data), "-t", "1", *flags], capture_output=True,
                           text=True, timeout=600)
        m = re.search(r"Number of matches: (\d+)", r.stdout)
        return {"pattern": name, "mode": mode, "plan": plan_block(r.stdout),
                "count": int(m.group(1)) if m else None, "rc": r.returncode}

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        rows = list(ex.map(run, jobs))
    (HERE / "reference_plans.json").write_text(json.dumps(
        {"graph": "ca_netscience", "rows": rows,
         "note": "plans printed by the reference's graph_mining_system (-t 1) after optCostPlan; "
                 "built from its sources by oracle/ref.mk"}, indent=0))
    print(f"{len(rows)} plans, {sum(r['rc'] == 0 for r in rows)} ran cleanly")


if __name__ == "__main__":
    main()
