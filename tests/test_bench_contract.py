"""bench.py's CPU reference arm prints one JSON line with the keys the
benchmark contract names (run on a small root sample)."""
import json
import os
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    env = dict(os.environ, SGE_REF_STRIDE="256")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    assert d["unit"] == "embeddings/s" and d["config"]["plans_per_step"] == 12
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_profile_traffic_is_read_from_the_committed_summary():
    sys.path.insert(0, str(REPO))
    import bench
    t = bench.profile_traffic()
    assert t is None or t > 0


def test_cpu_baseline_runs_on_the_host():
    sys.path.insert(0, str(REPO))
    sys.path.insert(0, str(REPO / "subgraph-enumeration_gb300"))
    import bench
    import sge
    g = bench.build_workload(sge)
    plans, _ = bench.make_plans(sge, g.stats())
    cb = bench.cpu_baseline(sge, g, plans, budget_s=1.5)
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1
    assert "inclusion-exclusion" in cb["sample"]
