"""bench.py: the CPU reference arm's JSON line (and that it loads only the
oracle library), the plan fixture it runs, and the sampling rule that makes
the learned and plain planners count the same instances."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))


def test_reference_arm_json_line_and_native_code():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--workload", "chunglu7100",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    assert d["unit"] == "embeddings/s" and d["config"]["plans_per_step"] == 12
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["native_loaded"] == ["oracle/_build/liboracle.so"], d["native_loaded"]


def test_plan_fixture_matches_the_planner(sge):
    import bench
    d = np.load(bench.PLAN_FIXTURE)
    st = sge.GraphStats.from_buffer_copy(bytes(d["chunglu7100_stats"]))
    plans = []
    for pname, (k, edges) in bench.CL_PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        for _, expl, iep in bench.CL_MODES:
            plans.append(sge.plan(p, st, iep=iep, exploration=expl).to_bytes())
    assert [bytes(b) for b in d["chunglu7100_plans"]] == plans
    st = sge.GraphStats.from_buffer_copy(bytes(d["rmat22_stats"]))
    fix = [bytes(b) for b in d["rmat22_plain"]]
    pats = bench.rmat22_patterns(sge)
    assert len(fix) == len(pats) == 78
    assert all(bench.plain_plan(sge, p, st).to_bytes() == f for p, f in zip(pats, fix))
    assert [bench.blob_multiplier(b) for b in d["rmat22_plain"]] == [1] * 78


def test_blob_multiplier_reads_the_struct(sge):
    import bench
    p = sge.PatternGraph.from_edges(4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)])  # K4: one bag
    b = sge.plan(p, None)
    assert b.count_multiplier == 24
    assert bench.blob_multiplier(np.frombuffer(b.to_bytes(), np.uint8)) == 24


def test_canonical_symmetry_makes_planners_agree_on_a_sample(sge, oracle):
    import bench
    g = sge.gen_chung_lu(380, 915, 2.3, 0, 1)
    st = g.stats()
    for p in bench.rmat22_patterns(sge)[:6]:
        seq, root = bench.canonical_symmetry(p.k, p.edges)
        plain = bench.plain_plan(sge, p, st)
        cands = sge.candidates(p, st, cap=64, symmetry_seq=seq, root_edge=root)
        assert sorted(plain.order[:2]) == sorted(root)
        want = oracle.count_plan(g.offsets, g.nbrs, plain, threads=4, stride=5, offset=2)[0]
        for b in cands[:8]:
            assert sorted(b.order[:2]) == sorted(root)
            assert oracle.count_plan(g.offsets, g.nbrs, b, threads=4, stride=5, offset=2)[0] == want


def test_sample_shards_partition_the_sample():
    import bench
    base = bench.sample_opts()
    m = 10_000_000
    whole = set(range(base["root_offset"], m, base["root_stride"]))
    for world in (2, 4):
        parts = [set(range(o["root_offset"], m, o["root_stride"]))
                 for o in (bench.sample_opts(world, r) for r in range(world))]
        assert set().union(*parts) == whole and sum(map(len, parts)) == len(whole)
    sub = bench.sample_opts(1, 0, bench.CPU_SUBSAMPLE)
    assert set(range(sub["root_offset"], m, sub["root_stride"])) <= whole
