"""The batch autotuner (sge_tune): its choices change how the work is split
and probed, never the counts.  Tuned and untuned batches (CUDA-graph replays)
must return identical counts, equal to the reference's on the Chung-Lu
n=7,100 graph and to the oracle's on an R-MAT root sample."""
import sys
from pathlib import Path

import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu
sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def test_tuned_batch_equals_untuned_and_reference(sge, patterns, golden, graphs):
    import sge_tune
    g = graphs("chunglu_n7100")
    rows = golden_rows(golden, "chunglu_n7100")
    with sge.Engine(g) as eng:
        plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng) for r in rows]
        t = sge_tune.tune(eng, plans, {})
        assert len(t.plans) == len(plans) and t.runs == 3 + len(sge_tune.CANDIDATES)
        with eng.batch(plans) as b0, eng.batch(plans, pin_tables=t.pin_tables, tuning=t.plans) as b1:
            c0, _, _ = b0.run()
            c1, _, _ = b1.run()
    assert c0 == c1 == [r["count"] for r in rows]


def test_tuned_rmat_sample_equals_oracle(sge, oracle):
    import bench
    import sge_tune
    with sge.Engine.rmat_device(18, 4_000_000, seed=4) as eng:
        st = eng.graph.stats()
        pats = bench.rmat22_patterns(sge)[:12]
        plans = [bench.plain_plan(sge, p, st) for p in pats]
        sample = dict(root_stride=1 << 12, root_offset=1, root_max_degree=1000)
        t = sge_tune.tune(eng, plans, sample)
        c0, _, _ = eng.count(plans, **sample)
        with eng.batch(plans, pin_tables=t.pin_tables, tuning=t.plans, **sample) as b:
            c1, _, _ = b.run()
        assert c0 == c1
        og = oracle.Graph(eng.graph.offsets, eng.graph.nbrs)
        inst, _ = og.count_plans(b"".join(p.to_bytes() for p in plans), len(plans), stride=1 << 12, offset=1,
                                 root_max_degree=1000)
        og.close()
        assert c1 == [i * p.count_multiplier for i, p in zip(inst, plans)]
