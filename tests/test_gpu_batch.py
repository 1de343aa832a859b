"""Batches replayed from a captured CUDA graph give the same counts as
sge_count, run after run."""
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


def test_batch_replay_matches_reference(sge, patterns, golden, graphs):
    g = graphs("ca_netscience")
    rows = golden_rows(golden, "ca_netscience")[:120]
    with sge.Engine(g) as eng:
        plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=i % 2 == 0, exploration=i % 3 == 0)
                 for i, r in enumerate(rows)]
        with eng.batch(plans) as b:
            for _ in range(3):
                c, inst, st = b.run()
                assert c == [r["count"] for r in rows]
                assert st["gpu_launches"] >= 1 and st["kernel_ms"] > 0


@pytest.mark.parametrize("heavy", [512, 0])
def test_batch_with_counters_and_splitting(sge, patterns, golden, graphs, heavy):
    # max degree ~800: with a threshold of 512 the heavy roots take a second
    # counting launch (after the kernel that numbers their tasks); the
    # automatic threshold splits none at this size
    g = graphs("chunglu_n7100")
    names = ["light_query/p2", "light_query/p4", "k5_minus_e", "light_query/p6"]
    want = {r["pattern"]: r["count"] for r in golden_rows(golden, "chunglu_n7100")}
    with sge.Engine(g) as eng:
        plans = [sge.plan(pattern_of(sge, patterns, n), eng) for n in names]
        with eng.batch(plans, stats=True, heavy_threshold=heavy) as b:
            for _ in range(2):
                c, _, st = b.run()
                assert c == [want[n] for n in names]
                assert st["gpu_launches"] == (3 if heavy else 1) and st["set_ops"] > 0 and st["alg_bytes"] > 0
