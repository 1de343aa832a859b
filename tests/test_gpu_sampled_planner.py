"""GPU root sampling as the planner's cost (sge_plan_pattern_sampled): the
chosen plan is the shortlist's fastest sample and counts like any plan."""
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


def test_sampled_planner_picks_the_fastest_sample(sge, patterns, golden, graphs):
    g = graphs("chunglu_n7100")
    want = {r["pattern"]: r["count"] for r in golden_rows(golden, "chunglu_n7100")}
    names = [n for n in ["k5_minus_e", "light_query/p4", "light_query/p6"] if n in want]
    assert names
    with sge.Engine(g) as eng:
        for name in names:
            b, ms = sge.plan_sampled(pattern_of(sge, patterns, name), eng, shortlist=6, sample_stride=32)
            timed = [t for t in ms if t >= 0]
            assert timed and len(ms) == 6
            counts, _, _ = eng.count([b])
            assert counts[0] == want[name]
