"""Failure paths on the GPU without a GPU fault: a per-level buffer that would
overflow and a launch that runs out of its time budget both end the kernel
early with a status the host reads; the context stays usable afterwards."""
import pytest

from conftest import pattern_of

pytestmark = pytest.mark.gpu


def test_overflow_is_reported_not_silent(sge, patterns, graphs):
    g = graphs("chunglu_n7100")
    with sge.Engine(g) as eng:
        b = sge.plan(pattern_of(sge, patterns, "6vertex/4"), eng, iep=False)
        with pytest.raises(sge.SgeError) as e:
            eng.count([b], max_level_capacity=32)
        assert e.value.status_name == "STACK_OVERFLOW"
        c1, _, _ = eng.count([sge.plan(pattern_of(sge, patterns, "light_query/p2"), eng)])
        assert c1[0] > 0


def test_time_budget_is_reported(sge, patterns, graphs):
    g = graphs("chunglu_n7100")
    with sge.Engine(g) as eng:
        b = sge.plan(pattern_of(sge, patterns, "light_query/p4"), eng, iep=False)
        with pytest.raises(sge.SgeError) as e:
            eng.count([b], time_budget_s=1e-9)
        assert e.value.status_name == "TIMEOUT"
        full, _, _ = eng.count([b])
        assert full[0] == 14984077424
