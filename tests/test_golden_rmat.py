"""Reference counts on down-scaled R-MAT graphs of the batch configurations'
generator (2^14 / 262K and 2^16 / 1M edges, edge factor 16), recorded from the
reference compiled from its sources (tests/golden/make_golden_rmat.py): the
CPU oracle on the quick rows, the GPU on every row in all four modes."""
import json

import pytest

from conftest import GOLDEN, pattern_of


@pytest.fixture(scope="module")
def gold():
    return json.loads((GOLDEN / "golden_rmat.json").read_text())


def graph_of(sge, gold, name):
    spec = gold["graphs"][name]
    g = sge.gen_rmat(spec["scale"], spec["m"], spec["a"], spec["b"], spec["c"], spec["seed"])
    assert g.fingerprint() == spec["fingerprint"]
    return g


def test_oracle_matches_reference_on_rmat_s14(sge, oracle, patterns, gold):
    g = graph_of(sge, gold, "rmat_s14")
    rows = [r for r in gold["results"] if r["graph"] == "rmat_s14" and r["rc"] == 0
            and r["pattern"] in ("light_query/p2", "triangle", "k5_minus_e")]
    assert len(rows) == 3
    for r in rows:
        b = sge.plan(pattern_of(sge, patterns, r["pattern"]), g)
        inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=0)
        assert inst * b.count_multiplier == r["count"], r["pattern"]


@pytest.mark.gpu
@pytest.mark.parametrize("graph", ["rmat_s14", "rmat_s16"])
def test_gpu_matches_reference_on_downscaled_rmat(sge, patterns, gold, graph):
    g = graph_of(sge, gold, graph)
    rows = [r for r in gold["results"] if r["graph"] == graph and r["rc"] == 0 and r["count"] is not None]
    assert len(rows) >= 5
    with sge.Engine(g) as eng:
        for iep in (False, True):
            for expl in (False, True):
                plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=iep, exploration=expl)
                         for r in rows]
                counts, _, _ = eng.count(plans)
                bad = [(r["pattern"], c, r["count"]) for r, c in zip(rows, counts) if c != r["count"]]
                assert not bad, (iep, expl, bad)


def test_imported_decompositions_on_the_oracle(sge, oracle, patterns, gold):
    """The decompositions the reference printed on R-MAT 2^14 (its quick
    multi-bag rows), imported as the reference's plan and run by the CPU
    oracle, give the reference's counts."""
    g = graph_of(sge, gold, "rmat_s14")
    rows = [r for r in gold["results"] if r["graph"] == "rmat_s14" and r["rc"] == 0 and r.get("plan")
            and r["num_bags"] > 1 and r["seconds"] < 6]
    assert len(rows) >= 3
    for r in rows:
        p = pattern_of(sge, patterns, r["pattern"])
        b, nb = sge.plan_from_reference(p, r["plan"], g, iep=True)
        assert nb == r["num_bags"]
        inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=0)
        assert inst * b.count_multiplier == r["count"], r["pattern"]
