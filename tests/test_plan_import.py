"""The reference planner's own plans, imported through
sge_plan_from_order_text (the hand-off text HyperTree::writeToStream prints,
plan/decomposition.cpp:537-552), run to the reference's "Number of matches".
The plans and counts were recorded from the reference compiled from its
sources (tests/golden/make_reference_plans.py)."""
import json

import pytest

from conftest import GOLDEN, pattern_of


@pytest.fixture(scope="module")
def ref_plans():
    return json.loads((GOLDEN / "reference_plans.json").read_text())["rows"]


@pytest.fixture(scope="module")
def ca(sge):
    return sge.DataGraph.load(GOLDEN / "ca_netscience.el")


def imported(sge, patterns, ca, rows):
    out = []
    for r in rows:
        p = pattern_of(sge, patterns, r["pattern"])
        b, nb = sge.plan_from_reference(p, r["plan"], ca, iep=r["mode"] == "u")
        assert nb == int(r["plan"].split("\n")[0].split(":")[1])
        out.append(b)
    return out


# Recorded runs where the reference's -u (inclusion-exclusion) leaf printed a
# wrong count for the plan its sampler happened to pick: light_query/p5 gives
# 137419 under the plan with global bag (0,2,3,4) and 107993 (the brute-force
# count, the default mode's) under others.  The imported plan counts 107993.
REFERENCE_IEP_MISCOUNTS = {("light_query/p5", "u"): 137419}


def expected(r, golden_default):
    want = golden_default[r["pattern"]]
    if (r["pattern"], r["mode"]) in REFERENCE_IEP_MISCOUNTS:
        assert r["count"] == REFERENCE_IEP_MISCOUNTS[(r["pattern"], r["mode"])]
    else:
        assert r["count"] == want, (r["pattern"], r["mode"])
    return want


@pytest.fixture(scope="module")
def golden_default(golden):
    return {r["pattern"]: r["count"] for r in golden["results"]
            if r["graph"] == "ca_netscience" and r["mode"] == "default" and r["rc"] == 0}


def test_every_recorded_plan_imports_and_counts_on_the_oracle(sge, oracle, patterns, ca, ref_plans, golden_default):
    rows = [r for r in ref_plans if r["rc"] == 0 and r["count"] is not None]
    assert len(rows) == 214
    plans = imported(sge, patterns, ca, rows)
    bad = []
    for r, b in zip(rows, plans):
        assert b.choose_wrap == 1
        inst, _ = oracle.count_plan(ca.offsets, ca.nbrs, b, threads=4)
        if inst * b.count_multiplier != expected(r, golden_default):
            bad.append((r["pattern"], r["mode"], inst * b.count_multiplier, r["count"]))
    assert not bad, bad[:5]


def test_one_bag_plans_count_embeddings(sge, patterns, ca, ref_plans):
    one = [r for r in ref_plans if r["plan"].startswith("num bags: 1\n")]
    assert one
    for b, r in zip(imported(sge, patterns, ca, one), one):
        assert b.single_bag == 1 and b.count_multiplier == b.aut_size > 1, r["pattern"]


def test_import_follows_the_global_bag_order(sge, patterns, ca):
    # 6vertex/0 with bags (4,5,3,0) (4,5,2) (4,5,3,1): the global bag runs first
    p = pattern_of(sge, patterns, "6vertex/0")
    b, nb = sge.plan_from_reference(p, "num bags: 3\n4,5,3,0\n4,5,2\n4,5,3,1\n", ca, iep=False)
    assert nb == 3 and list(b.order[:4]) == [4, 5, 3, 1]
    assert sorted(b.order[:6]) == list(range(6))


@pytest.mark.parametrize("text", [
    "",                                   # no bag
    "num bags: 2\n0,1,2\n",               # fewer orders than announced
    "num bags: 1\n0,1,2,9\n",             # vertex out of range
    "num bags: 2\n0,1\n2,3\n",            # edges (1,2), (0,3) ... in no bag, vertices of a 4-cycle split
    "num bags: 1\n0,1,1,2,3\n",           # repeated vertex
])
def test_malformed_plan_text_is_rejected(sge, text):
    p = sge.PatternGraph.from_edges(4, [(0, 1), (1, 2), (2, 3), (0, 3)])
    with pytest.raises(sge.SgeError) as e:
        sge.plan_from_reference(p, text)
    assert e.value.status_name == "BAD_INPUT"


@pytest.mark.gpu
def test_every_recorded_plan_runs_on_the_gpu(sge, patterns, ca, ref_plans, golden_default):
    rows = [r for r in ref_plans if r["rc"] == 0 and r["count"] is not None]
    plans = imported(sge, patterns, ca, rows)
    with sge.Engine(ca) as eng:
        counts, _, _ = eng.count(plans)       # one batched launch of all 214 imported plans
    bad = [(r["pattern"], r["mode"], c, r["count"]) for r, c in zip(rows, counts) if c != expected(r, golden_default)]
    assert not bad, bad[:5]


def test_import_counts_other_bags_own_attributes_at_the_leaf(sge):
    """As sharedJoin, the attributes outside the global bag are counted at the
    leaf: with -u the imported plan's tail is all of them (here 0 and 5, the
    own vertices of the triangle bags), without -u a single level."""
    p = sge.PatternGraph.from_edges(6, [(0, 1), (0, 2), (1, 2), (3, 4), (3, 5), (4, 5), (1, 3), (2, 4)])
    text = "num bags: 5\n1,0,2\n3,1,2\n3,4,2\n3,4,5\n3,4,1,2\n"
    b, nb = sge.plan_from_reference(p, text, None, iep=True)
    assert nb == 5 and b.tail_len == 2 and sorted(b.order[4:6]) == [0, 5] and b.tail_mode == 3
    b1, _ = sge.plan_from_reference(p, text, None, iep=False)
    assert b1.tail_len == 1 and list(b1.order[:4]) == [3, 4, 1, 2]
