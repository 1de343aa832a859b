"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's recorded counts and against the CPU oracle on the same seeded
inputs.  Integer results must be bit-exact."""
import numpy as np
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engines(sge, graphs):
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = sge.Engine(graphs(name))
        return cache[name]
    yield get
    for e in cache.values():
        e.close()


@pytest.mark.parametrize("iep", [False, True])
@pytest.mark.parametrize("exploration", [False, True])
def test_ca_netscience_all_shipped_patterns(sge, patterns, golden, engines, iep, exploration):
    eng = engines("ca_netscience")
    rows = golden_rows(golden, "ca_netscience")
    assert len(rows) > 300
    plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=iep, exploration=exploration) for r in rows]
    counts, inst, _ = eng.count(plans)          # one batched persistent launch
    bad = [(r["pattern"], c, r["count"]) for r, c in zip(rows, counts) if c != r["count"]]
    assert not bad, bad[:10]


@pytest.mark.parametrize("graph", ["chunglu_n380", "chunglu_n7100", "rmat_s12"])
def test_synthetic_graphs_match_reference(sge, patterns, golden, engines, graph):
    eng = engines(graph)
    rows = golden_rows(golden, graph) + golden_rows(golden, graph, "u")
    assert rows
    for exploration in (False, True):
        plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=True, exploration=exploration)
                 for r in rows]
        counts, _, _ = eng.count(plans)
        bad = [(r["pattern"], r["mode"], c, r["count"]) for r, c in zip(rows, counts) if c != r["count"]]
        assert not bad, bad[:10]


def test_exploration_mode_matches_default_count_not_reference_i(sge, patterns, golden, engines):
    """-i in the reference miscounts some patterns; the GPU -i path must give
    the default-mode count."""
    eng = engines("chunglu_n7100")
    want = {r["pattern"]: r["count"] for r in golden_rows(golden, "chunglu_n7100")}
    for r in golden_rows(golden, "chunglu_n7100", "i") + golden_rows(golden, "chunglu_n7100", "iu"):
        b = sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep="u" in r["mode"], exploration=True)
        (c,), _, _ = eng.count([b])
        assert c == want[r["pattern"]]


def test_random_orders_match_oracle(sge, oracle, patterns, engines, graphs):
    g = graphs("chunglu_n380")
    eng = engines("chunglu_n380")
    rng = np.random.default_rng(5)
    names = [n for n in patterns if n.startswith("random/")][:40]
    plans, want = [], []
    for n in names:
        p = pattern_of(sge, patterns, n)
        for _ in range(20):
            try:
                b = sge.plan(p, eng, iep=bool(rng.integers(2)), exploration=bool(rng.integers(2)),
                             force_order=rng.permutation(p.k).tolist())
                break
            except sge.SgeError:
                continue
        else:
            b = sge.plan(p, eng)
        inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=8)
        plans.append(b)
        want.append(inst * b.count_multiplier)
    counts, _, _ = eng.count(plans)
    assert counts == want


def test_sampled_roots_match_oracle_at_scale(sge, oracle, patterns):
    """A larger R-MAT where the oracle only runs a 1/97 sample of the roots:
    the GPU restricted to the same roots must agree exactly, and the sum over
    all residues must equal the full count."""
    g = sge.gen_rmat(16, 600_000, seed=11)
    with sge.Engine(g) as eng:
        plans = [sge.plan(pattern_of(sge, patterns, n), eng) for n in
                 ["light_query/p2", "light_query/p4", "k5_minus_e", "light_query/p7", "6vertex/2"]]
        s = 97
        gpu, _, _ = eng.count(plans, root_stride=s, root_offset=5)
        for b, c in zip(plans, gpu):
            inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=8, stride=s, offset=5)
            assert c == inst * b.count_multiplier
        full, _, _ = eng.count(plans[:2])
        parts = [eng.count(plans[:2], root_stride=4, root_offset=o)[0] for o in range(4)]
        assert [sum(p[i] for p in parts) % 2**64 for i in range(2)] == full


def test_edge_cases(sge, oracle, patterns):
    tri = pattern_of(sge, patterns, "triangle")
    star = sge.PatternGraph.from_edges(4, [(0, 1), (0, 2), (0, 3)])
    k5 = pattern_of(sge, patterns, "light_query/p7")
    # graph without edges
    empty = sge.DataGraph(np.zeros(6, np.uint32), np.zeros(0, np.uint32))
    with sge.Engine(empty) as eng:
        assert eng.count([sge.plan(tri, eng)])[0] == [0]
    # complete graph K_12: K5 embeddings = 12·11·10·9·8, triangles = 6·C(12,3)
    n = 12
    kn = sge.DataGraph.from_edges(np.array([(a, b) for a in range(n) for b in range(a + 1, n)]), n)
    with sge.Engine(kn) as eng:
        c, inst, _ = eng.count([sge.plan(k5, eng), sge.plan(tri, eng)])
        assert c == [12 * 11 * 10 * 9 * 8, 6 * 220]
        assert inst == [792, 6 * 220 // 6]
    # a hub with 50k leaves plus a ring: stars through the hub (choose-3 tail)
    leaves = 50_000
    e = [(0, i) for i in range(1, leaves + 1)] + [(i, i + 1) for i in range(1, leaves)]
    hub = sge.DataGraph.from_edges(np.array(e), leaves + 1)
    with sge.Engine(hub) as eng:
        b = sge.plan(star, eng)
        inst, _ = oracle.count_plan(hub.offsets, hub.nbrs, b, threads=8)
        assert eng.count([b])[0] == [inst * b.count_multiplier]
        from math import comb
        assert inst >= comb(leaves, 3)


def test_count_host_end_to_end(sge, patterns, golden, graphs):
    g = graphs("ca_netscience")
    rows = golden_rows(golden, "ca_netscience")[:50]
    st = g.stats()
    plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), st) for r in rows]
    counts, stats = sge.count_host(g, plans, stats=True)
    assert counts == [r["count"] for r in rows]
    # one launch, plus two when some root is split (deep plans on few roots):
    # the kernel numbering the split tasks and the launch running them
    assert stats["gpu_launches"] in (1, 3) and stats["root_tasks"] > 0


def test_match_api_like_reference_main(sge, tmp_path, patterns):
    q = tmp_path / "house.txt"
    q.write_text(pattern_of(sge, patterns, "light_query/p4").text())
    from conftest import GOLDEN
    r = sge.match(q, GOLDEN / "ca_netscience.el", iep=True)
    assert r["Number of matches"] == 36742
