"""The instrumented kernel's algorithmic-byte counter (sge_stats.alg_bytes, the
numerator of the roofline's `achieved`) checked against its definition
evaluated on the CPU (oracle.alg_bytes_root_leaf) for every plan with two
enumerated levels of five small patterns (SINGLE with an ordered or unordered
root, CHOOSE with one and with two lists, inclusion-exclusion) on the graphs
of the two Chung-Lu configurations (n=380 and n=7,100), with and without the
hub bitmaps and on a capped root sample."""
import numpy as np
import pytest

PATTERNS = {
    "triangle": (3, [(0, 1), (0, 2), (1, 2)]),
    "wedge": (3, [(0, 1), (1, 2)]),
    "diamond": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3)]),
    "tailed_triangle": (4, [(0, 1), (0, 2), (1, 2), (0, 3)]),
    "star3": (4, [(0, 1), (0, 2), (0, 3)]),
}


def root_leaf_plans(sge, st):
    out = []
    for name, (k, e) in PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, e)
        out += [(name, b) for b in sge.candidates(p, st, cap=64) if b.num_enum == 2]
    return out


def test_definition_on_a_direct_count(sge, oracle, graphs):
    """A wedge plan counts its one tail list directly: the definition reduces
    to 4·(2 + |check|)·⌊log2(len'+1)⌋ per root, len' the list inside the bounds."""
    g = graphs("chunglu_n380")
    p = sge.PatternGraph.from_edges(*PATTERNS["wedge"])
    b = [c for c in sge.candidates(p, g.stats(), cap=64) if c.num_enum == 2][0]
    assert b.tail_mode == 1 and bin(b.parents[2]).count("1") == 1 and b.root_kind == 0
    off, nb = g.offsets, g.nbrs
    roots = [(u, int(v)) for u in range(g.num_vertices) for v in nb[off[u]:off[u + 1]] if v > u]
    want = 0
    for u, v in roots:
        for a, c in ((u, v), (v, u)):  # both orientations (unordered root)
            m = (a, c)
            par = 0 if b.parents[2] & 1 else 1
            lst = nb[off[m[par]]:off[m[par] + 1]]
            keep = np.ones(lst.size, bool)
            for j in range(2):
                if (b.lower[2] >> j) & 1:
                    keep &= lst > m[j]
                if (b.upper[2] >> j) & 1:
                    keep &= lst < m[j]
            want += 4 * (2 + bin(b.check[2]).count("1")) * int(np.floor(np.log2(int(keep.sum()) + 1)))
    assert oracle.alg_bytes_root_leaf(off, nb, b) == want
    deeper = sge.plan(sge.PatternGraph.from_edges(*PATTERNS["diamond"]), g.stats(), iep=False)
    if deeper.num_enum != 2:
        with pytest.raises(ValueError):
            oracle.alg_bytes_root_leaf(off, nb, deeper)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", ["chunglu_n380", "chunglu_n7100"])
def test_device_counter_matches_its_definition(sge, oracle, graphs, graph):
    g = graphs(graph)
    plans = root_leaf_plans(sge, g.stats())
    assert len(plans) >= 40
    modes = {b.tail_mode for _, b in plans}
    assert modes == {1, 2, 3}
    with sge.Engine(g) as eng:
        hub_min = eng.info()["hub_min_degree"]
        bad = []
        for name, b in plans:
            for hubs, sample in ((False, {}), (True, {}), (True, dict(root_stride=3, root_offset=1, root_max_degree=40))):
                _, _, st = eng.count([b], stats=True, hub_bitmaps=hubs, **sample)
                want = oracle.alg_bytes_root_leaf(g.offsets, g.nbrs, b, stride=sample.get("root_stride", 1),
                                                  offset=sample.get("root_offset", 0),
                                                  root_max_degree=sample.get("root_max_degree", 0),
                                                  hub_min=hub_min if hubs else 0xFFFFFFFF)
                if st["alg_bytes"] != want:
                    bad.append((name, b.tail_mode, b.root_kind, hubs, bool(sample), st["alg_bytes"], want))
        assert not bad, bad[:5]
