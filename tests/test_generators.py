"""Seeded generators: deterministic (fingerprints pinned in the golden file),
clean (no self-loops or duplicates), and shaped as configured."""
import numpy as np


def test_golden_graph_fingerprints(graphs, golden):
    for name in golden["graphs"]:
        graphs(name)  # asserts the fingerprint


def test_rmat_clean_and_sized(sge):
    g = sge.gen_rmat(10, 5000, seed=7)
    assert g.num_edges == 5000
    e = g.edge_array()
    assert (e[:, 0] < e[:, 1]).all()
    assert len({(a, b) for a, b in e.tolist()}) == 5000
    g2 = sge.gen_rmat(10, 5000, seed=7)
    assert g2.fingerprint() == g.fingerprint()
    assert sge.gen_rmat(10, 5000, seed=8).fingerprint() != g.fingerprint()


def test_chung_lu_degree_shape(sge):
    g = sge.gen_chung_lu(7100, 100000, 2.1, 1000, 2)
    deg = np.diff(g.offsets)
    assert g.num_edges == 100000
    assert deg.max() <= 1100 and deg.max() > 500
    assert np.sort(deg)[-10:].mean() > 20 * deg.mean()


def test_random_patterns_connected(sge):
    for k in range(3, 9):
        for m in range(k - 1, k * (k - 1) // 2 + 1):
            p = sge.PatternGraph.random(k, m, 11 * k + m)
            assert p.m == m
            adj = np.zeros((k, k), bool)
            adj[p.edges[:, 0], p.edges[:, 1]] = adj[p.edges[:, 1], p.edges[:, 0]] = True
            seen = {0}
            frontier = [0]
            while frontier:
                u = frontier.pop()
                for w in np.nonzero(adj[u])[0]:
                    if w not in seen:
                        seen.add(int(w))
                        frontier.append(int(w))
            assert len(seen) == k


def test_oracle_generators_build_the_library_graphs(sge, oracle):
    # the CPU reference arm builds its graphs without the library
    import numpy as np
    for args in [(10, 8000, 0.57, 0.19, 0.19, 4), (14, 1 << 18, 0.57, 0.19, 0.19, 4)]:
        g = sge.gen_rmat(*args)
        off, nb = oracle.gen_rmat(*args)
        assert np.array_equal(g.offsets, off) and np.array_equal(g.nbrs, nb)
    for args in [(380, 915, 2.3, 0, 1), (7100, 100_000, 2.1, 1000, 2)]:
        g = sge.gen_chung_lu(*args)
        off, nb = oracle.gen_chung_lu(*args)
        assert np.array_equal(g.offsets, off) and np.array_equal(g.nbrs, nb)
