"""Labeled matching (the reference's LabeledGraph and candidate space,
relation/labeled_graph.cpp:63-143, relation/candidate_space.cpp:112-760; its
main() never reaches them, so the brute-force counter is the oracle): the
labeled text loader, label-preserving symmetry breaking, and on the GPU the
counts of labeled patterns against brute force."""
import numpy as np
import pytest

PATTERNS = {
    "triangle": (3, [(0, 1), (0, 2), (1, 2)]),
    "diamond": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3)]),
    "tailed_triangle": (4, [(0, 1), (0, 2), (1, 2), (0, 3)]),
    "cycle4": (4, [(0, 1), (1, 2), (2, 3), (0, 3)]),
    "star3": (4, [(0, 1), (0, 2), (0, 3)]),
    "house": (5, [(0, 1), (0, 2), (0, 4), (1, 3), (1, 4), (2, 3)]),
    "k4": (4, [(a, b) for a in range(4) for b in range(a + 1, 4)]),
}


def labelings(k, nlab, seed):
    rng = np.random.default_rng(seed)
    out = [[0] * k, [i % 2 for i in range(k)]]
    out += [rng.integers(0, nlab, k).tolist() for _ in range(2)]
    return out


def test_labeled_text_round_trip(sge, graphs, tmp_path):
    g = graphs("chunglu_n380")
    lab = np.random.default_rng(3).integers(0, 5, g.num_vertices).astype(np.uint32)
    f = tmp_path / "g.lg"
    g.save_labeled_text(f, lab)
    g2, lab2 = sge.DataGraph.load_labeled(f)
    assert np.array_equal(g2.offsets, g.offsets) and np.array_equal(g2.nbrs, g.nbrs)
    assert np.array_equal(lab2, lab)
    bad = tmp_path / "bad.lg"
    bad.write_text("t 3 2\nv 0 1 1\nv 1 0 2\nv 2 0 2\ne 0 1\ne 1 2\n")  # vertex 2 declares degree 2
    with pytest.raises(sge.SgeError) as e:
        sge.DataGraph.load_labeled(bad)
    assert e.value.status_name == "IO_ERROR" and "declares degree" in str(e.value)
    bad.write_text("3 2\n0 1\n1 2\n")
    with pytest.raises(sge.SgeError):
        sge.DataGraph.load_labeled(bad)


def test_label_preserving_symmetry(sge, oracle):
    for name, (k, e) in PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, e)
        for lab in labelings(k, 3, 7):
            b = sge.plan(p, None, labels=lab)
            assert b.labeled == 1
            assert b.aut_size == oracle.aut_size_labeled(k, e, lab), (name, lab)
            assert b.count_multiplier in (1, b.aut_size)
        assert sge.plan(p, None).labeled == 0
    with pytest.raises(sge.SgeError) as ex:
        sge.plan(sge.PatternGraph.from_edges(*PATTERNS["house"]), None, labels=[0] * 5, exploration=True)
    assert ex.value.status_name == "UNSUPPORTED"


def test_labels_only_on_labeled_plans(sge):
    import ctypes as C
    p = sge.PatternGraph.from_edges(*PATTERNS["triangle"])
    ph = C.c_void_p()
    b = sge.plan(p, None)
    sge._check(sge.lib().sge_plan_create(C.byref(b), C.byref(ph)))
    lab = np.zeros(3, np.uint32)
    assert sge.STATUS[sge.lib().sge_plan_set_labels(ph, sge._u32p(lab))] == "BAD_INPUT"
    sge.lib().sge_plan_destroy(ph)


def expected(oracle, g, glab, k, e, lab, b):
    emb = oracle.bruteforce_embeddings_labeled(g.offsets, g.nbrs, k, e, lab, glab)
    assert emb % b.aut_size == 0
    return emb // b.aut_size * b.count_multiplier


@pytest.mark.gpu
@pytest.mark.parametrize("graph,nlab", [("ca_netscience", 3), ("chunglu_n380", 2), ("rmat_s12", 4)])
def test_labeled_counts_match_brute_force(sge, oracle, graphs, graph, nlab):
    g = graphs(graph)
    glab = np.random.default_rng(11).integers(0, nlab, g.num_vertices).astype(np.uint32)
    plans, labs, want = [], [], []
    with sge.Engine(g) as eng:
        eng.set_labels(glab)
        for name, (k, e) in PATTERNS.items():
            p = sge.PatternGraph.from_edges(k, e)
            for lab in labelings(k, nlab, 5):
                for iep in (False, True):
                    b = sge.plan(p, eng, iep=iep, labels=lab)
                    plans.append(b)
                    labs.append(lab)
                    want.append(expected(oracle, g, glab, k, e, lab, b))
        got, _, _ = eng.count(plans, labels=labs)
        # heavy roots split into tasks, and unlabeled plans beside labeled ones
        split, _, _ = eng.count(plans, labels=labs, heavy_threshold=8)
        plain = sge.plan(sge.PatternGraph.from_edges(*PATTERNS["house"]), eng)
        mixed, _, _ = eng.count([plain] + plans[:6], labels=[None] + labs[:6])
    bad = [(i, g_, w) for i, (g_, w) in enumerate(zip(got, want)) if g_ != w]
    assert not bad, bad[:5]
    assert split == want and mixed[1:] == want[:6]
    assert sum(w > 0 for w in want) > len(want) // 2


@pytest.mark.gpu
def test_labeled_plans_need_labels(sge, graphs):
    g = graphs("chunglu_n380")
    b = sge.plan(sge.PatternGraph.from_edges(*PATTERNS["triangle"]), g, labels=[0, 1, 1])
    with sge.Engine(g) as eng:
        with pytest.raises(sge.SgeError) as e:
            eng.count([b], labels=[[0, 1, 1]])       # the graph has no labels
        assert e.value.status_name == "BAD_INPUT"
        eng.set_labels(np.zeros(g.num_vertices, np.uint32))
        with pytest.raises(sge.SgeError) as e:
            eng.count([b])                           # the plan has none
        assert e.value.status_name == "BAD_INPUT"
        assert eng.count([b], labels=[[0, 1, 1]])[0] == [0]   # no vertex has label 1


def test_labeled_brute_force_partitions_the_embeddings(sge, oracle, graphs):
    """Each embedding induces one pattern labeling (its images' labels), so the
    labeled counts over all 2^k labelings add up to the unlabeled count."""
    import itertools
    g = graphs("ca_netscience")
    glab = np.random.default_rng(2).integers(0, 2, g.num_vertices).astype(np.uint32)
    for name in ("diamond", "tailed_triangle", "cycle4"):
        k, e = PATTERNS[name]
        total = sum(oracle.bruteforce_embeddings_labeled(g.offsets, g.nbrs, k, e, list(lab), glab)
                    for lab in itertools.product((0, 1), repeat=k))
        assert total == oracle.bruteforce_embeddings(g.offsets, g.nbrs, k, e), name
