"""The CPU oracle, pinned before it is trusted: its restated reference
primitives against independent statements of the same functions, its
brute-force counter and its plan executor against the reference's recorded
counts (tests/golden/golden_counts.json)."""
import itertools
import random

import numpy as np
import pytest

from conftest import golden_rows, pattern_of


def test_choosec_matches_exact_binomial_until_the_reference_wraps(oracle):
    from math import comb
    for n in [0, 1, 2, 5, 1000, 65535, 65536, 2**20]:
        for k in range(0, 5):
            exact = comb(n, k) % 2**64
            assert oracle.binom_exact(n, k) == exact
            if n ** k < 2**64:
                assert oracle.choosec_ref(n, k) == exact
    # the reference's nom = n(n-1)(n-2)(n-3) wraps for n > 65536 at k = 4
    n = 100000
    assert oracle.choosec_ref(n, 4) != comb(n, 4)
    nom = 1
    for i in range(4):
        nom = (nom * (n - i)) % 2**64
    assert oracle.choosec_ref(n, 4) == nom // 24


@pytest.mark.parametrize("count", [0, 1, 5, 31, 32, 33, 200])
def test_bound_positions(oracle, count):
    rng = np.random.default_rng(count)
    a = np.unique(rng.integers(0, 1000, count * 2 + 1))[:count].astype(np.uint32)
    for bound in [0, 1, 500, 999, 1000, 2**32 - 1] + (a.tolist()[:5] if count else []):
        assert oracle.set_begin_pos(a, bound) == int(np.searchsorted(a, bound, side="right"))
        assert oracle.set_end_pos(a, bound) == int(np.searchsorted(a, bound, side="left"))


@pytest.mark.parametrize("na,nb", [(0, 5), (5, 0), (10, 10), (3, 200), (200, 3), (1, 10000), (64, 64 * 33),
                                   (50, 50 * 51), (32, 32 * 32), (1000, 1000)])
def test_intersections(oracle, na, nb):
    rng = np.random.default_rng(na * 7919 + nb)
    universe = max(na, nb) * 3 + 10
    a = np.unique(rng.integers(0, universe, na * 2)).astype(np.uint32)[:na]
    b = np.unique(rng.integers(0, universe, nb * 2)).astype(np.uint32)[:nb]
    want = np.intersect1d(a, b)
    assert np.array_equal(oracle.intersect(a, b), want)
    assert oracle.intersect_count(a, b) == want.size


def test_num_results_subtracts_matched_vertices_in_range(oracle):
    values = np.arange(0, 100, 3, dtype=np.uint32)
    pm = np.array([30, 31, 60, 99, 12], np.uint32)
    # range (12, 60): 15..57 step 3 = 15 values; 30 is inside and matched, 31 not a value
    got = oracle.num_results(values, pm, [0, 1], larger=[4], smaller=[2])
    assert got == 15 - 1
    assert oracle.num_results(values, pm, [], [], []) == values.size


def brute_unique(sets):
    return sum(1 for t in itertools.product(*sets) if len(set(t)) == len(t))


@pytest.mark.parametrize("seed", range(12))
def test_num_unique_combine(oracle, seed):
    rng = random.Random(seed)
    nsets = 2 + seed % 3
    sets = [sorted(rng.sample(range(12), rng.randint(0, 7))) for _ in range(nsets)]
    assert oracle.num_unique_combine(sets) == brute_unique(sets)


def test_bruteforce_matches_reference_counts(sge, oracle, patterns, golden, graphs):
    g = graphs("ca_netscience")
    rows = [r for r in golden_rows(golden, "ca_netscience") if not r["pattern"].startswith(("batch7", "random"))]
    assert len(rows) > 100
    for r in rows[::3]:
        p = pattern_of(sge, patterns, r["pattern"])
        aut = oracle.aut_size(p.k, p.edges)
        emb = oracle.bruteforce_embeddings(g.offsets, g.nbrs, p.k, p.edges)
        want = emb if r["num_bags"] == 1 else emb // aut
        assert emb % aut == 0
        assert want == r["count"], r


@pytest.mark.parametrize("graph", ["ca_netscience", "chunglu_n380"])
def test_plan_executor_matches_reference(sge, oracle, patterns, golden, graphs, graph):
    g = graphs(graph)
    st = g.stats()
    rows = golden_rows(golden, graph)
    assert rows
    for r in rows:
        p = pattern_of(sge, patterns, r["pattern"])
        b = sge.plan(p, st, iep=True)
        inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=4)
        assert inst * b.count_multiplier == r["count"], r


def test_plan_executor_matches_reference_on_chunglu_n7100(sge, oracle, patterns, golden, graphs):
    g = graphs("chunglu_n7100")
    st = g.stats()
    for r in golden_rows(golden, "chunglu_n7100"):
        if r["pattern"] not in ("light_query/p2", "light_query/p6", "k5_minus_e"):
            continue
        p = pattern_of(sge, patterns, r["pattern"])
        b = sge.plan(p, st, iep=True)
        inst, _ = oracle.count_plan(g.offsets, g.nbrs, b, threads=8)
        assert inst * b.count_multiplier == r["count"], r
