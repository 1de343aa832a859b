"""Bag relations on the device: enumeration, canonical instance sets, the
LSD radix sort of tuples and trie levels, against CPU restatements."""
import numpy as np
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


@pytest.mark.parametrize("arity,n,hi", [(1, 1, 10), (1, 5000, 50), (2, 100_000, 1 << 32), (3, 70_001, 7),
                                        (5, 20_000, 300), (4, 1025, 1 << 20)])
def test_radix_sort_matches_lexsort(sge, arity, n, hi):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(arity * 1000 + n)
    a = rng.integers(0, hi, size=(n, arity), dtype=np.uint64).astype(np.uint32)
    d = _dev(torch, a)
    sge.sort_tuples_device(d.data_ptr(), n, arity)
    got = d.cpu().numpy().view(np.uint32).reshape(n, arity)
    want = a[np.lexsort(a.T[::-1])]
    assert np.array_equal(got, want)


def trie_reference(rows):
    """TrieLevel::buildTrieFromSortedMatchesBatch (relation/relation.cpp:340-379),
    flattened: per level the values, and per node its child range."""
    arity = rows.shape[1]
    values = [[] for _ in range(arity)]
    child = [[] for _ in range(arity - 1)]

    def build(start, end, depth):
        if depth == arity - 1:
            values[depth].extend(rows[start:end, depth].tolist())
            return
        i = start
        while i < end:
            j = i
            while j < end and rows[j, depth] == rows[i, depth]:
                j += 1
            values[depth].append(int(rows[i, depth]))
            child[depth].append(len(values[depth + 1]))
            build(i, j, depth + 1)
            i = j
    build(0, len(rows), 0)
    return values, child


def test_trie_levels_match_reference_grouping(sge):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    rows = np.unique(rng.integers(0, 12, size=(3000, 3)).astype(np.uint32), axis=0)
    d = _dev(torch, rows)
    t = sge.trie_build_device(d.data_ptr(), len(rows), 3)
    try:
        want_vals, want_child = trie_reference(rows)
        for lvl in range(3):
            vals, child = sge.trie_level(t, lvl)
            assert vals.tolist() == want_vals[lvl]
            if lvl < 2:
                assert child[:-1].tolist() == want_child[lvl] and int(child[-1]) == t.level_len[lvl + 1]
    finally:
        sge.trie_free(t)


@pytest.mark.parametrize("name", ["light_query/p2", "light_query/p3", "light_query/p4", "light_query/p7",
                                  "huge_query/p5", "6vertex/3", "k4_pendant"])
def test_match_set_equals_brute_force_instances(sge, oracle, patterns, golden, graphs, name):
    g = graphs("ca_netscience")
    p = pattern_of(sge, patterns, name)
    with sge.Engine(g) as eng:
        got = eng.match_set(p)
    emb = oracle.list_embeddings(g.offsets, g.nbrs, p.k, p.edges)
    perms = np.array(sge_perms(sge, p))
    want = oracle.canonical_instances(emb, perms)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    r = [r for r in golden_rows(golden, "ca_netscience") if r["pattern"] == name]
    if r:
        aut, single = p.info()
        assert len(got) * (aut if single else 1) == r[0]["count"]


def sge_perms(sge, p):
    import ctypes as C
    cap = 4096
    out = (C.c_uint8 * (cap * p.k))()
    n = C.c_uint32()
    e = p.flat()
    sge._check(sge.lib().sge_pattern_automorphisms(p.k, p.m, sge._u32p(e), out, cap, C.byref(n)))
    return [list(out[i * p.k:(i + 1) * p.k]) for i in range(n.value)]
