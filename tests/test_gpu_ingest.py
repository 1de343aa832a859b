"""Device graph ingest: CSR built on the GPU from a device edge list, and
R-MAT graphs generated on the GPU, against the host generator and host CSR
build (Graph::addDirectedEdges, relation/graph.cpp:143-173)."""
import numpy as np
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


def device_u32(torch, a):
    """A device copy of uint32 ids (all < 2^31 here, so the int32 view is exact)."""
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


@pytest.mark.parametrize("scale,m,seed", [(6, 100, 1), (10, 8000, 4), (12, 40000, 7), (15, 300000, 3)])
def test_rmat_device_matches_host_generator(sge, scale, m, seed):
    host = sge.gen_rmat(scale, m, seed=seed)
    with sge.Engine.rmat_device(scale, m, seed=seed) as eng:
        off, nb = eng.csr()
        assert eng.info()["num_directed_edges"] == 2 * m
    assert np.array_equal(off, host.offsets)
    assert np.array_equal(nb, host.nbrs)


def test_device_edges_drop_repeats_and_self_loops(sge):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    n = 300
    e = rng.integers(0, n, size=(5000, 2), dtype=np.uint32)
    e = np.concatenate([e, e[:100, ::-1], np.array([[7, 7], [9, 9], [n - 1, 0]], np.uint32)])
    rng.shuffle(e)
    d = device_u32(torch, e)
    with sge.Engine.from_device_edges(d.data_ptr(), len(e), n) as eng:
        off, nb = eng.csr()
    host = sge.DataGraph.from_edges(e, n, dedup=True)
    assert np.array_equal(off, host.offsets)
    assert np.array_equal(nb, host.nbrs)


def test_device_built_graph_counts_like_the_host_built_one(sge, patterns, golden, graphs):
    torch = pytest.importorskip("torch")
    g = graphs("ca_netscience")
    src = np.repeat(np.arange(g.num_vertices, dtype=np.uint32), np.diff(g.offsets))
    keep = src < g.nbrs
    e = np.stack([g.nbrs[keep], src[keep]], 1)  # reversed pairs, CSR order
    d = device_u32(torch, e)
    rows = golden_rows(golden, "ca_netscience")[:40]
    with sge.Engine.from_device_edges(d.data_ptr(), len(e), g.num_vertices) as eng:
        off, nb = eng.csr()
        assert np.array_equal(off, g.offsets) and np.array_equal(nb, g.nbrs)
        plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=i % 2 == 0) for i, r in enumerate(rows)]
        counts, _, _ = eng.count(plans)
    assert counts == [r["count"] for r in rows]


def test_device_rmat_counts_match_oracle(sge, oracle):
    host = sge.gen_rmat(11, 20000, seed=9)
    p = sge.PatternGraph.from_edges(4, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)])
    with sge.Engine.rmat_device(11, 20000, seed=9) as eng:
        b = sge.plan(p, eng)
        counts, _, _ = eng.count([b])
    inst, _ = oracle.count_plan(host.offsets, host.nbrs, b)
    assert counts[0] == inst * b.count_multiplier


def test_empty_and_bad_edge_lists(sge):
    torch = pytest.importorskip("torch")
    d = device_u32(torch, np.zeros((1, 2), np.uint32))
    with sge.Engine.from_device_edges(d.data_ptr(), 0, 5) as eng:
        off, nb = eng.csr()
        assert off.tolist() == [0] * 6 and nb.size == 0
    bad = device_u32(torch, np.array([[0, 1], [2, 10]], np.uint32))
    with pytest.raises(sge.SgeError) as ei:
        sge.Engine.from_device_edges(bad.data_ptr(), 2, 10)
    assert ei.value.status_name == "BAD_INPUT"
    with pytest.raises(sge.SgeError):
        sge.Engine.rmat_device(4, 1000, seed=1)  # too dense for 16 vertices



def test_large_host_csr_is_checked_on_the_device(sge):
    """Above 2^22 directed entries sge_graph_create checks the lists on the
    device (the offsets still on the host): the same errors as the host check."""
    import ctypes as C
    g = sge.gen_rmat(18, 3_000_000, seed=2)
    off, nb = g.offsets.copy(), g.nbrs.copy()
    assert nb.size > (1 << 22)
    with sge.Engine(g) as eng:
        assert eng.info()["num_directed_edges"] == nb.size
    deg = np.diff(off)
    v = int(np.argmax(deg > 8))  # a vertex with a list long enough to edit in place
    a = int(off[v])
    lst = nb[a:a + int(deg[v])]
    gap = int(np.argmax(np.diff(lst.astype(np.int64)) > 1))  # two entries with room between them
    cases = {}
    bad = nb.copy(); bad[a + gap], bad[a + gap + 1] = bad[a + gap + 1], bad[a + gap]
    cases["strictly increasing"] = bad                      # two entries swapped
    bad = nb.copy(); bad[a + gap] = lst[gap] + 1
    cases["not symmetric"] = bad                            # an entry with no reverse entry
    bad = nb.copy(); bad[-1] = g.num_vertices
    cases["out of range"] = bad                             # the last list's last entry past n
    for want, arr in cases.items():
        h = C.c_void_p()
        st = sge.lib().sge_graph_create(sge._u32p(off), sge._u32p(arr), g.num_vertices, arr.size, 0, C.byref(h))
        assert sge.STATUS[st] == "BAD_INPUT", want
        assert want in sge.lib().sge_last_error().decode(), (want, sge.lib().sge_last_error())
