"""sge_count_noalloc: counting for callers that cannot allocate device memory
(a host framework that owns the GPU memory pool, a caller with a fixed memory
budget).  The caller passes device inputs and outputs; the launch works in the
library's fixed static device array.  Its counts must equal sge_count's on the
same plans, on consecutive calls (the array keeps the previous call's
contents, which must not leak into the next result)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_rows, pattern_of

pytestmark = pytest.mark.gpu


def _dev_u32(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def _noalloc(sge, torch, g, plans, max_degree=None):
    off = _dev_u32(torch, g.offsets)
    nb = _dev_u32(torch, g.nbrs if g.nbrs.size else np.zeros(1, np.uint32))
    out = torch.full((len(plans),), 7, dtype=torch.int64, device="cuda")  # garbage the call must clear
    arr = (sge.PlanBlob * len(plans))(*plans)
    stream = torch.cuda.current_stream().cuda_stream
    md = g.max_degree if max_degree is None else max_degree
    st = sge.lib().sge_count_noalloc(C.c_void_p(off.data_ptr()), C.c_void_p(nb.data_ptr()), g.num_vertices,
                                     g.nbrs.size, md, arr, len(plans), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(stream))
    torch.cuda.synchronize()
    return st, [int(x) for x in out.cpu().numpy().view(np.uint64)]


def test_noalloc_matches_sge_count_on_consecutive_calls(sge, patterns, golden, graphs):
    torch = pytest.importorskip("torch")
    g = graphs("ca_netscience")
    rows = golden_rows(golden, "ca_netscience")
    sets = [rows[:40], rows[40:90:2]]
    with sge.Engine(g) as eng:
        for batch in sets + sets:  # consecutive calls with different and repeated batches
            plans = [sge.plan(pattern_of(sge, patterns, r["pattern"]), eng, iep=i % 2 == 0,
                              exploration=i % 3 == 0) for i, r in enumerate(batch)]
            want, _, _ = eng.count(plans)
            st, got = _noalloc(sge, torch, g, plans)
            assert sge.STATUS[st] == "OK", sge.lib().sge_last_error()
            assert got == want
            assert got == [r["count"] for r in batch]


def test_noalloc_larger_graph_two_calls(sge, patterns, golden, graphs):
    torch = pytest.importorskip("torch")
    g = graphs("chunglu_n7100")
    names = ["light_query/p2", "light_query/p4", "k5_minus_e", "light_query/p6", "light_query/p3"]
    with sge.Engine(g) as eng:
        plans = [sge.plan(pattern_of(sge, patterns, n), eng) for n in names]
        want, _, _ = eng.count(plans)
    for _ in range(2):
        st, got = _noalloc(sge, torch, g, plans)
        assert sge.STATUS[st] == "OK", sge.lib().sge_last_error()
        assert got == want


def test_noalloc_limits_are_reported(sge, patterns, graphs):
    torch = pytest.importorskip("torch")
    g = graphs("chunglu_n7100")
    plans = [sge.plan(pattern_of(sge, patterns, "6vertex/4"), g.stats(), iep=False)]
    st, _ = _noalloc(sge, torch, g, plans, max_degree=1 << 24)   # lists cannot fit the static array
    assert sge.STATUS[st] == "UNSUPPORTED"
    assert b"static" in sge.lib().sge_last_error()
    st, _ = _noalloc(sge, torch, g, plans, max_degree=8)         # under-stated bound: reported
    assert sge.STATUS[st] == "STACK_OVERFLOW"
    too_many = [plans[0]] * 65
    st, _ = _noalloc(sge, torch, g, too_many)
    assert sge.STATUS[st] == "UNSUPPORTED"
    st, got = _noalloc(sge, torch, g, plans)                     # and the next call is clean
    assert sge.STATUS[st] == "OK"
