"""ctypes binding of liboracle.so (oracle/sge_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline/reference arm, never by the product.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

SO = Path(__file__).resolve().parent / "_build" / "liboracle.so"
_lib = None
u32, u64 = C.c_uint32, C.c_uint64
_P = C.POINTER


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not SO.exists():
            raise FileNotFoundError(f"{SO} missing: run __graft_entry__.build()")
        L = C.CDLL(str(SO))
        L.oracle_choosec_ref.restype = u64
        L.oracle_choosec_ref.argtypes = [u64, C.c_int]
        L.oracle_binom_exact.restype = u64
        L.oracle_binom_exact.argtypes = [u64, C.c_int]
        L.oracle_set_begin_pos.restype = u32
        L.oracle_set_begin_pos.argtypes = [_P(u32), u32, u32]
        L.oracle_set_end_pos.restype = u32
        L.oracle_set_end_pos.argtypes = [_P(u32), u32, u32]
        L.oracle_intersect.restype = u32
        L.oracle_intersect.argtypes = [_P(u32), u32, _P(u32), u32, _P(u32)]
        L.oracle_intersect_count.restype = u32
        L.oracle_intersect_count.argtypes = [_P(u32), u32, _P(u32), u32]
        L.oracle_num_results.restype = u64
        L.oracle_num_results.argtypes = [_P(u32), u32, _P(u32), _P(u32), u32, _P(u32), u32, _P(u32), u32]
        L.oracle_num_unique_combine.restype = u64
        L.oracle_num_unique_combine.argtypes = [_P(_P(u32)), _P(u32), C.c_int]
        L.oracle_aut_size.restype = u64
        L.oracle_aut_size.argtypes = [u32, u32, _P(u32)]
        L.oracle_bruteforce_embeddings.restype = u64
        L.oracle_bruteforce_embeddings.argtypes = [_P(u32), _P(u32), u32, u32, u32, _P(u32), C.c_int]
        L.oracle_count_plan.restype = u64
        L.oracle_count_plan.argtypes = [_P(u32), _P(u32), u32, C.c_void_p, C.c_int, u64, u64, _P(u64)]
        L.oracle_count_plans.restype = None
        L.oracle_count_plans.argtypes = [_P(u32), _P(u32), u32, C.c_void_p, u32, C.c_int, u64, u64, u32, _P(u64),
                                         _P(u64)]
        L.oracle_ctx_create.restype = C.c_void_p
        L.oracle_ctx_create.argtypes = [_P(u32), _P(u32), u32]
        L.oracle_ctx_free.restype = None
        L.oracle_ctx_free.argtypes = [C.c_void_p]
        L.oracle_ctx_count_plans.restype = None
        L.oracle_ctx_count_plans.argtypes = [C.c_void_p, C.c_void_p, u32, C.c_int, u64, u64, u32, _P(u64), _P(u64)]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_list_embeddings.restype = u64
        L.oracle_list_embeddings.argtypes = [_P(u32), _P(u32), u32, u32, u32, _P(u32), _P(u32), u64]
        L.oracle_gen_rmat.restype = C.c_int
        L.oracle_gen_rmat.argtypes = [u32, u64, u32, u32, u32, u64, _P(_P(u32)), _P(u64)]
        L.oracle_gen_chung_lu.restype = C.c_int
        L.oracle_gen_chung_lu.argtypes = [u32, u64, u32, u32, u64, _P(_P(u32)), _P(u64)]
        L.oracle_csr_from_sorted_edges.restype = None
        L.oracle_csr_from_sorted_edges.argtypes = [_P(u32), u64, u32, _P(u32), _P(u32)]
        L.oracle_free.restype = None
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_aut_size_labeled.restype = u64
        L.oracle_aut_size_labeled.argtypes = [u32, u32, _P(u32), _P(u32)]
        L.oracle_bruteforce_embeddings_labeled.restype = u64
        L.oracle_bruteforce_embeddings_labeled.argtypes = [_P(u32), _P(u32), u32, u32, u32, _P(u32), _P(u32), _P(u32),
                                                          C.c_int]
        L.oracle_alg_bytes_root_leaf.restype = u64
        L.oracle_alg_bytes_root_leaf.argtypes = [_P(u32), _P(u32), u32, C.c_void_p, u64, u64, u32, u32]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_P(u32))


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.uint32)


def choosec_ref(n: int, k: int) -> int:
    return int(lib().oracle_choosec_ref(n, k))


def binom_exact(n: int, k: int) -> int:
    return int(lib().oracle_binom_exact(n, k))


def set_begin_pos(a, bound: int) -> int:
    a = _arr(a)
    return int(lib().oracle_set_begin_pos(_p(a), a.size, bound))


def set_end_pos(a, bound: int) -> int:
    a = _arr(a)
    return int(lib().oracle_set_end_pos(_p(a), a.size, bound))


def intersect(a, b) -> np.ndarray:
    a, b = _arr(a), _arr(b)
    out = np.zeros(max(min(a.size, b.size), 1), np.uint32)
    n = lib().oracle_intersect(_p(a), a.size, _p(b), b.size, _p(out))
    return out[:n]


def intersect_count(a, b) -> int:
    a, b = _arr(a), _arr(b)
    return int(lib().oracle_intersect_count(_p(a), a.size, _p(b), b.size))


def num_results(values, part_match, to_check, larger, smaller) -> int:
    v, pm, tc, lg, sm = map(_arr, (values, part_match, to_check, larger, smaller))
    return int(lib().oracle_num_results(_p(v), v.size, _p(pm), _p(tc), tc.size, _p(lg), lg.size, _p(sm), sm.size))


def num_unique_combine(sets) -> int:
    arrs = [_arr(s) for s in sets]
    ptrs = (_P(u32) * len(arrs))(*[_p(a) for a in arrs])
    lens = (u32 * len(arrs))(*[a.size for a in arrs])
    return int(lib().oracle_num_unique_combine(ptrs, lens, len(arrs)))


def aut_size(k: int, edges) -> int:
    e = _arr(edges).reshape(-1)
    return int(lib().oracle_aut_size(k, e.size // 2, _p(e)))


def bruteforce_embeddings(offsets, nbrs, k: int, edges, threads: int = 0) -> int:
    off, nb, e = _arr(offsets), _arr(nbrs), _arr(edges).reshape(-1)
    return int(lib().oracle_bruteforce_embeddings(_p(off), _p(nb), off.size - 1, k, e.size // 2, _p(e), threads))


def count_plan(offsets, nbrs, blob, threads: int = 0, stride: int = 1, offset: int = 0) -> tuple[int, int]:
    """Runs a plan blob on the CPU.  Returns (instances over the sampled roots, roots done)."""
    off, nb = _arr(offsets), _arr(nbrs)
    done = u64()
    r = lib().oracle_count_plan(_p(off), _p(nb), off.size - 1, C.addressof(blob), threads, stride, offset,
                                C.byref(done))
    return int(r), int(done.value)


def count_plans(offsets, nbrs, blobs: bytes, nplans: int, threads: int = 0, stride: int = 1,
                offset: int = 0, root_max_degree: int = 0) -> tuple[list[int], list[int]]:
    """Runs nplans plan blobs (their raw bytes back to back) over the same root
    sample (undirected edges e ≡ offset mod stride; root_max_degree > 0 keeps
    the roots whose endpoints both have at most that degree).  Returns
    (instances per plan, root tasks per plan)."""
    off, nb = _arr(offsets), _arr(nbrs)
    buf = C.create_string_buffer(bytes(blobs), len(blobs))
    counts = (u64 * nplans)()
    roots = (u64 * nplans)()
    lib().oracle_count_plans(_p(off), _p(nb), off.size - 1, C.addressof(buf), nplans, threads, stride, offset,
                             root_max_degree, counts, roots)
    return [int(x) for x in counts], [int(x) for x in roots]


class Graph:
    """A CSR prepared once (root edge list) for many counting calls."""

    def __init__(self, offsets, nbrs):
        self.off, self.nb = _arr(offsets), _arr(nbrs)
        self._h = lib().oracle_ctx_create(_p(self.off), _p(self.nb), self.off.size - 1)

    def count_plans(self, blobs: bytes, nplans: int, threads: int = 0, stride: int = 1, offset: int = 0,
                    root_max_degree: int = 0) -> tuple[list[int], list[int]]:
        """As count_plans(), on this graph."""
        buf = C.create_string_buffer(bytes(blobs), len(blobs))
        counts = (u64 * nplans)()
        roots = (u64 * nplans)()
        lib().oracle_ctx_count_plans(self._h, C.addressof(buf), nplans, threads, stride, offset, root_max_degree,
                                     counts, roots)
        return [int(x) for x in counts], [int(x) for x in roots]

    def close(self):
        if getattr(self, "_h", None):
            lib().oracle_ctx_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def list_embeddings(offsets, nbrs, k: int, edges, cap: int = 1 << 22) -> np.ndarray:
    """Every embedding as k ids in pattern-vertex order (brute force)."""
    off, nb, e = _arr(offsets), _arr(nbrs), _arr(edges).reshape(-1)
    out = np.zeros(cap * k, np.uint32)
    n = int(lib().oracle_list_embeddings(_p(off), _p(nb), off.size - 1, k, e.size // 2, _p(e), _p(out), cap))
    if n > cap:
        raise ValueError(f"{n} embeddings exceed cap {cap}")
    return out[: n * k].reshape(n, k)


def canonical_instances(emb: np.ndarray, perms: np.ndarray) -> np.ndarray:
    """One row per instance: the lexicographically smallest image of an
    embedding under the automorphisms, unique, sorted."""
    imgs = np.stack([emb[:, p] for p in perms])           # naut × n × k
    # lexicographic minimum over automorphisms, row by row
    best = imgs[0].copy()
    for a in range(1, imgs.shape[0]):
        cand = imgs[a]
        less = np.zeros(len(best), bool)
        decided = np.zeros(len(best), bool)
        for j in range(best.shape[1]):
            lt = (cand[:, j] < best[:, j]) & ~decided
            gt = (cand[:, j] > best[:, j]) & ~decided
            less |= lt
            decided |= lt | gt
        best[less] = cand[less]
    return np.unique(best, axis=0)


def _take_edges(ep, m: int) -> np.ndarray:
    e = np.ctypeslib.as_array(ep, shape=(2 * max(m, 1),))[: 2 * m].copy()
    lib().oracle_free(C.cast(ep, C.c_void_p))
    return e


def csr_from_sorted_edges(edges: np.ndarray, n: int) -> tuple[np.ndarray, np.ndarray]:
    """Symmetric sorted CSR (offsets, neighbours) of sorted distinct u<v pairs."""
    e = _arr(edges).reshape(-1)
    m = e.size // 2
    off = np.zeros(n + 1, np.uint32)
    nb = np.zeros(max(2 * m, 1), np.uint32)
    lib().oracle_csr_from_sorted_edges(_p(e), m, n, _p(off), _p(nb))
    return off, nb[: 2 * m]


def gen_rmat(scale: int, m: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """The library's seeded R-MAT graph (sge_gen_rmat), built without the library: (offsets, neighbours)."""
    ep, mo = _P(u32)(), u64()
    if not lib().oracle_gen_rmat(scale, m, round(a * 1e6), round(b * 1e6), round(c * 1e6), seed, C.byref(ep),
                                 C.byref(mo)):
        raise ValueError("oracle_gen_rmat: bad arguments")
    return csr_from_sorted_edges(_take_edges(ep, mo.value), 1 << scale)


def gen_chung_lu(n: int, m: int, gamma: float, max_deg: int = 0, seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """The library's seeded Chung-Lu graph (sge_gen_chung_lu), built without the library."""
    ep, mo = _P(u32)(), u64()
    if not lib().oracle_gen_chung_lu(n, m, round(gamma * 1000), max_deg, seed, C.byref(ep), C.byref(mo)):
        raise ValueError("oracle_gen_chung_lu: bad arguments")
    return csr_from_sorted_edges(_take_edges(ep, mo.value), n)


def alg_bytes_root_leaf(offsets, nbrs, blob, stride: int = 1, offset: int = 0, root_max_degree: int = 0,
                        hub_min: int = 0xFFFFFFFF) -> int:
    """The instrumented kernel's algorithmic bytes for a WCOJ plan with two
    enumerated levels, from the counter's definition (sge_oracle.c, part 5);
    hub_min is the graph's hub threshold (0xFFFFFFFF: no hub bitmaps)."""
    off, nb = _arr(offsets), _arr(nbrs)
    r = lib().oracle_alg_bytes_root_leaf(_p(off), _p(nb), off.size - 1, C.addressof(blob), stride, offset,
                                         root_max_degree, hub_min)
    if r == (1 << 64) - 1:
        raise ValueError("alg_bytes_root_leaf needs a WCOJ plan with two enumerated levels")
    return int(r)


def aut_size_labeled(k: int, edges, labels) -> int:
    """Automorphisms that preserve adjacency and the vertex labels."""
    e = np.ascontiguousarray(np.asarray(edges, np.uint32).reshape(-1))
    lab = np.ascontiguousarray(labels, np.uint32)
    return int(lib().oracle_aut_size_labeled(k, e.size // 2, _p(e), _p(lab)))


def bruteforce_embeddings_labeled(offsets, nbrs, k: int, edges, pattern_labels, graph_labels,
                                  threads: int = 0) -> int:
    """Embeddings of a labeled pattern (pattern vertex u onto vertices of label
    pattern_labels[u] only), by brute-force DFS."""
    off, nb = _arr(offsets), _arr(nbrs)
    e = np.ascontiguousarray(np.asarray(edges, np.uint32).reshape(-1))
    pl = np.ascontiguousarray(pattern_labels, np.uint32)
    gl = np.ascontiguousarray(graph_labels, np.uint32)
    return int(lib().oracle_bruteforce_embeddings_labeled(_p(off), _p(nb), off.size - 1, k, e.size // 2, _p(e), _p(pl),
                                                          _p(gl), threads))
