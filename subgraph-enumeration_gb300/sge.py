"""Python mirror of the libsge C ABI (include/sge.h), shaped like the
reference's own entry points so callers and tests read like the reference:

  reference (C++)                                  here
  ---------------------------------------------    ----------------------------------------
  DataGraph::loadDataGraph (relation/graph.cpp:255) DataGraph.load(path)
  PatternGraph::loadPatternGraph (graph.cpp:661)    PatternGraph.load(path)
  optCostPlan + selectSymmetry + buildTraverse…     plan(pattern, graph, iep=, exploration=)
    (main.cpp:60-69)
  sharedJoin / parSharedJoin (main.cpp:86,192)      Engine(graph).count(plans)
  singleThreadMatch / parallelMatch (main.cpp:12,114) match(query_path, data_path, iep=, exploration=)

The compute path is libsge.so (CUDA kernels for sm_103a).  There is no CPU
fallback: if the library or a GPU is missing, calls raise SgeError.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libsge.so"
CLI_PATH = _PKG / "_build" / "graph_mining_system"

SGE_MAX_K = 16
SGE_MAX_TAIL = 4
SGE_MAX_PARTITIONS = 15

STATUS = {0: "OK", 1: "BAD_INPUT", 2: "OOM", 3: "TIMEOUT", 4: "STACK_OVERFLOW", 5: "CUDA_ERROR",
          6: "UNSUPPORTED", 7: "IO_ERROR", 8: "NO_DEVICE"}
TAIL_SINGLE, TAIL_CHOOSE, TAIL_IEP = 1, 2, 3
JOIN_WCOJ, JOIN_EXPLORATION = 0, 1

u32, i32, u64 = C.c_uint32, C.c_int32, C.c_uint64


class SgeError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status
        self.status_name = STATUS.get(status, str(status))


class PlanBlob(C.Structure):
    _fields_ = [
        ("magic", u32), ("abi_version", u32), ("k", u32), ("num_enum", u32), ("tail_mode", u32),
        ("tail_len", u32), ("join_style", u32), ("root_kind", u32),
        ("order", u32 * SGE_MAX_K), ("parents", u32 * SGE_MAX_K), ("lower", u32 * SGE_MAX_K),
        ("upper", u32 * SGE_MAX_K), ("check", u32 * SGE_MAX_K), ("base", i32 * SGE_MAX_K),
        ("rest", u32 * SGE_MAX_K), ("first_parent", u32 * SGE_MAX_K),
        ("num_partitions", u32), ("part_coef", i32 * SGE_MAX_PARTITIONS),
        ("part_nblocks", u32 * SGE_MAX_PARTITIONS), ("part_block", (u32 * SGE_MAX_TAIL) * SGE_MAX_PARTITIONS),
        ("count_multiplier", u64), ("aut_size", u64), ("single_bag", u32), ("num_restrictions", u32),
        ("est_cost", C.c_double), ("choose_wrap", u32), ("labeled", u32),
    ]

    def summary(self) -> dict:
        return {"k": self.k, "order": list(self.order[: self.k]), "num_enum": self.num_enum,
                "tail_len": self.tail_len, "tail_mode": self.tail_mode, "join_style": self.join_style,
                "root_kind": self.root_kind, "single_bag": self.single_bag, "aut_size": self.aut_size,
                "count_multiplier": self.count_multiplier, "est_cost": self.est_cost}

    def to_bytes(self) -> bytes:
        return bytes(memoryview(self))

    @classmethod
    def from_bytes(cls, b: bytes) -> "PlanBlob":
        return cls.from_buffer_copy(b)


class PlanOpts(C.Structure):
    _fields_ = [("join_style", u32), ("use_iep", u32), ("max_tail", u32), ("seed", u64),
                ("force_order", C.POINTER(u32)), ("symmetry_seq", C.POINTER(u32)), ("root_edge", C.POINTER(u32)),
                ("vertex_labels", C.POINTER(u32))]


class CountOpts(C.Structure):
    _fields_ = [("blocks_per_sm", u32), ("warps_per_block", u32), ("chunk", u32), ("time_budget_s", C.c_double),
                ("max_level_capacity", u32), ("root_stride", u64), ("root_offset", u64), ("collect_counters", u32),
                ("heavy_threshold", u32), ("no_hub_bitmaps", u32), ("root_max_degree", u32), ("pin_tables", u32)]


class PlanTuning(C.Structure):
    """Per-plan execution choices (sge_plan_set_tuning); zero = automatic."""
    _fields_ = [("heavy_threshold", u32), ("level3_parts", u32), ("no_hub_bitmaps", u32)]


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("total_ms", C.c_double), ("root_tasks", u64), ("set_ops", u64),
                ("alg_bytes", u64), ("partial_matches", u64), ("gpu_launches", u32), ("status_flags", u32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class GraphStats(C.Structure):
    _fields_ = [("num_vertices", C.c_double), ("num_directed_edges", C.c_double),
                ("moments", C.c_double * (SGE_MAX_K + 2)), ("clustering", C.c_double), ("max_degree", C.c_double)]


class Trie(C.Structure):
    _fields_ = [("arity", u32), ("level_len", u64 * 16), ("values", C.c_void_p * 16), ("child", C.c_void_p * 16)]


class GraphInfo(C.Structure):
    _fields_ = [("num_vertices", u32), ("num_directed_edges", u64), ("max_degree", u32), ("device_bytes", u64),
                ("hub_count", u32), ("hub_min_degree", u32)]


_lib = None

# C-ABI symbols and their signatures (restype, argtypes).
_P = C.POINTER
SIGNATURES = {
    "sge_struct_size": (C.c_size_t, [C.c_int]),
    "sge_last_error": (C.c_char_p, []),
    "sge_version": (C.c_char_p, []),
    "sge_device_count": (C.c_int, []),
    "sge_load_graph_file": (C.c_int, [C.c_char_p, _P(_P(u32)), _P(_P(u32)), _P(u32), _P(u64)]),
    "sge_save_graph_binary": (C.c_int, [C.c_char_p, _P(u32), _P(u32), u32]),
    "sge_load_pattern_file": (C.c_int, [C.c_char_p, _P(u32), _P(u32), _P(u32)]),
    "sge_csr_from_edges": (C.c_int, [_P(u32), u64, u32, C.c_int, _P(_P(u32)), _P(_P(u32)), _P(u64)]),
    "sge_free_host": (None, [C.c_void_p]),
    "sge_gen_rmat": (C.c_int, [u32, u64, u32, u32, u32, u64, _P(_P(u32)), _P(u64)]),
    "sge_gen_chung_lu": (C.c_int, [u32, u64, u32, u32, u64, _P(_P(u32)), _P(u64)]),
    "sge_gen_pattern": (C.c_int, [u32, u32, u64, _P(u32)]),
    "sge_plan_pattern": (C.c_int, [u32, u32, _P(u32), C.c_void_p, _P(PlanOpts), _P(PlanBlob)]),
    "sge_pattern_info": (C.c_int, [u32, u32, _P(u32), _P(u64), _P(u32)]),
    "sge_plan_validate": (C.c_int, [_P(PlanBlob)]),
    "sge_plan_from_order_text": (C.c_int, [u32, u32, _P(u32), C.c_char_p, _P(GraphStats), _P(PlanOpts),
                                           _P(PlanBlob), _P(u32)]),
    "sge_graph_stats_compute": (C.c_int, [_P(u32), _P(u32), u32, _P(GraphStats)]),
    "sge_plan_pattern_stats": (C.c_int, [u32, u32, _P(u32), _P(GraphStats), _P(PlanOpts), _P(PlanBlob)]),
    "sge_graph_create": (C.c_int, [_P(u32), _P(u32), u32, u64, C.c_int, _P(C.c_void_p)]),
    "sge_graph_destroy": (C.c_int, [C.c_void_p]),
    "sge_graph_get_info": (C.c_int, [C.c_void_p, _P(GraphInfo)]),
    "sge_graph_create_from_device_edges": (C.c_int, [C.c_void_p, u64, u32, C.c_int, _P(C.c_void_p)]),
    "sge_graph_create_rmat": (C.c_int, [u32, u64, u32, u32, u32, u64, C.c_int, _P(C.c_void_p)]),
    "sge_plan_pattern_sampled": (C.c_int, [u32, u32, _P(u32), C.c_void_p, _P(PlanOpts), u32, u64, _P(PlanBlob),
                                           _P(C.c_double)]),
    "sge_graph_copy_csr": (C.c_int, [C.c_void_p, _P(u32), _P(u32)]),
    "sge_plan_create": (C.c_int, [_P(PlanBlob), _P(C.c_void_p)]),
    "sge_plan_destroy": (C.c_int, [C.c_void_p]),
    "sge_plan_set_tuning": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sge_count": (C.c_int, [C.c_void_p, _P(C.c_void_p), u32, _P(CountOpts), _P(u64), _P(u64), _P(Stats)]),
    "sge_count_plan_times": (C.c_int, [C.c_void_p, _P(C.c_void_p), u32, _P(CountOpts), _P(u64), _P(C.c_double),
                                       _P(Stats)]),
    "sge_count_host": (C.c_int, [_P(u32), _P(u32), u32, u64, _P(PlanBlob), u32, _P(CountOpts), _P(u64), _P(Stats)]),
    "sge_plan_candidates": (C.c_int, [u32, u32, _P(u32), _P(GraphStats), _P(PlanOpts), _P(PlanBlob), u32, _P(u32)]),
    "sge_plan_features": (C.c_int, [_P(PlanBlob), _P(GraphStats), _P(C.c_float)]),
    "sge_mlp_create": (C.c_int, [u32, u32, u64, C.c_int, _P(C.c_void_p)]),
    "sge_mlp_destroy": (C.c_int, [C.c_void_p]),
    "sge_mlp_num_params": (C.c_int, [C.c_void_p, _P(C.c_size_t)]),
    "sge_mlp_get_params": (C.c_int, [C.c_void_p, _P(C.c_float)]),
    "sge_mlp_set_params": (C.c_int, [C.c_void_p, _P(C.c_float)]),
    "sge_mlp_forward": (C.c_int, [C.c_void_p, _P(C.c_float), u32, _P(C.c_float)]),
    "sge_mlp_forward_bf16": (C.c_int, [C.c_void_p, _P(C.c_float), u32, _P(C.c_float)]),
    "sge_mlp_loss_grad": (C.c_int, [C.c_void_p, _P(C.c_float), _P(C.c_float), u32, _P(C.c_float), _P(C.c_float)]),
    "sge_mlp_train": (C.c_int, [C.c_void_p, _P(C.c_float), _P(C.c_float), u32, u32, u32, C.c_float, u64,
                                _P(C.c_float)]),
    "sge_plan_pattern_learned": (C.c_int, [u32, u32, _P(u32), _P(GraphStats), _P(PlanOpts), C.c_void_p, u32,
                                           _P(PlanBlob)]),
    "sge_batch_create": (C.c_int, [C.c_void_p, _P(C.c_void_p), u32, _P(CountOpts), _P(C.c_void_p)]),
    "sge_batch_run": (C.c_int, [C.c_void_p, _P(u64), _P(u64), _P(Stats)]),
    "sge_batch_destroy": (C.c_int, [C.c_void_p]),
    "sge_enumerate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, u64, _P(u64)]),
    "sge_pattern_automorphisms": (C.c_int, [u32, u32, _P(u32), _P(C.c_uint8), u32, _P(u32)]),
    "sge_canonicalize": (C.c_int, [C.c_void_p, u64, u32, _P(C.c_uint8), u32]),
    "sge_sort_tuples": (C.c_int, [C.c_void_p, u64, u32]),
    "sge_trie_build": (C.c_int, [C.c_void_p, u64, u32, _P(Trie)]),
    "sge_trie_free": (C.c_int, [_P(Trie)]),
    "sge_trie_copy_level": (C.c_int, [_P(Trie), u32, _P(u32), _P(u64)]),
    "sge_match_set": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, _P(u32), _P(u32), u64, _P(u64)]),
    "sge_count_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, u32, u64, u32, _P(PlanBlob), u32, C.c_void_p,
                                    C.c_void_p]),
    "sge_bags_create": (C.c_int, [C.c_void_p, u32, u32, _P(u32), C.c_char_p, u64, _P(C.c_void_p)]),
    "sge_load_labeled_graph_file": (C.c_int, [C.c_char_p, _P(_P(u32)), _P(_P(u32)), _P(_P(u32)), _P(u32), _P(u64)]),
    "sge_graph_set_labels": (C.c_int, [C.c_void_p, _P(u32)]),
    "sge_plan_set_labels": (C.c_int, [C.c_void_p, _P(u32)]),
    "sge_bags_info": (C.c_int, [C.c_void_p, _P(u32), _P(u64), _P(u64), _P(u32), _P(u32)]),
    "sge_bags_destroy": (C.c_int, [C.c_void_p]),
    "sge_plan_use_bags": (C.c_int, [C.c_void_p, C.c_void_p, _P(u32)]),
}


def lib() -> C.CDLL:
    """Loads libsge.so (built by sge_build.build_sge); raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise SgeError(6, f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(st: int) -> None:
    if st != 0:
        raise SgeError(st, lib().sge_last_error().decode(errors="replace"))


def _u32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(u32))


def _take_u32(ptr, n: int) -> np.ndarray:
    out = np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].copy() if n else np.zeros(0, np.uint32)
    lib().sge_free_host(C.cast(ptr, C.c_void_p))
    return out


# ---------------------------------------------------------------- graphs ----
@dataclass
class DataGraph:
    """Symmetric CSR with sorted neighbour lists (relation/graph.h:113-213)."""
    offsets: np.ndarray
    nbrs: np.ndarray

    @property
    def num_vertices(self) -> int:
        return int(self.offsets.shape[0] - 1)

    @property
    def num_edges(self) -> int:
        return int(self.nbrs.shape[0] // 2)

    @property
    def max_degree(self) -> int:
        return int(np.diff(self.offsets).max()) if self.num_vertices else 0

    @classmethod
    def load(cls, path: str | os.PathLike) -> "DataGraph":
        off, nb = C.POINTER(u32)(), C.POINTER(u32)()
        n, nnz = u32(), u64()
        _check(lib().sge_load_graph_file(str(path).encode(), C.byref(off), C.byref(nb), C.byref(n), C.byref(nnz)))
        return cls(_take_u32(off, n.value + 1), _take_u32(nb, nnz.value))

    @classmethod
    def load_labeled(cls, path: str | os.PathLike) -> "tuple[DataGraph, np.ndarray]":
        """A labeled graph in the reference's "t / v id label degree / e u v"
        text format (sge_load_labeled_graph_file): the graph and its labels."""
        off, nb, lab = C.POINTER(u32)(), C.POINTER(u32)(), C.POINTER(u32)()
        n, nnz = u32(), u64()
        _check(lib().sge_load_labeled_graph_file(str(path).encode(), C.byref(off), C.byref(nb), C.byref(lab),
                                                 C.byref(n), C.byref(nnz)))
        g = cls(_take_u32(off, n.value + 1), _take_u32(nb, nnz.value))
        return g, _take_u32(lab, n.value)

    def save_labeled_text(self, path: str | os.PathLike, labels) -> None:
        """The reference's labeled text format (t / v / e lines)."""
        deg = np.diff(self.offsets)
        src = np.repeat(np.arange(self.num_vertices, dtype=np.uint32), deg)
        keep = src < self.nbrs
        with open(path, "w") as f:
            f.write(f"t {self.num_vertices} {int(keep.sum())}\n")
            for v in range(self.num_vertices):
                f.write(f"v {v} {int(labels[v])} {int(deg[v])}\n")
            for a, b in zip(src[keep].tolist(), self.nbrs[keep].tolist()):
                f.write(f"e {a} {b}\n")

    @classmethod
    def from_edges(cls, edges: np.ndarray, num_vertices: int, dedup: bool = True) -> "DataGraph":
        e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1)
        off, nb = C.POINTER(u32)(), C.POINTER(u32)()
        nnz = u64()
        _check(lib().sge_csr_from_edges(_u32p(e), e.size // 2, num_vertices, int(dedup), C.byref(off), C.byref(nb),
                                        C.byref(nnz)))
        return cls(_take_u32(off, num_vertices + 1), _take_u32(nb, nnz.value))

    def save_binary(self, path: str | os.PathLike) -> None:
        _check(lib().sge_save_graph_binary(str(path).encode(), _u32p(self.offsets), _u32p(self.nbrs),
                                           self.num_vertices))

    def save_text(self, path: str | os.PathLike) -> None:
        src = np.repeat(np.arange(self.num_vertices, dtype=np.uint32), np.diff(self.offsets))
        keep = src < self.nbrs
        with open(path, "w") as f:
            f.write(f"{self.num_vertices} {int(keep.sum())}\n")
            np.savetxt(f, np.stack([src[keep], self.nbrs[keep]], 1), fmt="%d")

    def stats(self) -> GraphStats:
        """Planner statistics (degree moments, sampled clustering) on the host."""
        st = GraphStats()
        _check(lib().sge_graph_stats_compute(_u32p(np.ascontiguousarray(self.offsets, np.uint32)),
                                             _u32p(np.ascontiguousarray(self.nbrs, np.uint32)),
                                             self.num_vertices, C.byref(st)))
        return st

    def edge_array(self) -> np.ndarray:
        src = np.repeat(np.arange(self.num_vertices, dtype=np.uint32), np.diff(self.offsets))
        keep = src < self.nbrs
        return np.stack([src[keep], self.nbrs[keep]], 1)

    def fingerprint(self) -> str:
        import hashlib
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.offsets, np.uint32).tobytes())
        h.update(np.ascontiguousarray(self.nbrs, np.uint32).tobytes())
        return h.hexdigest()[:16]


@dataclass
class PatternGraph:
    """Unlabeled query pattern (relation/graph.h PatternGraph)."""
    k: int
    edges: np.ndarray  # (m, 2) uint32

    @property
    def m(self) -> int:
        return int(self.edges.shape[0])

    @classmethod
    def load(cls, path: str | os.PathLike) -> "PatternGraph":
        k, m = u32(), u32()
        buf = (u32 * (2 * SGE_MAX_K * SGE_MAX_K))()
        _check(lib().sge_load_pattern_file(str(path).encode(), C.byref(k), C.byref(m), buf))
        return cls(k.value, np.array(buf[: 2 * m.value], dtype=np.uint32).reshape(-1, 2))

    @classmethod
    def from_edges(cls, k: int, edges) -> "PatternGraph":
        return cls(int(k), np.asarray(edges, dtype=np.uint32).reshape(-1, 2))

    @classmethod
    def random(cls, k: int, m: int, seed: int) -> "PatternGraph":
        buf = (u32 * (2 * m))()
        _check(lib().sge_gen_pattern(k, m, seed, buf))
        return cls(k, np.array(buf[:], dtype=np.uint32).reshape(-1, 2))

    def flat(self) -> np.ndarray:
        return np.ascontiguousarray(self.edges, dtype=np.uint32).reshape(-1)

    def info(self) -> tuple[int, bool]:
        """(|Aut|, single_bag)"""
        a, s = u64(), u32()
        e = self.flat()
        _check(lib().sge_pattern_info(self.k, self.m, _u32p(e), C.byref(a), C.byref(s)))
        return int(a.value), bool(s.value)

    def text(self) -> str:
        return f"{self.k} {self.m}\n" + "".join(f"{a} {b}\n" for a, b in self.edges)


# ------------------------------------------------------------ generators ----
def gen_rmat(scale: int, m: int, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 0) -> DataGraph:
    ep, mo = C.POINTER(u32)(), u64()
    _check(lib().sge_gen_rmat(scale, m, round(a * 1e6), round(b * 1e6), round(c * 1e6), seed, C.byref(ep),
                              C.byref(mo)))
    e = _take_u32(ep, 2 * mo.value)
    return DataGraph.from_edges(e, 1 << scale, dedup=False)


def gen_chung_lu(n: int, m: int, gamma: float, max_deg: int = 0, seed: int = 0) -> DataGraph:
    ep, mo = C.POINTER(u32)(), u64()
    _check(lib().sge_gen_chung_lu(n, m, round(gamma * 1000), max_deg, seed, C.byref(ep), C.byref(mo)))
    e = _take_u32(ep, 2 * mo.value)
    return DataGraph.from_edges(e, n, dedup=False)


# --------------------------------------------------------------- planner ----
def _fix(o: "PlanOpts", symmetry_seq, root_edge, labels=None) -> list:
    keep = []
    if labels is not None:
        keep.append(np.ascontiguousarray(labels, dtype=np.uint32))
        o.vertex_labels = _u32p(keep[-1])
    if symmetry_seq is not None:
        keep.append(np.ascontiguousarray(symmetry_seq, dtype=np.uint32))
        o.symmetry_seq = _u32p(keep[-1])
    if root_edge is not None:
        keep.append(np.ascontiguousarray(root_edge, dtype=np.uint32))
        o.root_edge = _u32p(keep[-1])
    return keep


def plan(pattern: PatternGraph, graph: "Engine | GraphStats | DataGraph | None" = None, iep: bool = True,
         exploration: bool = False, max_tail: int = SGE_MAX_TAIL, force_order=None, seed: int = 1,
         symmetry_seq=None, root_edge=None, labels=None) -> PlanBlob:
    """Plans a pattern (the host planning half of graph_mining_system).  The
    cost model reads the graph's statistics: pass the Engine, a DataGraph, or
    precomputed GraphStats (None = a generic sparse graph).  symmetry_seq and
    root_edge fix the symmetry restrictions and the root pattern edge of every
    candidate, so plans agree on any root sample.  labels (k values) plans
    labeled matching: count with the same labels (Engine.count(labels=...))
    on a graph with vertex labels (Engine.set_labels)."""
    o = PlanOpts(JOIN_EXPLORATION if exploration else JOIN_WCOJ, int(iep), max_tail, seed, None)
    keep = _fix(o, symmetry_seq, root_edge, labels)
    if force_order is not None:
        keep.append(np.ascontiguousarray(force_order, dtype=np.uint32))
        o.force_order = _u32p(keep[-1])
    b = PlanBlob()
    e = pattern.flat()
    if isinstance(graph, DataGraph):
        graph = graph.stats()
    if isinstance(graph, GraphStats):
        _check(lib().sge_plan_pattern_stats(pattern.k, pattern.m, _u32p(e), C.byref(graph), C.byref(o), C.byref(b)))
    else:
        _check(lib().sge_plan_pattern(pattern.k, pattern.m, _u32p(e), graph._h if graph else None, C.byref(o),
                                      C.byref(b)))
    return b


def plan_from_reference(pattern: PatternGraph, text: str, graph: "Engine | GraphStats | DataGraph | None" = None,
                        iep: bool = True, exploration: bool = False) -> tuple[PlanBlob, int]:
    """Imports the reference's own plan (sge_plan_from_order_text): the bag
    orders HyperTree::writeToStream prints ("num bags: N" + one order per bag,
    global bag last), a whole reference log holding them, or an order file.
    Returns (plan, number of bags)."""
    o = PlanOpts(JOIN_EXPLORATION if exploration else JOIN_WCOJ, int(iep), SGE_MAX_TAIL, 1, None)
    if isinstance(graph, Engine):
        graph = graph.graph
    if isinstance(graph, DataGraph):
        graph = graph.stats()
    b = PlanBlob()
    nb = u32()
    e = pattern.flat()
    _check(lib().sge_plan_from_order_text(pattern.k, pattern.m, _u32p(e), text.encode(),
                                          C.byref(graph) if graph is not None else None, C.byref(o), C.byref(b),
                                          C.byref(nb)))
    return b, nb.value


def plan_sampled(pattern: PatternGraph, engine: "Engine", iep: bool = True, exploration: bool = False,
                 max_tail: int = SGE_MAX_TAIL, shortlist: int = 8, sample_stride: int = 64,
                 seed: int = 1) -> tuple[PlanBlob, list[float]]:
    """Plans with GPU root sampling (sge_plan_pattern_sampled): the cost
    model's best `shortlist` candidates count the roots t ≡ 0 (mod
    sample_stride) and the fastest wins.  Returns (plan, per-candidate
    sample times in ms, -1 for candidates past the budget or absent)."""
    o = PlanOpts(JOIN_EXPLORATION if exploration else JOIN_WCOJ, int(iep), max_tail, seed, None)
    b = PlanBlob()
    e = pattern.flat()
    ms = (C.c_double * shortlist)()
    _check(lib().sge_plan_pattern_sampled(pattern.k, pattern.m, _u32p(e), engine._h, C.byref(o), shortlist,
                                          sample_stride, C.byref(b), ms))
    return b, list(ms)


SGE_FEATURES = 64


def _plan_opts(iep: bool, exploration: bool, max_tail: int, seed: int) -> PlanOpts:
    return PlanOpts(JOIN_EXPLORATION if exploration else JOIN_WCOJ, int(iep), max_tail, seed, None)


def candidates(pattern: PatternGraph, stats: "GraphStats | None", iep: bool = True, exploration: bool = False,
               cap: int = 64, max_tail: int = SGE_MAX_TAIL, symmetry_seq=None, root_edge=None,
               force_order=None, labels=None) -> list[PlanBlob]:
    """Every executable plan of the pattern, cheapest first by the cost model
    (symmetry_seq / root_edge as in plan(); force_order: only that matching
    order, with every tail length and restriction scheme)."""
    arr = (PlanBlob * cap)()
    n = u32()
    e = pattern.flat()
    o = _plan_opts(iep, exploration, max_tail, 1)
    keep = _fix(o, symmetry_seq, root_edge, labels)  # (kept alive for the call)
    if force_order is not None:
        keep.append(np.ascontiguousarray(force_order, dtype=np.uint32))
        o.force_order = _u32p(keep[-1])
    _check(lib().sge_plan_candidates(pattern.k, pattern.m, _u32p(e), C.byref(stats) if stats is not None else None,
                                     C.byref(o), arr, cap, C.byref(n)))
    return [PlanBlob.from_buffer_copy(arr[i]) for i in range(n.value)]


def features(blob: PlanBlob, stats: "GraphStats | None") -> np.ndarray:
    out = np.zeros(SGE_FEATURES, np.float32)
    _check(lib().sge_plan_features(C.byref(blob), C.byref(stats) if stats is not None else None,
                                   out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MLP:
    """The learned plan scorer (sge_mlp): FP32 training and BF16 inference on the GPU."""

    def __init__(self, in_dim: int = SGE_FEATURES, hidden: int = 128, seed: int = 0, device: int = 0):
        h = C.c_void_p()
        _check(lib().sge_mlp_create(in_dim, hidden, seed, device, C.byref(h)))
        self._h = h
        self.in_dim, self.hidden = in_dim, hidden

    @property
    def num_params(self) -> int:
        n = C.c_size_t()
        _check(lib().sge_mlp_num_params(self._h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        _check(lib().sge_mlp_get_params(self._h, _fp(out)))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        _check(lib().sge_mlp_set_params(self._h, _fp(p)))

    def forward(self, x: np.ndarray, bf16: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(x.shape[0], np.float32)
        fn = lib().sge_mlp_forward_bf16 if bf16 else lib().sge_mlp_forward
        _check(fn(self._h, _fp(x), x.shape[0], _fp(y)))
        return y

    def loss_grad(self, x: np.ndarray, t: np.ndarray) -> tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float()
        g = np.zeros(self.num_params, np.float32)
        _check(lib().sge_mlp_loss_grad(self._h, _fp(x), _fp(t), x.shape[0], C.byref(loss), _fp(g)))
        return float(loss.value), g

    def train(self, x: np.ndarray, t: np.ndarray, epochs: int = 200, batch: int = 256, lr: float = 1e-3,
              seed: int = 0) -> float:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float()
        _check(lib().sge_mlp_train(self._h, _fp(x), _fp(t), x.shape[0], epochs, batch, lr, seed, C.byref(loss)))
        return float(loss.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sge_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_learned(pattern: PatternGraph, stats: "GraphStats", scorer: MLP, iep: bool = True,
                 exploration: bool = False, shortlist: int = 64) -> PlanBlob:
    """Plans with the learned scorer (cost-model shortlist, MLP picks)."""
    b = PlanBlob()
    e = pattern.flat()
    o = _plan_opts(iep, exploration, SGE_MAX_TAIL, 1)
    _check(lib().sge_plan_pattern_learned(pattern.k, pattern.m, _u32p(e), C.byref(stats), C.byref(o), scorer._h,
                                          shortlist, C.byref(b)))
    return b


def validate_plan(b: PlanBlob) -> None:
    _check(lib().sge_plan_validate(C.byref(b)))


# ---------------------------------------------------------------- engine ----
class Engine:
    """A device-resident data graph (sge_graph) plus batched counting."""

    def __init__(self, graph: DataGraph, device: int = 0):
        self.graph = graph
        self._off = np.ascontiguousarray(graph.offsets, np.uint32)
        self._nb = np.ascontiguousarray(graph.nbrs, np.uint32)
        h = C.c_void_p()
        _check(lib().sge_graph_create(_u32p(self._off), _u32p(self._nb), graph.num_vertices, self._nb.size, device,
                                      C.byref(h)))
        self._h = h

    @classmethod
    def _adopt(cls, h: C.c_void_p) -> "Engine":
        eng = cls.__new__(cls)
        eng._h = h
        off, nb = eng.csr()
        eng.graph = DataGraph(off, nb)
        eng._off, eng._nb = eng.graph.offsets, eng.graph.nbrs
        return eng

    @classmethod
    def rmat_device(cls, scale: int, m: int, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 0,
                    device: int = 0) -> "Engine":
        """R-MAT generated and turned into a CSR on the GPU
        (sge_graph_create_rmat): the same graph as gen_rmat(scale, m, a, b, c, seed)."""
        h = C.c_void_p()
        _check(lib().sge_graph_create_rmat(scale, m, round(a * 1e6), round(b * 1e6), round(c * 1e6), seed, device,
                                           C.byref(h)))
        return cls._adopt(h)

    @classmethod
    def from_device_edges(cls, ptr: int, m: int, num_vertices: int, device: int = 0) -> "Engine":
        """CSR built on the GPU from m undirected (u, v) pairs at device address
        ptr (sge_graph_create_from_device_edges; self-loops and repeats dropped)."""
        h = C.c_void_p()
        _check(lib().sge_graph_create_from_device_edges(C.c_void_p(ptr), m, num_vertices, device, C.byref(h)))
        return cls._adopt(h)

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        """The device CSR copied to host (offsets, neighbours)."""
        gi = self.info()
        off = np.zeros(gi["num_vertices"] + 1, np.uint32)
        nb = np.zeros(max(gi["num_directed_edges"], 1), np.uint32)
        _check(lib().sge_graph_copy_csr(self._h, _u32p(off), _u32p(nb)))
        return off, nb[: gi["num_directed_edges"]]

    def info(self) -> dict:
        gi = GraphInfo()
        _check(lib().sge_graph_get_info(self._h, C.byref(gi)))
        return {f: getattr(gi, f) for f, _ in gi._fields_}

    def count(self, plans: list[PlanBlob], stats: bool = False, time_budget_s: float = 0.0,
              max_level_capacity: int = 0, blocks_per_sm: int = 0, warps_per_block: int = 0, chunk: int = 0,
              root_stride: int = 1, root_offset: int = 0, heavy_threshold: int = 0, hub_bitmaps: bool = True,
              root_max_degree: int = 0, pin_tables: int = 0, tuning: "list[PlanTuning | None] | None" = None,
              plan_times: bool = False, bags: "list[Bags | None] | None" = None, labels=None):
        """Counts every plan over the graph in one launch.  Returns (counts,
        instances, stats-dict); counts are the reference's "Number of matches"
        (uint64).  stats=True runs the instrumented kernel (set operations,
        algorithmic bytes); kernel_ms is reported either way.
        root_stride/root_offset restrict the run to root tasks
        t ≡ root_offset (mod root_stride) (sharding, sampling).  heavy_threshold
        (0 = auto) splits roots whose level-2 list may exceed it into tasks of
        a second launch.  hub_bitmaps=False probes every adjacency list by
        binary search (comparison runs).  root_max_degree > 0 keeps only the
        sampled roots whose endpoints both have at most that degree.
        pin_tables: 0 automatic, 1 no per-warp shared-memory tables, 2 hashed
        tables on large graphs (sge_count_opts.pin_tables); tuning
        gives each plan its PlanTuning (None = automatic).  plan_times=True
        also returns stats["plan_busy_ms"]: per plan, the warp-milliseconds
        its roots took (sge_count_plan_times; instances are then not read).
        bags gives each plan the bag relations its tail levels read
        (sge_plan_use_bags; None = intersect adjacency lists);
        stats["bag_levels"] then lists, per plan, the tail levels that did.
        labels gives each labeled plan its k pattern labels (sge_plan_set_labels;
        the graph's come from set_labels)."""
        handles = []
        bag_levels = []
        try:
            for i, b in enumerate(plans):
                ph = C.c_void_p()
                _check(lib().sge_plan_create(C.byref(b), C.byref(ph)))
                handles.append(ph)
                if tuning is not None and tuning[i] is not None:
                    _check(lib().sge_plan_set_tuning(ph, C.byref(tuning[i])))
                if labels is not None and labels[i] is not None:
                    la = np.ascontiguousarray(labels[i], np.uint32)
                    _check(lib().sge_plan_set_labels(ph, _u32p(la)))
                if bags is not None and bags[i] is not None:
                    lv = u32()
                    _check(lib().sge_plan_use_bags(ph, bags[i]._h, C.byref(lv)))
                    bag_levels.append(lv.value)
                else:
                    bag_levels.append(0)
            arr = (C.c_void_p * len(handles))(*[h.value for h in handles])
            counts = (u64 * len(plans))()
            inst = (u64 * len(plans))()
            st = Stats()
            o = CountOpts(blocks_per_sm, warps_per_block, chunk, time_budget_s, max_level_capacity, root_stride,
                          root_offset, int(stats), heavy_threshold, int(not hub_bitmaps), root_max_degree,
                          int(pin_tables))
            if plan_times:
                busy = (C.c_double * len(plans))()
                _check(lib().sge_count_plan_times(self._h, arr, len(plans), C.byref(o), counts, busy, C.byref(st)))
                d = st.as_dict()
                d["plan_busy_ms"] = list(busy)
                return list(counts), [], d
            _check(lib().sge_count(self._h, arr, len(plans), C.byref(o), counts, inst, C.byref(st)))
            d = st.as_dict()
            if bags is not None:
                d["bag_levels"] = bag_levels
            return list(counts), list(inst), d
        finally:
            for h in handles:
                lib().sge_plan_destroy(h)

    def set_labels(self, labels) -> None:
        """One label per data vertex (sge_graph_set_labels); None removes them."""
        if labels is None:
            _check(lib().sge_graph_set_labels(self._h, None))
            return
        la = np.ascontiguousarray(labels, np.uint32)
        if la.size != self.info()["num_vertices"]:
            raise SgeError(1, f"{la.size} labels for {self.info()['num_vertices']} vertices")
        _check(lib().sge_graph_set_labels(self._h, _u32p(la)))

    def bags(self, pattern: PatternGraph, text: str, max_rows: int = 0) -> "Bags":
        """Bag relations of the decomposition in `text` on this graph
        (sge_bags_create): each bag with one attribute of its own and 3 or 4
        attributes, as a trie.  A bag with more than max_rows tuples (0 = no
        limit) is skipped."""
        return Bags(self, pattern, text, max_rows)

    def match_set(self, pattern: PatternGraph, exploration: bool = False, max_rows: int = 1 << 26) -> np.ndarray:
        """Sorted instance set: one row per instance (canonical image under the
        automorphisms), pattern-vertex order."""
        b = plan(pattern, self, iep=False, exploration=exploration)
        ph = C.c_void_p()
        _check(lib().sge_plan_create(C.byref(b), C.byref(ph)))
        try:
            n = u64()
            e = pattern.flat()
            # size from the count first
            _, inst, _ = self.count([b])
            rows = int(inst[0])
            if rows > max_rows:
                raise SgeError(2, f"{rows} instances exceed max_rows={max_rows}")
            out = np.zeros(max(rows, 1) * pattern.k, np.uint32)
            _check(lib().sge_match_set(self._h, ph, pattern.k, pattern.m, _u32p(e), _u32p(out), rows, C.byref(n)))
            return out[: n.value * pattern.k].reshape(n.value, pattern.k)
        finally:
            lib().sge_plan_destroy(ph)

    def batch(self, plans: list[PlanBlob], stats: bool = False, **opts) -> "Batch":
        """A batch captured into a CUDA graph (replay with Batch.run)."""
        return Batch(self, plans, stats, **opts)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sge_graph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Bags:
    """sge_bags: bag relations (tries) of a decomposition on one graph."""

    def __init__(self, engine: Engine, pattern: PatternGraph, text: str, max_rows: int = 0):
        self.engine = engine  # the relations belong to this graph: keep it alive
        h = C.c_void_p()
        e = pattern.flat()
        _check(lib().sge_bags_create(engine._h, pattern.k, pattern.m, _u32p(e), text.encode(), max_rows,
                                     C.byref(h)))
        self._h = h

    def info(self) -> dict:
        n, rows, nbytes, skipped = u32(), u64(), u64(), u32()
        own = (u32 * 16)()
        _check(lib().sge_bags_info(self._h, C.byref(n), C.byref(rows), C.byref(nbytes), own, C.byref(skipped)))
        return {"relations": n.value, "rows": rows.value, "device_bytes": nbytes.value,
                "own_vertices": list(own)[: n.value], "skipped": skipped.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sge_bags_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """sge_batch: plans uploaded once, launch sequence captured into a CUDA graph."""

    def __init__(self, engine: Engine, plans: list[PlanBlob], stats: bool = False, time_budget_s: float = 0.0,
                 blocks_per_sm: int = 0, warps_per_block: int = 0, chunk: int = 0, root_stride: int = 1,
                 root_offset: int = 0, heavy_threshold: int = 0, hub_bitmaps: bool = True,
                 root_max_degree: int = 0, max_level_capacity: int = 0, pin_tables: int = 0,
                 tuning: "list[PlanTuning | None] | None" = None):
        self.engine = engine
        self.n = len(plans)
        self._ph = []
        for i, b in enumerate(plans):
            ph = C.c_void_p()
            _check(lib().sge_plan_create(C.byref(b), C.byref(ph)))
            self._ph.append(ph)
            if tuning is not None and tuning[i] is not None:
                _check(lib().sge_plan_set_tuning(ph, C.byref(tuning[i])))
        arr = (C.c_void_p * self.n)(*[h.value for h in self._ph])
        o = CountOpts(blocks_per_sm, warps_per_block, chunk, time_budget_s, max_level_capacity, root_stride,
                      root_offset, int(stats), heavy_threshold, int(not hub_bitmaps), root_max_degree,
                      int(pin_tables))
        h = C.c_void_p()
        try:
            _check(lib().sge_batch_create(engine._h, arr, self.n, C.byref(o), C.byref(h)))
        except SgeError:
            self._free_plans()
            raise
        self._h = h

    def run(self):
        counts = (u64 * self.n)()
        inst = (u64 * self.n)()
        st = Stats()
        _check(lib().sge_batch_run(self._h, counts, inst, C.byref(st)))
        return list(counts), list(inst), st.as_dict()

    def _free_plans(self):
        for h in self._ph:
            lib().sge_plan_destroy(h)
        self._ph = []

    def close(self):
        if getattr(self, "_h", None):
            lib().sge_batch_destroy(self._h)
            self._h = None
        self._free_plans()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort_tuples_device(ptr: int, n: int, arity: int) -> None:
    """Lexicographic LSD radix sort of n device rows (uint32 × arity) in place."""
    _check(lib().sge_sort_tuples(C.c_void_p(ptr), n, arity))


def trie_build_device(ptr: int, n: int, arity: int) -> Trie:
    t = Trie()
    _check(lib().sge_trie_build(C.c_void_p(ptr), n, arity, C.byref(t)))
    return t


def trie_level(t: Trie, level: int) -> tuple[np.ndarray, np.ndarray | None]:
    n = int(t.level_len[level])
    vals = np.zeros(max(n, 1), np.uint32)
    child = np.zeros(n + 1, np.uint64) if level + 1 < t.arity else None
    _check(lib().sge_trie_copy_level(C.byref(t), level, _u32p(vals),
                                     child.ctypes.data_as(C.POINTER(u64)) if child is not None else None))
    return vals[:n], child


def trie_free(t: Trie) -> None:
    lib().sge_trie_free(C.byref(t))


def count_host(graph: DataGraph, plans: list[PlanBlob], stats: bool = False, root_stride: int = 1,
               root_offset: int = 0, root_max_degree: int = 0):
    """End-to-end call through sge_count_host: host CSR in, counts out
    (root_stride/root_offset: the sampled root edges, as in Engine.count)."""
    arr = (PlanBlob * len(plans))(*plans)
    counts = (u64 * len(plans))()
    st = Stats()
    off = np.ascontiguousarray(graph.offsets, np.uint32)
    nb = np.ascontiguousarray(graph.nbrs, np.uint32)
    o = CountOpts(0, 0, 0, 0.0, 0, root_stride, root_offset, int(stats), 0, 0, root_max_degree)
    _check(lib().sge_count_host(_u32p(off), _u32p(nb), graph.num_vertices, nb.size, arr, len(plans), C.byref(o),
                                counts, C.byref(st)))
    return list(counts), st.as_dict()


def match(query_path, data_path, iep: bool = False, exploration: bool = False, device: int = 0) -> dict:
    """singleThreadMatch / parallelMatch (main.cpp:12-218) on the GPU: load,
    plan, count.  Returns the log fields as a dict."""
    import time
    q = PatternGraph.load(query_path)
    g = DataGraph.load(data_path)
    with Engine(g, device) as eng:
        t0 = time.perf_counter()
        b = plan(q, eng, iep=iep, exploration=exploration)
        t1 = time.perf_counter()
        counts, inst, st = eng.count([b], stats=True)
        t2 = time.perf_counter()
    return {"Number of matches": counts[0], "Number of instances": inst[0], "Planning time (s)": t1 - t0,
            "Execution Time": t2 - t1, "Number of intersections": st["set_ops"], "plan": b.summary()}
