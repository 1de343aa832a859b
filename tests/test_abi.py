"""The C-ABI library loads, exports every entry point include/sge.h declares,
and its structs have the layout the bindings assume.  No GPU needed."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parent.parent / "include" / "sge.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(sge_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(sge):
    lib = sge.lib()
    names = declared_functions()
    assert len(names) >= 24
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(sge):
    assert set(declared_functions()) <= set(sge.SIGNATURES), set(declared_functions()) - set(sge.SIGNATURES)


@pytest.mark.parametrize("which,cls", [(0, "PlanBlob"), (1, "PlanOpts"), (2, "CountOpts"), (3, "Stats"),
                                       (4, "GraphInfo"), (5, "GraphStats"), (6, "Trie"),
                                       (7, "PlanTuning")])
def test_struct_layout(sge, which, cls):
    assert sge.lib().sge_struct_size(which) == C.sizeof(getattr(sge, cls))


def test_version_and_device_count(sge):
    assert b"sm_103a" in sge.lib().sge_version()
    assert sge.lib().sge_device_count() >= 0


def test_graph_create_rejects_bad_csr_before_touching_a_device(sge):
    lib = sge.lib()
    h = C.c_void_p()
    off = np.array([0, 2, 3, 4], np.uint32)
    unsorted = np.array([2, 1, 0, 0], np.uint32)
    st = lib.sge_graph_create(sge._u32p(off), sge._u32p(unsorted), 3, 4, 0, C.byref(h))
    assert sge.STATUS[st] == "BAD_INPUT"
    asym = np.array([1, 2, 0, 1], np.uint32)  # 2 lists 1 but 1 does not list 2
    off2 = np.array([0, 2, 3, 4], np.uint32)
    st = lib.sge_graph_create(sge._u32p(off2), sge._u32p(asym), 3, 4, 0, C.byref(h))
    assert sge.STATUS[st] == "BAD_INPUT"
    loop = np.array([0, 1, 0, 1], np.uint32)
    st = lib.sge_graph_create(sge._u32p(np.array([0, 2, 4], np.uint32)), sge._u32p(loop), 2, 4, 0, C.byref(h))
    assert sge.STATUS[st] == "BAD_INPUT"
    assert b"self-loop" in lib.sge_last_error() or b"strictly" in lib.sge_last_error()


def test_no_device_is_an_error_not_a_fallback(sge):
    if sge.lib().sge_device_count() > 0:
        pytest.skip("a GPU is visible")
    g = sge.DataGraph.from_edges(np.array([[0, 1], [1, 2], [0, 2]]), 3)
    with pytest.raises(sge.SgeError) as e:
        sge.Engine(g)
    assert e.value.status_name == "NO_DEVICE"


def test_loaders_report_io_errors(sge, tmp_path):
    with pytest.raises(sge.SgeError) as e:
        sge.DataGraph.load(tmp_path / "missing.txt")
    assert e.value.status_name == "IO_ERROR"
    bad = tmp_path / "trunc.bin"
    bad.write_bytes(b"BINGRPH" + np.array([4, 10], np.uint32).tobytes() + b"\0" * 8)
    with pytest.raises(sge.SgeError) as e:
        sge.DataGraph.load(bad)
    assert e.value.status_name == "IO_ERROR"
    short = tmp_path / "short.txt"
    short.write_text("4 3\n0 1\n1 2\n")
    with pytest.raises(sge.SgeError) as e:
        sge.DataGraph.load(short)
    assert "expecting 3 edges" in str(e.value)


def test_text_and_binary_roundtrip(sge, tmp_path, graphs):
    g = graphs("ca_netscience")
    g.save_binary(tmp_path / "g.bin")
    g2 = sge.DataGraph.load(tmp_path / "g.bin")
    assert g2.fingerprint() == g.fingerprint()
    g.save_text(tmp_path / "g.txt")
    assert sge.DataGraph.load(tmp_path / "g.txt").fingerprint() == g.fingerprint()


def test_pattern_orbit_spec_relabels(sge, tmp_path):
    f = tmp_path / "p.txt"
    f.write_text("4 3\n0 1\n1 2\n2 3\n1 2\n")  # vertex orbit 2 → becomes vertex 0
    p = sge.PatternGraph.load(f)
    deg = np.bincount(p.edges.reshape(-1), minlength=4)
    assert deg[0] == 2 and p.m == 3
    f.write_text("4 3\n0 1\n1 2\n2 3\n7 1\n")
    with pytest.raises(sge.SgeError):
        sge.PatternGraph.load(f)


def test_device_ingest_checks_arguments_before_touching_a_device(sge):
    lib = sge.lib()
    h = C.c_void_p()
    # R-MAT: bad scale, a+b+c > 1, too dense for the vertex count
    assert sge.STATUS[lib.sge_graph_create_rmat(0, 10, 570000, 190000, 190000, 1, 0, C.byref(h))] == "BAD_INPUT"
    assert sge.STATUS[lib.sge_graph_create_rmat(8, 10, 600000, 300000, 200000, 1, 0, C.byref(h))] == "BAD_INPUT"
    assert sge.STATUS[lib.sge_graph_create_rmat(4, 1000, 570000, 190000, 190000, 1, 0, C.byref(h))] == "BAD_INPUT"
    # device edge list: null pointer with edges, more than 2^31 edges
    assert sge.STATUS[lib.sge_graph_create_from_device_edges(None, 5, 10, 0, C.byref(h))] == "BAD_INPUT"
    assert sge.STATUS[lib.sge_graph_create_from_device_edges(C.c_void_p(16), 1 << 31, 10, 0, C.byref(h))] == "BAD_INPUT"
    assert sge.STATUS[lib.sge_graph_copy_csr(None, None, None)] == "BAD_INPUT"
    # sampled planning needs a graph
    b = sge.PlanBlob()
    e = np.array([0, 1, 1, 2, 2, 0], np.uint32)
    assert sge.STATUS[lib.sge_plan_pattern_sampled(3, 3, sge._u32p(e), None, None, 4, 8, C.byref(b), None)] == "BAD_INPUT"


def test_device_ingest_without_a_device_is_an_error(sge):
    if sge.lib().sge_device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(sge.SgeError) as e:
        sge.Engine.rmat_device(10, 5000, seed=1)
    assert e.value.status_name == "NO_DEVICE"
    with pytest.raises(sge.SgeError) as e:
        sge.Engine.from_device_edges(0, 0, 10)
    assert e.value.status_name == "NO_DEVICE"
