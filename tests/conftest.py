"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
a CPU-only host.  The libraries are built in-tree on first use."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "subgraph-enumeration_gb300"
GOLDEN = REPO / "tests" / "golden"
for p in (str(PKG), str(REPO / "oracle"), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _ensure_built():
    import sge_build
    if not (PKG / "_build" / "libsge.so").exists() or not (PKG / "_build" / "graph_mining_system").exists():
        sge_build.build_sge()
    if not (REPO / "oracle" / "_build" / "liboracle.so").exists():
        sge_build.build_oracle()


_ensure_built()


@pytest.fixture(scope="session")
def sge():
    import sge as m
    return m


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    return o


@pytest.fixture(scope="session")
def patterns():
    return json.loads((GOLDEN / "patterns.json").read_text())


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN / "golden_counts.json").read_text())


def make_golden_graph(sge, golden, name):
    spec = golden["graphs"][name]
    if spec["kind"] == "file":
        g = sge.DataGraph.load(GOLDEN / spec["path"])
    elif spec["kind"] == "chung_lu":
        g = sge.gen_chung_lu(spec["n"], spec["m"], spec["gamma"], spec["max_deg"], spec["seed"])
    else:
        g = sge.gen_rmat(spec["scale"], spec["m"], spec["a"], spec["b"], spec["c"], spec["seed"])
    assert g.fingerprint() == spec["fingerprint"], f"generator output for {name} changed"
    return g


@pytest.fixture(scope="session")
def graphs(sge, golden):
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = make_golden_graph(sge, golden, name)
        return cache[name]
    return get


def pattern_of(sge, patterns, name):
    p = patterns[name]
    return sge.PatternGraph.from_edges(p["k"], p["edges"])


def golden_rows(golden, graph=None, mode="default"):
    return [r for r in golden["results"] if (graph is None or r["graph"] == graph) and r["mode"] == mode
            and r["count"] is not None and r["rc"] == 0]


@pytest.fixture(scope="session")
def has_gpu(sge):
    return sge.lib().sge_device_count() > 0
