"""CHOOSE leaves over ranges where the reference's choosec wraps.

The reference counts r symmetric last vertices with choosec(num, r)
(utility/utils.cpp:80-94), which multiplies num(num-1)…(num-r+1) in uint64
before dividing by r!; at r = 4 the product passes 2^64 from num = 65,538.
Plans carry the choice: choose_wrap = 0 counts the exact binomial (this
library's planner), 1 reproduces the reference's arithmetic (plans imported
from the reference's planner).  Either way the wrap is reported in
status_flags bit 2.  Workload: a star whose centre has 70,000 leaves and the
pattern K_{1,5}, planned as a root edge (centre, leaf) plus a CHOOSE leaf of
the other four leaves above it."""
from math import comb

import numpy as np
import pytest

LEAVES = 70_000
MASK = (1 << 64) - 1


@pytest.fixture(scope="module")
def star(sge):
    edges = np.array([[0, i] for i in range(1, LEAVES + 1)], np.uint32)
    return sge.DataGraph.from_edges(edges, LEAVES + 1)


@pytest.fixture(scope="module")
def plan(sge, star):
    p = sge.PatternGraph.from_edges(6, [(0, 1), (0, 2), (0, 3), (0, 4), (0, 5)])
    b = sge.plan(p, star, iep=True)
    assert b.tail_mode == sge.TAIL_CHOOSE and b.tail_len == 4 and b.choose_wrap == 0
    return b


def wrapped_expectation(oracle):
    # root (centre, leaf x): the four other leaves lie above x, LEAVES - x of them
    tot = 0
    for x in range(1, LEAVES + 1):
        tot = (tot + oracle.choosec_ref(LEAVES - x, 4)) & MASK
    return tot


def with_wrap(sge, b, wrap):
    w = sge.PlanBlob.from_bytes(b.to_bytes())
    w.choose_wrap = wrap
    return w


def test_oracle_counts_exact_and_reference_arithmetic(sge, oracle, star, plan):
    exact, _ = oracle.count_plan(star.offsets, star.nbrs, plan, threads=4)
    assert exact == comb(LEAVES, 5) & MASK
    wrapped, _ = oracle.count_plan(star.offsets, star.nbrs, with_wrap(sge, plan, 1), threads=4)
    assert wrapped == wrapped_expectation(oracle)
    assert wrapped != exact


@pytest.mark.gpu
def test_gpu_choose_leaf_exact_and_wrapping(sge, oracle, star, plan):
    with sge.Engine(star) as eng:
        c, _, st = eng.count([plan])
        assert c[0] == comb(LEAVES, 5) & MASK
        assert st["status_flags"] & 4, "a falling product past 2^64 must be reported"
        c2, _, st2 = eng.count([with_wrap(sge, plan, 1)])
        assert c2[0] == wrapped_expectation(oracle)
        assert st2["status_flags"] & 4
    # below the wrap the two agree and nothing is reported
    small = sge.DataGraph.from_edges(np.array([[0, i] for i in range(1, 2001)], np.uint32), 2001)
    with sge.Engine(small) as eng:
        a, _, sa = eng.count([plan])
        bw, _, sb = eng.count([with_wrap(sge, plan, 1)])
        assert a[0] == bw[0] == comb(2000, 5)
        assert not (sa["status_flags"] & 4) and not (sb["status_flags"] & 4)
