"""GPU parity on the full-size R-MAT configurations, on stated root samples.

Exact counts of the dense patterns over every root edge of these graphs are
beyond any executor (see bench.py), so each test counts a fixed sample: the
undirected root edges e ≡ offset (mod stride), optionally only those whose
endpoints both have degree <= D, on the GPU through the C ABI and on the CPU
oracle (the port of the reference executor) with the same plans.  Counts
must be bit-identical.  Graphs are built on the GPU (sge_graph_create_rmat);
the oracle reads the same CSR copied back to the host.
  configuration 3: R-MAT 2^20 / 16M edges (seed 3), 16 random 6-vertex
                   patterns with 11-13 edges, one batched launch;
  configuration 4: R-MAT 2^22 / 64M edges (seed 4), the 78 random 7-vertex
                   patterns of the benchmark, plain and learned plans;
  configuration 5: R-MAT 2^24 / 256M edges (seed 5), K5 (one bag: counted as
                   embeddings) and the two 6-vertex fhtd patterns.
"""
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))


def cpu_counts(oracle, eng, plans, stride, offset, max_deg):
    og = oracle.Graph(eng.graph.offsets, eng.graph.nbrs)
    raw = b"".join(b.to_bytes() for b in plans)
    inst, roots = og.count_plans(raw, len(plans), threads=0, stride=stride, offset=offset, root_max_degree=max_deg)
    og.close()
    return [i * b.count_multiplier % (1 << 64) for i, b in zip(inst, plans)], roots


def test_config3_rmat20_batch_of_16_six_vertex_patterns(sge, oracle):
    import bench
    with sge.Engine.rmat_device(20, 16_000_000, seed=3) as eng:
        assert eng.info()["num_directed_edges"] == 32_000_000
        st = eng.graph.stats()
        pats = [sge.PatternGraph.random(6, 11 + i % 3, 1000 + i) for i in range(16)]
        plans = [bench.plain_plan(sge, p, st) for p in pats]
        opts = dict(root_stride=1 << 14, root_offset=1, root_max_degree=1000)
        gpu, _, _ = eng.count(plans, **opts)
        cpu, roots = cpu_counts(oracle, eng, plans, 1 << 14, 1, 1000)
        assert sum(roots) > 1000 and sum(gpu) > 10_000_000
        assert gpu == cpu


def test_config4_rmat22_benchmark_sample(sge, oracle):
    import bench
    import sge_learn
    with sge.Engine.rmat_device(22, 64_000_000, seed=4) as eng:
        st = eng.graph.stats()
        pats = bench.rmat22_patterns(sge)
        plain = [bench.plain_plan(sge, p, st) for p in pats]
        learned = bench.learned_plans(sge, pats, st, sge_learn.load_mlp())
        # the benchmark's sample: learned and plain plans count the same instances
        s = bench.sample_opts()
        cp, _, _ = eng.count(plain, **s)
        cl, _, _ = eng.count(learned, **s)
        assert cp == cl and sum(cp) > 10 ** 9
        # every 16th edge of it on the CPU: the check patterns bench.py uses
        sub = bench.sample_opts(1, 0, bench.CPU_SUBSAMPLE)
        chk = [b for i, b in enumerate(learned) if i % bench.CPU_CHECK_EVERY == 0]
        gpu, _, _ = eng.count(chk, **sub)
        cpu, _ = cpu_counts(oracle, eng, chk, sub["root_stride"], sub["root_offset"], sub["root_max_degree"])
        assert gpu == cpu
        # all 78 on every 64th edge of the sample
        sparse = bench.sample_opts(1, 0, 64)
        gpu, _, _ = eng.count(plain, **sparse)
        cpu, _ = cpu_counts(oracle, eng, plain, sparse["root_stride"], sparse["root_offset"], sparse["root_max_degree"])
        assert gpu == cpu


CONFIG5 = {
    "k5": (5, [(a, b) for a in range(5) for b in range(a + 1, 5)]),
    "c6_two_chords": (6, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (0, 5), (0, 3), (1, 4)]),
    "two_triangles_4cycle": (6, [(0, 1), (0, 2), (1, 2), (3, 4), (3, 5), (4, 5), (1, 3), (2, 4)]),
}


def test_config5_rmat24_k5_and_fhtd_patterns(sge, oracle):
    import bench
    with sge.Engine.rmat_device(24, 256_000_000, seed=5) as eng:
        info = eng.info()
        assert info["num_directed_edges"] == 512_000_000
        st = eng.graph.stats()
        plans = [bench.plain_plan(sge, sge.PatternGraph.from_edges(k, e), st) for k, e in CONFIG5.values()]
        assert plans[0].single_bag == 1 and plans[0].count_multiplier == 120  # K5: embeddings
        stride, offset, cap = CONFIG5_SAMPLE
        gpu, _, _ = eng.count(plans, root_stride=stride, root_offset=offset, root_max_degree=cap)
        cpu, roots = cpu_counts(oracle, eng, plans, stride, offset, cap)
        assert sum(roots) > 100 and all(c > 0 for c in gpu)
        assert gpu == cpu


# stride, offset, endpoint-degree cap of the configuration-5 sample
CONFIG5_SAMPLE = (1 << 18, 1, 1000)
