"""Root-edge sharding across ranks (the multi-GPU decomposition): ranks take
root tasks t ≡ rank (mod world) and the per-pattern counts are summed with one
all-reduce.  Exercised here with world_size=2 gloo ranks on CPU, each rank
running the CPU executor on its residue class."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import sys
    from pathlib import Path
    repo = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(repo / "subgraph-enumeration_gb300"), str(repo / "oracle")]
    import torch
    import torch.distributed as dist
    import sge
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = sge.gen_chung_lu(380, 915, 2.3, 0, 1)
    pats = [sge.PatternGraph.from_edges(5, [(0, 1), (0, 2), (0, 4), (1, 3), (1, 4), (2, 3)]),
            sge.PatternGraph.from_edges(4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)])]
    plans = [sge.plan(p, g, iep=True) for p in pats]
    part = [oracle.count_plan(g.offsets, g.nbrs, b, threads=1, stride=world, offset=rank)[0] * b.count_multiplier
            for b in plans]
    t = torch.tensor(part, dtype=torch.int64)
    dist.all_reduce(t)
    full = [oracle.count_plan(g.offsets, g.nbrs, b, threads=1)[0] * b.count_multiplier for b in plans]
    q.put((rank, t.tolist(), full))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_gloo_root_sharding_sums_to_full_count(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, summed, full in res:
        assert summed == full
