#!/usr/bin/env python3
"""Benchmark of the subgraph-enumeration hot path on GB300.

Workload (the configuration the headline metric is quoted on that fits one
GPU): a seeded Chung-Lu power-law data graph with n=7,100 vertices, 100,000
undirected edges, degree exponent 2.1 and maximum degree ~1,000 (uint32 CSR),
and the query patterns house (5 vertices, 6 edges), K5 minus one edge (9
edges) and the reference's 8-edge near-5-clique, each planned in the four
modes WCOJ / exploration (-i) × without / with IEP (-u).  One step = one
batched persistent launch counting all 12 plans; value = Σ counts / Σ step
time (embeddings per second in the reference's "Number of matches" units).

Arms:
  --impl sge        (default) the CUDA engine through libsge
  --impl reference  the CPU implementation of the same path on the host cores
                    (the oracle port of the reference executor, all threads)
Under torchrun (N>1) root tasks are sharded across ranks
(root_stride = world size, root_offset = rank) and per-pattern counts summed.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
PKG = REPO / "subgraph-enumeration_gb300"
sys.path.insert(0, str(PKG))

PATTERNS = {
    "house": (5, [(0, 1), (0, 2), (0, 4), (1, 3), (1, 4), (2, 3)]),
    "k5_minus_e": (5, [(a, b) for a in range(5) for b in range(a + 1, 5) if (a, b) != (3, 4)]),
    "near5clique_8e": (5, [(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 3), (1, 4), (2, 3)]),
}
MODES = [("wcoj", False, False), ("wcoj-u", False, True), ("explore", True, False), ("explore-u", True, True)]
GRAPH = dict(n=7100, m=100_000, gamma=2.1, max_deg=1000, seed=2)
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes (read + write) of one count_kernel launch of this workload,
    from the committed ncu summary (None when it is absent)."""
    f = REPO / "profiles" / "count_kernel_bench-step_chunglu-n7100.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("| dram bytes per launch (read + write) |"):
            try:
                return int(line.split("|")[2].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(sge):
    g = sge.gen_chung_lu(GRAPH["n"], GRAPH["m"], GRAPH["gamma"], GRAPH["max_deg"], GRAPH["seed"])
    return g


def make_plans(sge, stats_or_engine):
    plans, names = [], []
    for pname, (k, edges) in PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        for mname, expl, iep in MODES:
            plans.append(sge.plan(p, stats_or_engine, iep=iep, exploration=expl))
            names.append(f"{pname}/{mname}")
    return plans, names


def make_reference_plans(sge, oracle, g, stats, threads):
    """Plans for the CPU reference arm: the engine's plans, except that for
    the IEP modes (-u) the cheapest multi-level-tail plan (the reference's
    inclusion-exclusion leaf) replaces the engine's plan when it is faster on
    the host, timed on 1/64 of the roots.  The CPU side then runs the better
    of the two rather than a plan chosen for the GPU."""
    plans, names = [], []
    for pname, (k, edges) in PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        for mname, expl, iep in MODES:
            b = sge.plan(p, stats, iep=iep, exploration=expl)
            if iep and b.tail_len < 2:
                multi = [c for c in sge.candidates(p, stats, iep=True, exploration=expl, cap=4096) if c.tail_len >= 2]
                if multi:
                    alt = min(multi, key=lambda c: c.est_cost)
                    t = []
                    for cand in (b, alt):
                        t0 = time.perf_counter()
                        oracle.count_plan(g.offsets, g.nbrs, cand, threads=threads, stride=64, offset=0)
                        t.append(time.perf_counter() - t0)
                    if t[1] < t[0]:
                        b = alt
            plans.append(b)
            names.append(f"{pname}/{mname}")
    return plans, names


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """CPU arm: the oracle port of the reference executor on the host cores."""
    world, rank, _ = dist_env()
    if world > 1 and rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    import sge
    import oracle
    g = build_workload(sge)
    st = g.stats()
    threads = os.cpu_count() or 1
    plans, names = make_reference_plans(sge, oracle, g, st, threads)
    # bounded sample: every stride-th root; stride sized for ~10-20 s per step
    stride = int(os.environ.get("SGE_REF_STRIDE", "8"))
    def step(offset):
        t0 = time.perf_counter()
        total = 0
        roots = 0
        for b in plans:
            inst, done = oracle.count_plan(g.offsets, g.nbrs, b, threads=threads, stride=stride,
                                           offset=offset % stride)
            total += inst * b.count_multiplier
            roots += done
        return total, time.perf_counter() - t0, roots
    for w in range(args.warmup):
        step(w)
    tot_c, tot_t, roots = 0, 0.0, 0
    for s in range(args.steps):
        c, t, r = step(args.warmup + s)
        tot_c += c
        tot_t += t
        roots += r
    value = tot_c / tot_t
    line = {"metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "embeddings/s", "cores": threads, "kind": "port",
                             "sample": f"1/{stride} of the root edges of each of the 12 plans per step "
                                       f"({roots} roots over {args.steps} steps), extrapolation-free rate; "
                                       "IEP modes run the faster on the host of the engine's plan and the "
                                       "best inclusion-exclusion plan"},
            "e2e": {"value": value, "unit": "embeddings/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


METRIC = "embeddings/sec on 1 GB300 (reference 'Number of matches' units), bit-exact"


def workload_config():
    return {"workload": "chunglu_n7100_m100k_g2.1 x {house, k5_minus_e, near5clique_8e} x "
                        "{wcoj, wcoj-u, explore, explore-u}",
            "graph": dict(GRAPH, generator="chung_lu"), "patterns": list(PATTERNS), "plans_per_step": 12,
            "l2": "flushed between timed steps (512 MiB write); the 0.8 MB CSR itself is L2-resident",
            "parallelism": "root-edge sharding across ranks"}


def cpu_sample(oracle, g, plans, stride, offset, threads):
    t0 = time.perf_counter()
    total = roots = 0
    for b in plans:
        inst, done = oracle.count_plan(g.offsets, g.nbrs, b, threads=threads, stride=stride, offset=offset)
        total += inst * b.count_multiplier
        roots += done
    return total, time.perf_counter() - t0, roots


def cpu_baseline(sge, g, plans, budget_s=15.0):
    """The oracle port on all host cores over the same root sample of every
    pattern and mode of the step (every stride-th root edge), the stride
    shrunk until the sample takes about budget_s/3 .. budget_s seconds.  The
    plans are the reference arm's: the engine's, or for the IEP modes the best
    inclusion-exclusion plan when that is faster on the host."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    plans, _ = make_reference_plans(sge, oracle, g, g.stats(), threads)
    stride = 1 << 14
    while True:
        total, dt, roots = cpu_sample(oracle, g, plans, stride, 7 % stride, threads)
        if dt >= budget_s / 3 or stride == 1:
            break
        # aim at budget_s/2, never shrinking the stride by more than 16x per step
        stride = max(1, stride // max(2, min(16, int(budget_s / 2 / max(dt, 1e-3)))))
    return {"value": total / dt, "unit": "embeddings/s", "cores": threads, "kind": "port",
            "sample": f"root edges t = {7 % stride} mod {stride} of all {len(plans)} plans of a step ({roots} roots, "
                      f"{dt:.1f} s); value = embeddings of the sample / its time; IEP modes run the faster on the "
                      "host of the engine's plan and the best inclusion-exclusion plan"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="sge", choices=["sge", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plans", default="", help="comma-separated subset, e.g. house/wcoj-u (profiling)")
    ap.add_argument("--per-plan", action="store_true", help="time each plan alone and print one JSON per plan")
    ap.add_argument("--workload", default="chunglu7100", choices=["chunglu7100", "batch7", "ingest"],
                    help="batch7: 78 random 7-vertex patterns, learned+batched vs plain planning; "
                         "ingest: R-MAT 2^20 vertices / 16M edges generated and built on the GPU vs the host "
                         "(separate lines)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch7":
        return run_batch7(args)
    if args.workload == "ingest":
        return run_ingest(args)
    world, rank, local = dist_env()
    import torch
    import sge
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(device)
    g = build_workload(sge)
    eng = sge.Engine(g, device=device)
    plans, names = make_plans(sge, eng)
    if args.plans:
        keep = set(args.plans.split(","))
        sel = [i for i, n in enumerate(names) if n in keep]
        plans, names = [plans[i] for i in sel], [names[i] for i in sel]
    if args.per_plan:
        for b, n in zip(plans, names):
            eng.count([b])
            c, _, st = eng.count([b], stats=True)
            c2, _, st2 = eng.count([b])
            print(json.dumps({"plan": n, "count": c[0], "kernel_ms": st2["kernel_ms"], "alg_bytes": st["alg_bytes"],
                              "set_ops": st["set_ops"], "partial_matches": st["partial_matches"],
                              "roots": st["root_tasks"], "stats_kernel_ms": st["kernel_ms"],
                              "plan_summary": b.summary()}), flush=True)
        eng.close()
        return
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=f"cuda:{device}")
    shard = dict(root_stride=world, root_offset=rank) if world > 1 else {}

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up
    for _ in range(args.warmup):
        eng.count(plans, **shard)
    # algorithmic bytes of one launch (stats variant, untimed)
    _, _, st = eng.count(plans, stats=True, **shard)
    alg_bytes = st["alg_bytes"]
    # timed steps: one replay of the captured batch (CUDA graph) per step, L2
    # flushed before each; device time from events around the graph launch
    kernel_ms, host_ms, counts, launches = [], [], None, 0
    batch = eng.batch(plans, **shard)
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            barrier()
            t0 = time.perf_counter()
            c, inst, s = batch.run()
            t1 = time.perf_counter()
            barrier()
            kernel_ms.append(s["kernel_ms"])
            host_ms.append((t1 - t0) * 1e3)
            launches += s["gpu_launches"]
            counts = c
    batch.close()
    # reduce over ranks: counts summed, times max
    if dist:
        tc = torch.tensor(counts, dtype=torch.int64, device=f"cuda:{device}")
        dist.all_reduce(tc)
        counts = [int(x) % 2**64 for x in tc.tolist()]
        tk = torch.tensor([sum(kernel_ms), sum(host_ms)], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(tk, op=dist.ReduceOp.MAX)
        sum_k, sum_h = tk.tolist()
    else:
        sum_k, sum_h = sum(kernel_ms), sum(host_ms)
    total_count = sum(counts)
    value = total_count * args.steps / (sum_k / 1e3)
    # e2e: host buffers through the C ABI (H2D, count, D2H inside the timed region)
    e2e_ms = []
    for _ in range(max(2, min(args.steps, 5))):
        barrier()
        t0 = time.perf_counter()
        ec, est = sge.count_host(g, plans, stats=False)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        assert ec == counts or world > 1
    e2e_value = total_count / (statistics.median(e2e_ms) / 1e3)
    h2d = 4 * (g.num_vertices + 1) + 4 * g.nbrs.size + 8 * g.num_edges + 300 * len(plans)
    d2h = 8 * len(plans) + 4
    peak, peak_kind = peaks()
    avg_launch_s = sum_k / len(kernel_ms) / 1e3
    achieved = alg_bytes / avg_launch_s / 1e9
    traffic = profile_traffic()
    line = {
        "metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum_k / len(kernel_ms), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
        "config": workload_config(),
        "counts": dict(zip(names, counts)),
        "host_ms_per_step": sum_h / len(host_ms),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes,
                     "note": "algorithmic bytes = 4·(base + probed list elements) per set operation + 8 B per "
                             "CSR offset pair; the CSR is L2-resident at this size"},
        "e2e": {"value": e2e_value, "unit": "embeddings/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": statistics.median(e2e_ms)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sge, g, plans)
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


INGEST_GRAPH = dict(scale=20, m=16_000_000, a=0.57, b=0.19, c=0.19, seed=11)


def run_ingest(args):
    """Graph ingest for the batch configuration's data graph (R-MAT a=.57
    b=.19 c=.19, 2^20 vertices, 16M undirected edges): generation, dedup and
    CSR build on the GPU (sge_graph_create_rmat) against the host generator,
    host CSR build and upload (sge_gen_rmat + sge_csr_from_edges +
    sge_graph_create).  Both give the same CSR, which is checked."""
    import sge
    import numpy as np
    gs = INGEST_GRAPH
    rgs = (gs["scale"], gs["m"], gs["a"], gs["b"], gs["c"], gs["seed"])
    sge.Engine.rmat_device(10, 5000, seed=1).close()  # context and module load outside the timing
    dev_s, host_s = [], []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        eng = sge.Engine.rmat_device(*rgs)
        dev_s.append(time.perf_counter() - t0)
        off, nb = eng.graph.offsets, eng.graph.nbrs
        eng.close()
    t0 = time.perf_counter()
    g = sge.gen_rmat(*rgs)
    hg = sge.Engine(g)
    host_s.append(time.perf_counter() - t0)
    hg.close()
    assert np.array_equal(off, g.offsets) and np.array_equal(nb, g.nbrs)
    line = {"metric": "R-MAT data graph ingest (generate, dedup, symmetric CSR on the device), seconds",
            "value": statistics.median(dev_s), "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "steps": args.steps, "host_s": host_s[0], "speedup_vs_host": host_s[0] / statistics.median(dev_s),
            "data": "synthetic", "dtype": "u32 ids",
            "config": {"workload": "rmat_s20_m16M ingest", "graph": dict(gs, generator="rmat"),
                       "directed_edges": int(nb.size), "csr_identical_to_host": True,
                       "device_path": "sge_graph_create_rmat (includes the host copy used for planner statistics)",
                       "host_path": "sge_gen_rmat + sge_csr_from_edges + sge_graph_create (validation, upload)"}}
    print(json.dumps(line), flush=True)


BATCH7_GRAPH = dict(scale=10, m=8000, a=0.57, b=0.19, c=0.19, seed=4)


def run_batch7(args):
    """Learned + batched vs plain planning on a batch of 78 seeded random
    7-vertex patterns (16-19 edges) over a seeded R-MAT graph (scale 10,
    8,000 edges: the batch configuration's generator at a size whose exact
    counts finish in seconds).  Wall time includes planning.
      plain:   per pattern, cost-model plan then its own launch (as the
               reference runs one process per pattern)
      learned: shortlists on host threads, one BF16 MLP scoring call for all
               patterns, one launch of all plans replayed from a CUDA graph."""
    import concurrent.futures as cf
    import numpy as np
    import torch
    import sge
    import sge_learn
    gs = BATCH7_GRAPH
    g = sge.gen_rmat(gs["scale"], gs["m"], gs["a"], gs["b"], gs["c"], gs["seed"])
    pats = [sge.PatternGraph.random(7, 16 + i % 4, 2000 + i) for i in range(78)]
    eng = sge.Engine(g)
    st = g.stats()
    mlp = sge_learn.load_mlp()

    def plain():
        t0 = time.perf_counter()
        counts, plan_s, kern = [], 0.0, 0.0
        for p in pats:
            a = time.perf_counter()
            b = sge.plan(p, st)
            plan_s += time.perf_counter() - a
            c, _, s = eng.count([b])
            kern += s["kernel_ms"]
            counts.append(c[0])
        return counts, time.perf_counter() - t0, plan_s, kern

    def learned():
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            shortlists = list(ex.map(lambda p: sge.candidates(p, st, cap=64), pats))
        feats = np.concatenate([np.stack([sge.features(b, st) for b in sl]) for sl in shortlists])
        pred = mlp.forward(feats, bf16=True)
        plans, o = [], 0
        for sl in shortlists:
            plans.append(sl[int(np.argmin(pred[o:o + len(sl)]))])
            o += len(sl)
        plan_s = time.perf_counter() - t0
        with eng.batch(plans) as bt:
            c, _, s = bt.run()
        return c, time.perf_counter() - t0, plan_s, s["kernel_ms"]

    for _ in range(args.warmup):
        learned()
    pw, lw, pk, lk, pp, lp = [], [], [], [], [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        cp, tp, plan_p, kp = plain()
        cl, tl, plan_l, kl = learned()
        assert cp == cl, "plain and learned plans disagree"
        pw.append(tp); lw.append(tl); pk.append(kp); lk.append(kl); pp.append(plan_p); lp.append(plan_l)
    total = sum(cl)
    # the same learned plans with no heavy-root splitting (one launch, a warp per root)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        shortlists = list(ex.map(lambda p: sge.candidates(p, st, cap=64), pats))
    feats = np.concatenate([np.stack([sge.features(b, st) for b in sl]) for sl in shortlists])
    pred = mlp.forward(feats, bf16=True)
    plans, o = [], 0
    for sl in shortlists:
        plans.append(sl[int(np.argmin(pred[o:o + len(sl)]))])
        o += len(sl)
    with eng.batch(plans, heavy_threshold=1 << 30) as bt:
        cn, _, sn = bt.run()
    assert cn == cl
    line = {"metric": "embeddings/sec, learned+batched planning and execution (wall time incl. planning)",
            "value": total / statistics.median(lw), "unit": "embeddings/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(lw), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
            "config": {"workload": "rmat_s10_m8000 x 78 random 7-vertex patterns (16-19 edges)",
                       "graph": dict(gs, generator="rmat"), "patterns": "PatternGraph.random(7, 16 + i%4, 2000 + i)"},
            "learned_batched": {"wall_s": statistics.median(lw), "planning_s": statistics.median(lp),
                                "kernel_ms": statistics.median(lk), "kernel_ms_without_root_split": sn["kernel_ms"]},
            "plain": {"wall_s": statistics.median(pw), "planning_s": statistics.median(pp),
                      "kernel_ms": statistics.median(pk), "value": total / statistics.median(pw)},
            "speedup_wall": statistics.median(pw) / statistics.median(lw),
            "speedup_kernel": statistics.median(pk) / statistics.median(lk),
            "total_count": total}
    eng.close()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
