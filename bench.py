#!/usr/bin/env python3
"""Benchmark of the subgraph-enumeration hot path on GB300.

Default workload (the configuration the headline metric is quoted on):
78 seeded random connected 7-vertex patterns with 16-19 edges
(PatternGraph.random(7, 16 + i % 4, 2000 + i)) counted on a seeded R-MAT data
graph with 2^22 vertices and 64M undirected edges (a=.57 b=.19 c=.19, seed 4,
deduplicated, self-loop-free, ids unpermuted), built on the GPU.  Exact counts
of these dense patterns over all 64M root edges are beyond any executor: the
reference needs more than a minute for one of them on a 65K-edge R-MAT, 61
sampled root edges already hold ~1e15 instances of a pattern, and a single
root between two degree-3,000 vertices holds 1.4e9 (about 3,000 CPU
core-seconds).  So a step counts a fixed root sample: the undirected root
edges e ≡ SAMPLE_OFFSET (mod SAMPLE_STRIDE) in CSR order, both orientations,
whose two endpoints both have degree <= ROOT_MAX_DEGREE.  For
each pattern the planner keeps one symmetry-restriction sequence and one
root pattern edge (canonical_symmetry), so every plan of a pattern counts
the same instances on the sample and the two planners below are compared on
identical counts.

  plain   per pattern: the cost model's plan, then its own launch
  learned shortlists on host threads, one BF16 MLP scoring call for all 78
          patterns, one persistent launch of all plans replayed from a CUDA
          graph (the headline value)

value = Σ sample counts / device time of one batched step (inputs resident in
HBM); e2e = the same through sge_count_host with the CSR in host memory.
Counts are the reference's "Number of matches" units (instances: every
pattern here is a multi-bag plan).

Other workloads: --workload chunglu7100 (a seeded Chung-Lu n=7,100 graph,
house / K5-e / 8-edge near-5-clique in the four modes WCOJ, WCOJ+IEP,
exploration, exploration+IEP; full counts), --workload ingest, --workload
bags (the two 6-vertex patterns of the R-MAT 2^24 configuration through their
bag relations' tries against the plain DFS leaf, on a down-scaled R-MAT).

Arms:
  --impl sge        (default) the CUDA engine through libsge
  --impl reference  the CPU implementation of the same path on the host cores:
                    the oracle port of the reference executor with all host
                    threads, on a bounded sub-sample of the same workload; it
                    loads only oracle/_build/liboracle.so (graphs from the
                    oracle's copies of the seeded generators, plans from
                    tests/golden/bench_plans.npz)
Under torchrun (N>1) the sampled root edges are sharded across ranks and the
per-pattern counts summed.
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

METRIC = "embeddings/sec on 1 GB300, learned+batched vs plain plan, bit-exact; %HBM peak"

RMAT22 = dict(scale=22, m=64_000_000, a=0.57, b=0.19, c=0.19, seed=4)
SAMPLE_STRIDE = 1 << 16      # root edges e ≡ SAMPLE_OFFSET (mod SAMPLE_STRIDE) ...
SAMPLE_OFFSET = 1
ROOT_MAX_DEGREE = 1000       # ... whose endpoints both have degree <= ROOT_MAX_DEGREE
CPU_SUBSAMPLE = 16           # the CPU runs every CPU_SUBSAMPLE-th edge of the sample ...
CPU_SLICES = 13              # ... for 78/13 = 6 patterns per reference-arm step (a 13-step cycle covers all)
CPU_CHECK_EVERY = 6          # cpu_baseline and the GPU/CPU check: patterns i ≡ 0 (mod 6), 13 of them
N_PATTERNS = 78

CL_GRAPH = dict(n=7100, m=100_000, gamma=2.1, max_deg=1000, seed=2)
CL_PATTERNS = {
    "house": (5, [(0, 1), (0, 2), (0, 4), (1, 3), (1, 4), (2, 3)]),
    "k5_minus_e": (5, [(a, b) for a in range(5) for b in range(a + 1, 5) if (a, b) != (3, 4)]),
    "near5clique_8e": (5, [(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 3), (1, 4), (2, 3)]),
}
CL_MODES = [("wcoj", False, False), ("wcoj-u", False, True), ("explore", True, False), ("explore-u", True, True)]
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2
PLAN_FIXTURE = REPO / "tests" / "golden" / "bench_plans.npz"


# ------------------------------------------------------------------ shared ----
def peaks():
    f = REPO / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name: str):
    """DRAM bytes (read + write) of one count_kernel launch of a workload,
    from its committed ncu summary (None when absent)."""
    f = REPO / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("| dram bytes per launch (read + write) |"):
            try:
                return int(line.split("|")[2].strip().replace(",", ""))
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


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def canonical_symmetry(k: int, edges) -> tuple[list[int], list[int]]:
    """The symmetry-restriction sequence and root pattern edge every plan of a
    pattern keeps: the root is the edge with the largest degree sum (ties:
    smaller ids), its higher-degree end first; the sequence is the root, then
    the other vertices by decreasing degree."""
    E = [(int(a), int(b)) for a, b in edges]
    deg = [0] * k
    for a, b in E:
        deg[a] += 1
        deg[b] += 1
    a, b = max(E, key=lambda e: (deg[e[0]] + deg[e[1]], -min(e), -max(e)))
    if deg[b] > deg[a]:
        a, b = b, a
    rest = sorted((v for v in range(k) if v not in (a, b)), key=lambda v: (-deg[v], v))
    return [a, b] + rest, [a, b]


def rmat22_patterns(sge):
    return [sge.PatternGraph.random(7, 16 + i % 4, 2000 + i) for i in range(N_PATTERNS)]


def plain_plan(sge, p, st):
    seq, root = canonical_symmetry(p.k, p.edges)
    return sge.plan(p, st, symmetry_seq=seq, root_edge=root)


def learned_plans(sge, pats, st, mlp, threads: int = 16):
    """Shortlists (cost model, 64 candidates each, on host threads), one BF16
    scoring call for every candidate of every pattern, argmin per pattern."""
    import concurrent.futures as cf
    import numpy as np

    def shortlist(p):
        seq, root = canonical_symmetry(p.k, p.edges)
        sl = sge.candidates(p, st, cap=64, symmetry_seq=seq, root_edge=root)
        return sl, np.stack([sge.features(b, st) for b in sl])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(threads, os.cpu_count() or 1))) as ex:
        res = list(ex.map(shortlist, pats))
    pred = mlp.forward(np.concatenate([f for _, f in res]), bf16=True)
    plans, o = [], 0
    for sl, f in res:
        plans.append(sl[int(np.argmin(pred[o:o + len(sl)]))])
        o += len(sl)
    return plans


def sample_opts(world: int = 1, rank: int = 0, sub: int = 1) -> dict:
    """Root sample of a step (sub > 1: every sub-th edge of it; world > 1:
    this rank's share).  Edges e ≡ SAMPLE_OFFSET (mod SAMPLE_STRIDE) split as
    e ≡ SAMPLE_OFFSET + j·SAMPLE_STRIDE (mod SAMPLE_STRIDE·n), j < n."""
    n = world * sub
    return dict(root_stride=SAMPLE_STRIDE * n, root_offset=SAMPLE_OFFSET + rank * SAMPLE_STRIDE,
                root_max_degree=ROOT_MAX_DEGREE)


def rmat22_config(extra: dict | None = None, scale: int = RMAT22["scale"], npat: int = N_PATTERNS) -> dict:
    size = "m64M" if scale == RMAT22["scale"] else f"m{(16 << scale) // 1_000_000}M"
    c = {"workload": f"rmat_s{scale}_{size} x {npat} random 7-vertex patterns (16-19 edges), root sample: undirected "
                     f"edges e = {SAMPLE_OFFSET} mod {SAMPLE_STRIDE} (CSR order, both orientations) with both "
                     f"endpoint degrees <= {ROOT_MAX_DEGREE}",
         "graph": dict(RMAT22, generator="rmat", ids="unpermuted", built="on the GPU (sge_graph_create_rmat)"),
         "patterns": "PatternGraph.random(7, 16 + i % 4, 2000 + i), i < 78",
         "root_sample": {"stride": SAMPLE_STRIDE, "offset": SAMPLE_OFFSET, "max_endpoint_degree": ROOT_MAX_DEGREE,
                         "edges_before_degree_cap": (RMAT22["m"] if scale == RMAT22["scale"] else 16 << scale)
                         // SAMPLE_STRIDE},
         "symmetry": "per pattern one restriction sequence and root edge for every plan (canonical_symmetry)",
         "l2": "inputs larger than L2 (512 MB CSR + 4 GB hub bitmaps); 512 MiB L2 flush before each timed step",
         "parallelism": "root-edge sharding across ranks"}
    if extra:
        c.update(extra)
    return c


def chunglu_config() -> dict:
    return {"workload": "chunglu_n7100_m100k_g2.1 x {house, k5_minus_e, near5clique_8e} x "
                        "{wcoj, wcoj-u, explore, explore-u}, full counts",
            "graph": dict(CL_GRAPH, generator="chung_lu"), "patterns": list(CL_PATTERNS), "plans_per_step": 12,
            "l2": "flushed between timed steps (512 MiB write); the 0.8 MB CSR itself is L2-resident",
            "parallelism": "root-edge sharding across ranks"}


def native_loaded() -> list | None:
    """This repository's shared libraries mapped into the process."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    found = set()
    for ln in maps:
        path = ln.split()[-1] if ln.split() else ""
        if path.endswith(".so") and path.startswith(str(REPO) + "/"):
            found.add(path[len(str(REPO)) + 1:])
    return sorted(found)


# ------------------------------------------------------- reference (CPU) arm ----
def oracle_graph(name: str):
    """Data graph of a workload built by the oracle's copies of the seeded
    generators (the reference arm never loads the library)."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    if name == "rmat22":
        g = RMAT22
        return oracle.gen_rmat(g["scale"], g["m"], g["a"], g["b"], g["c"], g["seed"])
    g = CL_GRAPH
    return oracle.gen_chung_lu(g["n"], g["m"], g["gamma"], g["max_deg"], g["seed"])


def fixture_plans(key: str):
    import numpy as np
    d = np.load(PLAN_FIXTURE)
    return d[key]


def blob_multiplier(blob) -> int:
    """count_multiplier of a raw sge_plan_blob (layout of include/sge.h)."""
    import numpy as np
    # magic, abi, k, num_enum, tail_mode, tail_len, join_style, root_kind: 8 u32;
    # 8 arrays of SGE_MAX_K u32; num_partitions; 15 i32; 15 u32; 15x4 u32; then u64
    off = 4 * (8 + 8 * 16 + 1 + 15 + 15 + 60)
    off = (off + 7) & ~7
    return int(np.frombuffer(bytes(blob[off:off + 8]), np.uint64)[0])


def run_reference(args):
    """The CPU implementation of the path (the oracle port of the reference
    executor, every host thread) on a bounded sample of the workload."""
    world, rank, _ = dist_env()
    if world > 1 and rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    off, nb = oracle_graph(args.workload)
    og = oracle.Graph(off, nb)
    setup_s = time.perf_counter() - t0
    slices = 1
    if args.workload == "rmat22":
        blobs = fixture_plans("rmat22_plain")
        sub = dict(stride=SAMPLE_STRIDE * CPU_SUBSAMPLE, offset=SAMPLE_OFFSET, root_max_degree=ROOT_MAX_DEGREE)
        slices = CPU_SLICES
        sample_desc = (f"undirected root edges e = {SAMPLE_OFFSET} mod {SAMPLE_STRIDE * CPU_SUBSAMPLE} with endpoint "
                       f"degrees <= {ROOT_MAX_DEGREE} (every {CPU_SUBSAMPLE}th edge of the GPU's sample); step s runs "
                       f"patterns i = s mod {CPU_SLICES} (a {CPU_SLICES}-step cycle covers all 78), with the cost "
                       "model's plans under the same symmetry as the GPU's")
        config = rmat22_config()
    else:
        plans = fixture_plans("chunglu7100_plans")
        alts = fixture_plans("chunglu7100_alt")
        # the IEP modes run whichever of the engine's plan and the best
        # inclusion-exclusion plan is faster on these cores (timed on 1/64)
        blobs = []
        for b, a in zip(plans, alts):
            if bytes(a) == bytes(b):
                blobs.append(b)
                continue
            t = []
            for cand in (b, a):
                s = time.perf_counter()
                og.count_plans(bytes(cand), 1, threads=threads, stride=64, offset=0)
                t.append(time.perf_counter() - s)
            blobs.append(a if t[1] < t[0] else b)
        sub = dict(stride=8, offset=0)
        sample_desc = ("undirected root edges e = 0 mod 8 of all 12 plans per step; IEP modes run the faster on "
                       "the host of the engine's plan and the best inclusion-exclusion plan")
        config = chunglu_config()
    mult = [blob_multiplier(b) for b in blobs]

    def step(j):
        sel = [i for i in range(len(blobs)) if i % slices == j % slices]
        raw = b"".join(bytes(blobs[i]) for i in sel)
        s = time.perf_counter()
        inst, roots = og.count_plans(raw, len(sel), threads=threads, **sub)
        return sum(i * mult[k] for i, k in zip(inst, sel)) % (1 << 64), time.perf_counter() - s, sum(roots)
    for j in range(args.warmup):
        step(j)
    tot_c, tot_t, tot_r = 0, 0.0, 0
    for j in range(args.steps):
        c, t, r = step(args.warmup + j)
        tot_c += c
        tot_t += t
        tot_r += r
    value = tot_c / tot_t
    line = {"metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
            "impl": "reference", "config": config,
            "cpu_baseline": {"value": value, "unit": "embeddings/s", "cores": threads, "kind": "port",
                             "sample": f"{sample_desc} ({tot_r} root tasks over {args.steps} steps)"},
            "e2e": {"value": value, "unit": "embeddings/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": setup_s, "native_loaded": native_loaded()}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU arm ----
def cpu_port_check(off, nb, plans, gpu_sub_counts, sub: dict, what: str = "") -> dict:
    """The oracle port on every host core over a sub-sample of the step's
    roots, with the step's own plans: its rate is the CPU baseline, and its
    counts must equal the GPU's on the same sub-sample."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    raw = b"".join(b.to_bytes() for b in plans)
    og = oracle.Graph(off, nb)
    t0 = time.perf_counter()
    inst, roots = og.count_plans(raw, len(plans), threads=threads, stride=sub["root_stride"],
                                 offset=sub["root_offset"], root_max_degree=sub.get("root_max_degree", 0))
    dt = time.perf_counter() - t0
    og.close()
    cpu = [i * b.count_multiplier % (1 << 64) for i, b in zip(inst, plans)]
    cap = f" with endpoint degrees <= {sub['root_max_degree']}" if sub.get("root_max_degree") else ""
    return {"value": sum(cpu) / dt, "unit": "embeddings/s", "cores": threads, "kind": "port",
            "sample": f"undirected root edges e = {sub['root_offset']} mod {sub['root_stride']}{cap} of "
                      f"{what or 'all'} {len(plans)} plans ({sum(roots)} root tasks, {dt:.1f} s); value = embeddings "
                      "of the sample / its time",
            "parity_with_gpu": cpu == list(gpu_sub_counts), "seconds": dt}


def run_rmat22(args):
    import numpy as np
    import torch
    import sge
    import sge_learn
    import sge_tune
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(device)
    g = dict(RMAT22)
    if args.scale != g["scale"]:
        g.update(scale=args.scale, m=16 << args.scale)
    t0 = time.perf_counter()
    eng = sge.Engine.rmat_device(g["scale"], g["m"], g["a"], g["b"], g["c"], g["seed"], device=device)
    ingest_s = time.perf_counter() - t0
    info = eng.info()
    st = eng.graph.stats()
    pats = rmat22_patterns(sge)[:args.patterns]
    mlp = sge_learn.load_mlp()
    shard = sample_opts(world, rank)
    if args.max_level_capacity:
        shard["max_level_capacity"] = args.max_level_capacity

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def plain():
        tw = time.perf_counter()
        counts, plan_s, kern, pplans = [], 0.0, 0.0, []
        for p in pats:
            a = time.perf_counter()
            b = plain_plan(sge, p, st)
            plan_s += time.perf_counter() - a
            c, _, s = eng.count([b], **shard)
            kern += s["kernel_ms"]
            counts.append(c[0])
            pplans.append(b)
        return counts, time.perf_counter() - tw, plan_s, kern, pplans

    def learned():
        tw = time.perf_counter()
        plans = learned_plans(sge, pats, st, mlp)
        plan_s = time.perf_counter() - tw
        with eng.batch(plans, **shard) as bt:
            c, _, s = bt.run()
        return plans, c, time.perf_counter() - tw, plan_s, s["kernel_ms"]

    # warm-up (module load, allocations), then the planners' wall times
    learned()
    barrier()
    plans, cl, lw, lp, lk = learned()
    barrier()
    cp, pw, pp, pk, pplans = plain()
    barrier()
    assert cp == cl, "plain and learned plans disagree on the sample"
    # the plain plans in one batched launch (separates the planner's gain from batching)
    _, _, spb = eng.count(pplans, **shard)
    # the autotuner: shared-memory tables per launch, heavy-root split and hub
    # use per plan, from short runs on every 4th edge of the sample
    tt = time.perf_counter()
    tuned = sge_tune.tune(eng, plans, {k: v for k, v in shard.items() if k != "max_level_capacity"})
    tune_s = time.perf_counter() - tt
    # timed steps: replays of the tuned learned batch (CUDA graph), L2 flushed before each
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=f"cuda:{device}")
    batch = eng.batch(plans, pin_tables=tuned.pin_tables, tuning=tuned.plans, **shard)
    for _ in range(args.warmup):
        batch.run()
    kernel_ms, launches, counts = [], 0, None
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            barrier()
            c, _, s = batch.run()
            barrier()
            kernel_ms.append(s["kernel_ms"])
            launches += s["gpu_launches"]
            counts = c
    batch.close()
    # untimed: algorithmic bytes of one step (instrumented kernel) and the
    # same step without hub bitmaps
    _, _, sst = eng.count(plans, stats=True, pin_tables=tuned.pin_tables, tuning=tuned.plans, **shard)
    _, _, snh = eng.count(plans, hub_bitmaps=False, **shard)
    if dist:
        tc = torch.tensor([x % (1 << 63) for x in counts], dtype=torch.int64, device=f"cuda:{device}")
        dist.all_reduce(tc)
        counts_all = [int(x) for x in tc.tolist()]
        tk = torch.tensor([sum(kernel_ms)], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(tk, op=dist.ReduceOp.MAX)
        sum_k = float(tk.item())
    else:
        counts_all, sum_k = counts, sum(kernel_ms)
    total = sum(counts_all)
    avg_s = sum_k / len(kernel_ms) / 1e3
    value = total / avg_s
    # e2e through the C ABI with the CSR in host memory (upload, root list,
    # hub index, count and read-back inside the timed region)
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 2))):
        barrier()
        t = time.perf_counter()
        ec, _ = sge.count_host(eng.graph, plans, **{k: v for k, v in shard.items() if k != "max_level_capacity"})
        e2e_ms.append((time.perf_counter() - t) * 1e3)
        assert ec == counts
    e2e_value = sum(counts) / (statistics.median(e2e_ms) / 1e3)
    # the CSR and the plan blobs (the root edge list and the hub index are built on the device)
    h2d = 4 * (info["num_vertices"] + 1) + 4 * info["num_directed_edges"] + len(plans[0].to_bytes()) * len(plans)
    d2h = 8 * len(plans) + 4
    peak, peak_kind = peaks()
    achieved = sst["alg_bytes"] / avg_s / 1e9
    traffic = profile_traffic("count_kernel_rmat22-sample.md")  # DRAM bytes of one step, measured by ncu
    line = {
        "metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum_k / len(kernel_ms), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
        "config": rmat22_config({"graph": dict(g, generator="rmat", ids="unpermuted",
                                               built="on the GPU (sge_graph_create_rmat)"),
                                 "patterns_used": len(pats),
                                 "ingest_s": ingest_s, "hub_index": {"hubs": info["hub_count"],
                                                                      "min_degree": info["hub_min_degree"]},
                                 "max_degree": info["max_degree"]}, g["scale"], len(pats)),
        "learned_batched": {"wall_s": lw, "planning_s": lp, "kernel_ms": lk, "value_wall": total / lw,
                            "note": "planning + one launch with the automatic settings"},
        "autotuner": {"tuning_s": tune_s, "tuning_kernel_ms": tuned.tuning_ms, "runs": tuned.runs,
                      "pin_tables": tuned.pin_tables,
                      "choices": {str(k): tuned.choice.count(k) for k in sorted(set(tuned.choice))},
                      "candidates": [list(c) for c in sge_tune.CANDIDATES]},
        "kernel_ms_untuned": lk,
        "plain": {"wall_s": pw, "planning_s": pp, "kernel_ms": pk, "value_wall": total / pw,
                  "launches": len(pats)},
        "plain_plans_batched_kernel_ms": spb["kernel_ms"],
        "speedup_wall": pw / lw, "speedup_kernel": pk / lk,
        "kernel_ms_without_hub_bitmaps": snh["kernel_ms"],
        "total_count": total,
        "roofline": {"bound": "latency", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "dram_gbs": traffic / avg_s / 1e9 if traffic else None,
                     "dram_frac": traffic / avg_s / 1e9 / peak if traffic else None,
                     "alg_bytes_per_launch": sst["alg_bytes"],
                     "note": "one step = the batched launch sequence (phase 0, task numbering, phase 1); "
                             "algorithmic bytes = 4 B per scanned element + per probed list 4 B per probe through "
                             "a hub bitmap or pinned table, else the list as a merge consumes it (+8 B offsets), "
                             "summed by the instrumented kernel; traffic = ncu DRAM read+write of the same step "
                             "(profiles/count_kernel_rmat22-sample.md). The working set stays in L1/L2, so the DFS "
                             "is bound by dependent-load latency, not HBM bandwidth"},
        "e2e": {"value": e2e_value, "unit": "embeddings/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": statistics.median(e2e_ms)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sub = sample_opts(1, 0, CPU_SUBSAMPLE)
        chk = [b for i, b in enumerate(plans) if i % CPU_CHECK_EVERY == 0]
        gsub, _, gst = eng.count(chk, **sub)
        line["cpu_baseline"] = cpu_port_check(eng.graph.offsets, eng.graph.nbrs, chk, gsub, sub,
                                              f"patterns i = 0 mod {CPU_CHECK_EVERY}:")
        line["cpu_baseline"]["gpu_value_same_sample"] = sum(gsub) / (gst["kernel_ms"] / 1e3)
        # the GPU on exactly the reference arm's sample (every 16th edge, all
        # 78 patterns, the plain plans of its fixture)
        rc, _, rst = eng.count(pplans, **sub)
        line["reference_arm_sample_gpu_value"] = sum(rc) / (rst["kernel_ms"] / 1e3)
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_chunglu(args):
    import torch
    import sge
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(device)
    g = sge.gen_chung_lu(CL_GRAPH["n"], CL_GRAPH["m"], CL_GRAPH["gamma"], CL_GRAPH["max_deg"], CL_GRAPH["seed"])
    eng = sge.Engine(g, device=device)
    plans, names = [], []
    for pname, (k, edges) in CL_PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        for mname, expl, iep in CL_MODES:
            plans.append(sge.plan(p, eng, iep=iep, exploration=expl))
            names.append(f"{pname}/{mname}")
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
                              "roots": st["root_tasks"], "plan_summary": b.summary()}), flush=True)
        eng.close()
        return
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=f"cuda:{device}")
    shard = dict(root_stride=world, root_offset=rank) if world > 1 else {}

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
    for _ in range(args.warmup):
        eng.count(plans, **shard)
    _, _, st = eng.count(plans, stats=True, **shard)
    kernel_ms, launches, counts = [], 0, None
    batch = eng.batch(plans, **shard)
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            barrier()
            c, _, s = batch.run()
            barrier()
            kernel_ms.append(s["kernel_ms"])
            launches += s["gpu_launches"]
            counts = c
    batch.close()
    if dist:
        tc = torch.tensor(counts, dtype=torch.int64, device=f"cuda:{device}")
        dist.all_reduce(tc)
        counts = [int(x) % 2**64 for x in tc.tolist()]
        tk = torch.tensor([sum(kernel_ms)], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(tk, op=dist.ReduceOp.MAX)
        sum_k = float(tk.item())
    else:
        sum_k = sum(kernel_ms)
    total = sum(counts)
    value = total * args.steps / (sum_k / 1e3)
    e2e_ms = []
    for _ in range(max(2, min(args.steps, 5))):
        barrier()
        t0 = time.perf_counter()
        ec, _ = sge.count_host(g, plans)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        assert ec == counts or world > 1
    e2e_value = total / (statistics.median(e2e_ms) / 1e3)
    h2d = 4 * (g.num_vertices + 1) + 4 * g.nbrs.size + len(plans[0].to_bytes()) * len(plans)
    d2h = 8 * len(plans) + 4
    avg_s = sum_k / len(kernel_ms) / 1e3
    line = {
        "metric": METRIC, "value": value, "unit": "embeddings/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum_k / len(kernel_ms), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u32 ids / u64 counts", "data": "synthetic",
        "config": chunglu_config(), "counts": dict(zip(names, counts)),
        "roofline": {"bound": "l2/latency", "achieved": st["alg_bytes"] / avg_s / 1e9, "unit": "GB/s",
                     "alg_bytes_per_launch": st["alg_bytes"], "l2_hit_rate": profile_l2_hit(),
                     "traffic": profile_traffic("count_kernel_bench-step_chunglu-n7100.md"),
                     "note": "the 0.8 MB CSR and its hub bitmaps stay in L2, so the kernel is bound by L2/shared-"
                             "memory latency of the dependent probes; no HBM fraction is claimed"},
        "e2e": {"value": e2e_value, "unit": "embeddings/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": statistics.median(e2e_ms)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        gsub, _, _ = eng.count(plans, root_stride=8, root_offset=0)
        line["cpu_baseline"] = cpu_port_check(g.offsets, g.nbrs, plans, gsub, dict(root_stride=8, root_offset=0))
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def profile_l2_hit():
    f = REPO / "profiles" / "count_kernel_bench-step_chunglu-n7100.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("| lts__t_sector_hit_rate"):
            try:
                return float(line.split("|")[2].strip().rstrip("%")) / 100.0
            except ValueError:
                return None
    return None


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
                       "device_path": "sge_graph_create_rmat (includes the host copy used for planner statistics "
                                      "and the hub index)",
                       "host_path": "sge_gen_rmat + sge_csr_from_edges + sge_graph_create (validation, upload)"}}
    print(json.dumps(line), flush=True)


# the 6-vertex patterns of the R-MAT 2^24 configuration with a decomposition
# each in the reference's printed form (global bag last): the own vertex of
# every other bag is a tail level of the imported plan
BAG_PATTERNS = {
    "two_triangles_4cycle": ((6, [(0, 1), (0, 2), (1, 2), (3, 4), (3, 5), (4, 5), (1, 3), (2, 4)]),
                             "num bags: 5\n1,0,2\n3,1,2\n3,4,2\n3,4,5\n3,4,1,2\n"),
    "c6_two_chords": ((6, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (0, 5), (0, 3), (1, 4)]),
                      "num bags: 3\n1,2,3\n4,5,0\n0,1,3,4\n"),
}


def run_bags(args):
    """The bag-relation join against the DFS leaf: per pattern, the imported
    decomposition (sge_plan_from_order_text, inclusion-exclusion leaf) counted
    with its tail levels reading the bags' tries (sge_bags_create +
    sge_plan_use_bags) and without (intersections of adjacency lists), on an
    R-MAT with 2^scale vertices and 16·2^scale edges (a=.57 b=.19 c=.19,
    seed 4).  Both must give the same counts; the relation build (count,
    enumerate, sort, trie) is timed separately from the counting launches."""
    import sge
    scale = args.bag_scale
    eng = sge.Engine.rmat_device(scale, 16 << scale, seed=4)
    rows = []
    opts = dict(root_stride=args.bag_stride, root_offset=0)
    for name, ((k, edges), text) in BAG_PATTERNS.items():
        p = sge.PatternGraph.from_edges(k, edges)
        imp, nb = sge.plan_from_reference(p, text, eng, iep=True)
        # the imported order with its longest tail, so every bag's own vertex is
        # a tail level (the cost model may enumerate one instead)
        cands = sge.candidates(p, eng.graph.stats(), cap=64, force_order=list(imp.order[:k]))
        b = max(cands, key=lambda x: x.tail_len)
        b.count_multiplier, b.single_bag, b.choose_wrap = imp.count_multiplier, imp.single_bag, 1
        t0 = time.perf_counter()
        try:
            bags = eng.bags(p, text, max_rows=args.bag_max_rows)
        except sge.SgeError as e:
            rows.append({"pattern": name, "bags": nb, "relation": f"not built: {e}"})
            continue
        build_s = time.perf_counter() - t0
        info = bags.info()
        res = {}
        for arm, bg in (("dfs", None), ("trie", bags)):
            ms = []
            try:
                for i in range(args.warmup + args.steps):
                    c, _, st = eng.count([b], bags=[bg], time_budget_s=args.bag_budget_s, **opts)
                    if i >= args.warmup:
                        ms.append(st["kernel_ms"])
            except sge.SgeError as e:
                res[arm] = (None, None, str(e))
                continue
            res[arm] = (c[0], statistics.median(ms), st.get("bag_levels", [0])[0])
        if res["dfs"][0] is None or res["trie"][0] is None:
            rows.append({"pattern": name, "bags": nb, "dfs": res["dfs"], "trie": res["trie"],
                         "relation_build_s": round(build_s, 3)})
            bags.close()
            continue
        assert res["dfs"][0] == res["trie"][0], (name, res)
        rows.append({"pattern": name, "bags": nb, "order": list(b.order[:k]), "tail_len": b.tail_len,
                     "count": res["dfs"][0], "trie_levels": res["trie"][2],
                     "relations": info["relations"], "relation_rows": info["rows"],
                     "relation_bytes": info["device_bytes"], "relation_build_s": round(build_s, 3),
                     "dfs_kernel_ms": res["dfs"][1], "trie_kernel_ms": res["trie"][1],
                     "speedup_kernel": res["dfs"][1] / res["trie"][1] if res["trie"][1] else None,
                     "speedup_incl_build": res["dfs"][1] / (res["trie"][1] + 1e3 * build_s)})
        bags.close()
    eng.close()
    line = {"metric": "bag-relation trie join vs DFS leaf, kernel ms per count (same counts)",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic", "dtype": "u32 ids",
            "config": {"workload": f"rmat_s{scale} bags", "graph": dict(scale=scale, m=16 << scale, a=0.57, b=0.19,
                                                                       c=0.19, seed=4, generator="rmat"),
                       "root_sample": f"undirected root edges e = 0 mod {args.bag_stride}",
                       "plan": "the imported decomposition's order with its longest tail"},
            "rows": rows}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="sge", choices=["sge", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="rmat22", choices=["rmat22", "chunglu7100", "ingest", "bags"])
    ap.add_argument("--plans", default="", help="chunglu7100: comma-separated subset, e.g. house/wcoj-u")
    ap.add_argument("--per-plan", action="store_true", help="chunglu7100: time each plan alone")
    ap.add_argument("--scale", type=int, default=RMAT22["scale"],
                    help="rmat22: R-MAT scale (edges 16·2^scale below 22); smaller cases for profiling captures")
    ap.add_argument("--patterns", type=int, default=N_PATTERNS, help="rmat22: the first N of the 78 patterns")
    ap.add_argument("--max-level-capacity", type=int, default=0,
                    help="rmat22: per-level list capacity (0 = max degree; smaller values bound device memory "
                         "for profiling captures; a list past it fails loudly)")
    ap.add_argument("--bag-scale", type=int, default=16, help="bags: R-MAT scale (16·2^scale edges)")
    ap.add_argument("--bag-stride", type=int, default=64, help="bags: root sample stride (1 = every root)")
    ap.add_argument("--bag-budget-s", type=float, default=60.0, help="bags: time budget of one count")
    ap.add_argument("--bag-max-rows", type=int, default=4_000_000_000, help="bags: tuples per relation at most")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ingest":
        return run_ingest(args)
    if args.workload == "chunglu7100":
        return run_chunglu(args)
    if args.workload == "bags":
        return run_bags(args)
    return run_rmat22(args)


if __name__ == "__main__":
    main()
