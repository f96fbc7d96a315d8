"""Benchmark: BC edge-insertion updates/s at K roots (plus p50/p99 latency)
on one GB300, against the plain one-insertion-at-a-time GPU path and the
reference CPU path.

Default workload (--workload rmat20): R-MAT scale 20 (1,048,576 vertices,
edge factor 16, a/b/c/d = .57/.19/.19/.05), symmetrised and deduplicated,
seed 3; K = 1024 uniformly sampled roots; insertions drawn by the same R-MAT
process and filtered to new edges.  A step is one batch of B insertions
applied to all K roots (append + classify/cull + persistent update + seal).

Printed JSON line keys (rank 0): metric/value/unit (whole-job updates/s with
insertions resident in HBM), e2e (same metric through the host C-ABI with
host buffers: H2D of the batch and D2H of the BC vector every step), roofline
of the dominant kernel (k_update, HBM-bound), cpu_baseline (the oracle port
on a bounded sample, scaled to K roots), clocks sampled during the timed
region, gpu_launches, plain_gpu (one insertion per call), latency_ms.

--impl reference times the reference algorithm on the host instead (the
oracle port, all host threads) and prints the same metric.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BC edge-insertion updates/s at K roots"
UNIT = "insertions/s"


def roster_launches(nk: int) -> int:
    """Roster compactions per batch of a forest of nk roots: one, unless the
    library left rosters out (it allocates them only while they take at most
    1 GB: nk x 16 levels x 256 members x 4 B)."""
    return 1 if nk * 16 * 256 * 4 <= (1 << 30) else 0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["rmat20", "rmat18", "rmat16", "chunglu40k", "er1024", "rmat_group64",
                                          "serve16", "serve_rmat20"], default="rmat20")
    p.add_argument("--served-rate", type=float, default=4000.0,
                   help="rmat20 served form: offered insertions/s (Poisson)")
    p.add_argument("--served-requests", type=int, default=16384, help="rmat20 served form: timed requests")
    p.add_argument("--no-served", action="store_true", help="rmat20: skip the served form")
    p.add_argument("--serve-rate", type=float, default=50000.0, help="serve16: offered insertions/s")
    p.add_argument("--serve-requests", type=int, default=10000, help="serve16: timed requests")
    p.add_argument("--serve-max-batch", type=int, default=1024)
    p.add_argument("--serve-budget-gb", type=float, default=150.0)
    p.add_argument("--plain-requests", type=int, default=10000, help="serve16: requests on the plain path")
    p.add_argument("--batch", type=int, default=0,
                   help="insertions per batch (0: 256 on rmat20, whose config fixes none; 64 elsewhere)")
    p.add_argument("--group-batch", type=int, default=16,
                   help="rmat_group64: insertions per graph per step (64 graphs per step)")
    p.add_argument("--plain", type=int, default=128, help="insertions timed on the plain one-at-a-time path")
    p.add_argument("--cpu-insertions", type=int, default=32,
                   help="CPU baseline: insertions timed over all K roots with every host thread")
    p.add_argument("--cpu-insertions-nt1", type=int, default=2,
                   help="CPU baseline: the next insertions timed with one thread (the reference's NT = 1)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--variant", type=int, default=-1,
                   help="update-kernel launch shape (-1 = autotuned on the first warm-up batch)")
    p.add_argument("--workers", type=int, default=0, help="persistent workers (0 = automatic)")
    p.add_argument("--train-insertions", type=int, default=-1,
                   help="cost model: insertions whose per-job costs are logged for training "
                        "(-1 = 16384 on rmat20, else 0 = static schedule)")
    p.add_argument("--train-epochs", type=int, default=4)
    p.add_argument("--deletions", type=int, default=33, help="edge deletions timed after the insertion passes")
    p.add_argument("--compare-batches", type=int, default=8,
                   help="batches timed under both schedules after training")
    p.add_argument("--roots", type=int, default=0,
                   help="use only the first N roots of the workload (profiling captures; 0 = all)")
    return p.parse_args()


def workload_desc(name, g, roots):
    if name == "rmat20":
        return (f"rmat20: R-MAT scale 20, edge factor 16, a/b/c/d .57/.19/.19/.05, seed 3, symmetrised+deduplicated "
                f"({g.nv} vertices, {g.ne} edges); K={len(roots)} uniform roots; R-MAT-drawn new-edge insertions")
    if name in ("rmat16", "rmat18"):
        return (f"{name}: R-MAT scale {name[4:]}, edge factor 16, seed 3 ({g.nv} vertices, {g.ne} edges); "
                f"K={len(roots)} uniform roots; R-MAT-drawn new-edge insertions")
    if name == "chunglu40k":
        return (f"chunglu40k: Chung-Lu n=40000, gamma 2.5, degrees [1,300], seed 2, LCC ({g.nv} vertices, {g.ne} "
                f"edges); K={len(roots)}; insertions 70% at BFS distance <= 3")
    return f"er1024: ER G(1024, 8192) seed 1, exact K=1024; uniform non-edge insertions"


def load_workload(name, count):
    from streamingbc_gb300 import graphs as G
    if name == "rmat20":
        g = G.rmat(20, 16, seed=3)
        return g, G.pick_roots(g.nv, 1024, 3), G.rmat_insertions(g, 20, count, seed=3)
    if name == "rmat16":
        g = G.rmat(16, 16, seed=3)
        return g, G.pick_roots(g.nv, 256, 3), G.rmat_insertions(g, 16, count, seed=3)
    if name == "rmat18":
        g = G.rmat(18, 16, seed=3)
        return g, G.pick_roots(g.nv, 512, 3), G.rmat_insertions(g, 18, count, seed=3)
    if name == "chunglu40k":
        g = G.chung_lu(40000, 176000, 2.5, 1.0, 300.0, seed=2)
        return g, G.pick_roots(g.nv, 256, 2), G.local_insertions(g, max(count, 4096), seed=2)[:count]
    g = G.er(1024, 8192, seed=1)
    return g, G.pick_roots(g.nv, g.nv, 1), G.uniform_insertions(g, count, seed=1)


def kernel_source_hash() -> str:
    """sha256 (first 16 hex digits) of the CUDA sources and headers the
    library is built from: a committed DRAM-traffic capture counts only for
    the kernel sources it was taken with."""
    import glob
    import hashlib
    h = hashlib.sha256()
    csrc = os.path.join(ROOT, "streamingbc_gb300", "csrc")
    for path in sorted(glob.glob(os.path.join(csrc, "*.cu")) + glob.glob(os.path.join(csrc, "*.cuh")) +
                       glob.glob(os.path.join(csrc, "*.h"))):
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def traffic_estimate(workload, batch, alg_bytes_per_launch, roots=None, workers=None):
    """DRAM bytes per k_update launch from an ncu capture of the same case.
    profiles/k_update_traffic.json lists captures (dram__bytes_read.sum +
    dram__bytes_write.sum of one launch, that launch's algorithmic bytes, the
    hash of the kernel sources it ran and the case -- workload, roots, workers,
    batch -- it measured); the DRAM/algorithmic ratio of the capture of this
    case is applied to this run's algorithmic bytes.  No capture of this case,
    or one of other kernel sources, gives null."""
    path = os.path.join(ROOT, "profiles", "k_update_traffic.json")
    try:
        with open(path) as fh:
            caps = json.load(fh)["captures"]
    except (OSError, ValueError, KeyError):
        return None, "no capture file"
    case = f"{workload}/{roots} roots/{workers} workers/batch {batch}"
    cap = next((c for c in caps if case in c.get("applies_to", [])), None)
    if cap is None:
        return None, f"no ncu capture of this case ({case}); profiles/k_update_traffic.json lists the captured ones"
    if cap.get("source_hash") != kernel_source_hash():
        return None, (f"capture ({cap.get('case')}) was taken with other kernel sources ({cap.get('source_hash')}); "
                      f"not used")
    ratio = float(cap["dram_bytes_per_launch"]) / float(cap["alg_bytes_per_launch"])
    return ratio * alg_bytes_per_launch, (f"small-case ncu capture ({cap.get('case')}): DRAM/algorithmic bytes "
                                          f"{ratio:.3f}, applied to this run's algorithmic bytes; kernel sources "
                                          f"{cap['source_hash']}")


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value: float, world: int) -> float:
    """Max over ranks (replicas); a no-op on one process."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def host_avail_bytes() -> int:
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_AVPHYS_PAGES")
    except (ValueError, OSError):
        return 8 << 30


def cpu_port_time(g, roots, ins, n_all, n_one, threads):
    """The oracle port -- the reference's COARSE algorithm in C, OpenMP over
    roots -- over ALL K roots, no extrapolation: static init, then the first
    n_all insertions of the stream with every host thread, then the next
    n_one with one thread (the reference's NT = 1).  Each insertion is timed
    like updateEdgeNEW (src/sbcMain_utils.c:568-571): the per-root updates and
    the per-thread BC reduce, not the graph insert.  When the K x V forest
    (24 B per cell) does not fit half the free host memory, roots run in
    chunks (each chunk a fresh oracle on the same graph and stream): an
    insertion's time is then the sum of its per-root phase over the chunks
    plus the BC reduce once."""
    from oracle import oracle as orc
    orc.build()
    K = len(roots)
    cell = 24 * g.nv
    chunk = K
    while chunk > 1 and chunk * cell * 1.25 > host_avail_bytes() // 2:
        chunk = (chunk + 1) // 2
    t_all = np.zeros(n_all)
    t_one = np.zeros(n_one)
    static_s = 0.0
    for c in range(0, K, chunk):
        o = orc.PortOracle(g.nv, g.off, g.adj, roots[c:c + chunk], nthreads=threads)
        static_s += o.static_timed()
        for i, (u, v) in enumerate(ins[:n_all]):
            tr, tb = o.insert_timed(int(u), int(v))
            t_all[i] += tr + (tb if c == 0 else 0.0)
        o.set_threads(1)
        for i, (u, v) in enumerate(ins[n_all:n_all + n_one]):
            tr, tb = o.insert_timed(int(u), int(v))
            t_one[i] += tr + (tb if c == 0 else 0.0)
        o.close()
    return {"t_all": t_all, "t_one": t_one, "static_s": static_s, "chunk": chunk}


def _lat(ts) -> dict:
    return {"mean": float(np.mean(ts)) * 1e3, "p50": float(np.percentile(ts, 50)) * 1e3,
            "p99": float(np.percentile(ts, 99)) * 1e3}


def cpu_sample(g, roots, ins, n_all, n_one, threads):
    """CPU baseline of one forest: the oracle port over all K roots on the
    first n_all insertions of the stream (all host threads) and the next
    n_one (one thread)."""
    r = cpu_port_time(g, roots, ins, n_all, n_one, threads)
    out = {"value": 1.0 / float(np.mean(r["t_all"])), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"all {len(roots)} roots (no extrapolation), insertions 1..{n_all} of the stream after static "
                     f"init, {threads} threads; then insertions {n_all + 1}..{n_all + n_one} with 1 thread; "
                     f"timed like updateEdgeNEW (per-root updates + BC reduce, graph insert excluded)"
                     + (f"; roots in chunks of {r['chunk']} to fit host memory" if r["chunk"] < len(roots) else ""),
           "per_insertion_ms": _lat(r["t_all"]),
           "static_init_s": r["static_s"]}
    if n_one:
        out["nt1"] = {"value": 1.0 / float(np.mean(r["t_one"])), "unit": UNIT, "cores": 1,
                      "insertions": n_one, "per_insertion_ms": _lat(r["t_one"])}
    return out


GROUP_WORKLOAD = "rmat_group64"
GROUP_DESC = ("rmat_group64: 64 independent R-MAT graphs, scales uniform in 10..16 (drawn with seed 100), edge "
              "factor 8, a/b/c/d .57/.19/.19/.05, seeds 100..163, symmetrised+deduplicated; K=min(|V|,128) uniform "
              "roots each; R-MAT-drawn new-edge insertions, {b} per graph per step, all 64 graphs in one group batch")


def cpu_sample_group(specs, batch, n_ins, threads):
    """Oracle port on every graph of the group, all K roots of each, its
    first n_ins insertions; a group step's CPU time is the sum over graphs of
    batch x that graph's mean per-insertion time."""
    total = 0.0
    per_graph = []
    for g, roots, ins, _ in specs:
        r = cpu_port_time(g, roots, ins, n_ins, 0, threads)
        per_graph.append(float(np.mean(r["t_all"])))
        total += batch * per_graph[-1]
    value = len(specs) * batch / total
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every graph: all K roots (no extrapolation), its first {n_ins} insertions; step = {batch} "
                      f"insertions on each of {len(specs)} graphs",
            "per_graph_insertion_ms_mean": float(np.mean(per_graph)) * 1e3}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.workload == SERVE_WORKLOAD:
        from streamingbc_gb300 import graphs as G
        graphs = serving_set()
        gid, pairs, _ = G.poisson_trace(graphs, args.serve_requests, args.serve_rate, seed=11)
        cpu = cpu_sample_serve(graphs, gid, pairs, max(4, args.warmup + args.steps), threads)
        value = cpu["value"]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": SERVE_DESC.format(rate=args.serve_rate, budget=args.serve_budget_gb,
                                                         mb=args.serve_max_batch),
                           "step": "one insertion applied to all K roots of its graph"},
                "cpu_baseline": cpu,
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.workload == GROUP_WORKLOAD:
        from streamingbc_gb300 import graphs as G
        specs = G.rmat_group(insertions=max(512, args.warmup + args.steps))
        cpu = cpu_sample_group(specs, args.group_batch, max(args.warmup + args.steps, 4), threads)
        value = cpu["value"]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": len(specs) * args.group_batch / value * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": GROUP_DESC.format(b=args.group_batch), "graphs": len(specs)},
                "cpu_baseline": cpu,
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    need = args.warmup + args.steps
    g, roots, ins = load_workload(args.workload, need + args.cpu_insertions_nt1)
    r = cpu_port_time(g, roots, ins, need, args.cpu_insertions_nt1, threads)
    times = r["t_all"][args.warmup:]
    total = float(np.sum(times))
    value = len(times) / total
    cpu = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"all {len(roots)} roots (no extrapolation); step i = insertion i of the stream after static "
                     f"init ({args.warmup} untimed, {args.steps} timed), {threads} threads, timed like updateEdgeNEW "
                     f"(per-root updates + BC reduce)"
                     + (f"; roots in chunks of {r['chunk']} to fit host memory" if r["chunk"] < len(roots) else ""),
           "per_insertion_ms": _lat(times), "static_init_s": r["static_s"]}
    if args.cpu_insertions_nt1:
        cpu["nt1"] = {"value": 1.0 / float(np.mean(r["t_one"])), "unit": UNIT, "cores": 1,
                      "insertions": args.cpu_insertions_nt1, "per_insertion_ms": _lat(r["t_one"])}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_desc(args.workload, g, roots), "roots": int(len(roots)),
                       "batch": 1,
                       "step": "one insertion applied to all K roots (the reference applies insertions one at a time)"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


SERVE_WORKLOAD = "serve16"
SERVE_DESC = ("serve16: 16 Chung-Lu graphs, n log-spaced 1e4..1e6, exponent 2.3, average degree 12, expected "
              "degrees in [1, sqrt(2m)], seeds 200..215, LCC kept; K=512 uniform roots each; requests arrive as a "
              "Poisson process of {rate:g}/s, graph chosen proportional to its edges, uniform non-edge insertions; "
              "HBM admission budget {budget} GB; per-graph continuous batching up to {mb} requests")


def _serve_graph_one(i):
    """Graph i of the serving set (same construction as graphs.serving_graphs)."""
    from streamingbc_gb300 import graphs as G
    n = int(round(1e4 * 100.0 ** (i / 15)))
    m = int(round(12 * n / 2))
    g = G.chung_lu(n, m, 2.3, 1.0, float(np.sqrt(2.0 * m)), seed=200 + i)
    return g, G.pick_roots(g.nv, min(g.nv, 512), seed=200 + i)


def serving_set():
    """The 16 serving graphs, generated in parallel (spawned workers, before
    any CUDA call of this process)."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        return pool.map(_serve_graph_one, range(16))


def cpu_sample_serve(graphs, gid, pairs, n_ins, threads):
    """Oracle port per graph on all K roots and its first n_ins requests;
    the mix's CPU rate weights each graph's per-insertion time by its share
    of the requests."""
    share = np.bincount(gid, minlength=len(graphs)) / len(gid)
    per = []
    for i, (g, roots) in enumerate(graphs):
        mine = pairs[gid == i][:n_ins]
        if not len(mine):
            per.append(0.0)
            continue
        r = cpu_port_time(g, roots, mine, len(mine), 0, threads)
        per.append(float(np.mean(r["t_all"])))
    t_mix = float(np.dot(share, per))
    return {"value": 1.0 / t_mix, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every graph: all K roots (no extrapolation), first {n_ins} of its requests; mix weighted by "
                      f"request share"}


def run_serve(args):
    """Serving loop over 16 resident graphs: a Poisson trace played in real
    time into the batched server, then a prefix of it into the plain server
    (one request per batch)."""
    rank, world, local = dist_env()
    t0 = time.time()
    graphs = serving_set()
    gen_s = time.time() - t0
    import torch
    from streamingbc_gb300 import build as b
    from streamingbc_gb300 import graphs as G
    from streamingbc_gb300 import native
    if not os.path.exists(native.LIB_PATH):
        b.build()
    lib = native.load()
    lib.sbc_set_device(local if world > 1 else 0)
    torch.cuda.set_device(local if world > 1 else 0)
    rate = args.serve_rate
    n_warm = 200 * max(args.warmup, 1)
    n_req = args.serve_requests
    gid, pairs, t = G.poisson_trace(graphs, n_warm + n_req + args.plain_requests, rate, seed=11)
    budget = int(args.serve_budget_gb * (1 << 30))

    def serve(max_batch, lo, hi, warm_hi, max_inflight=0):
        srv = native.DeviceServer(budget_bytes=budget, max_batch=max_batch, max_inflight=max_inflight)
        ids = [srv.add_graph(g, roots) for g, roots in graphs]
        t1 = time.time()
        srv.drain()  # admission + static init of every graph that fits
        admit_s = time.time() - t1
        if warm_hi > lo:
            srv.play(gid[lo:warm_hi], pairs[lo:warm_hi], t[lo:warm_hi] - t[lo])
            srv.drain()
            srv.stats(reset=True)
        clk = ClockSampler(local)
        clk.start()
        t1 = time.perf_counter()
        srv.play(gid[warm_hi:hi], pairs[warm_hi:hi], t[warm_hi:hi] - t[warm_hi])
        srv.drain()
        wall = time.perf_counter() - t1
        clocks = clk.stop()
        st = srv.stats()
        info = [srv.graph_info(i) for i in ids]
        srv.close()
        return st, wall, admit_s, clocks, info

    st, wall, admit_s, clocks, info = serve(args.serve_max_batch, 0, n_warm + n_req, n_warm)
    plain = None
    if args.plain_requests:
        lo = n_warm + n_req
        pst, pwall, _, _, _ = serve(1, lo, lo + args.plain_requests, lo, max_inflight=1)
        plain = {"value": pst["throughput"], "unit": UNIT, "requests": args.plain_requests,
                 "p50_ms": pst["p50_us"] / 1e3, "p99_ms": pst["p99_us"] / 1e3, "wall_s": pwall,
                 "note": "same graphs, arrival process and rate; one insertion at a time over all graphs "
                         "(max_batch 1, one batch in flight): the unbatched plain GPU path"}
        cst, cwall, _, _, _ = serve(1, lo, lo + args.plain_requests, lo)
        plain["concurrent_graphs"] = {"value": cst["throughput"], "p50_ms": cst["p50_us"] / 1e3,
                                      "p99_ms": cst["p99_us"] / 1e3,
                                      "note": "one insertion per batch, but graphs overlap on the device"}
    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = cpu_sample_serve(graphs, gid[n_warm:n_warm + n_req], pairs[n_warm:n_warm + n_req], 4,
                               os.cpu_count() or 1)
    if rank == 0:
        value = st["throughput"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": int(st["batches"]),
            "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(st["batches"], 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64+f64", "data": "synthetic",
            "config": {"workload": SERVE_DESC.format(rate=rate, budget=args.serve_budget_gb, mb=args.serve_max_batch),
                       "graphs": len(graphs), "vertices": sum(g.nv for g, _ in graphs),
                       "requests": n_req, "warmup_requests": n_warm, "offered_rate": rate,
                       "admitted": sum(1 for x in info if x["state"] == "admitted"),
                       "bytes_admitted": st["bytes_admitted"], "admission_s": admit_s, "generate_s": gen_s,
                       "step": "one launched per-graph batch",
                       "timing": "arrival (scheduled trace time) to batch completion (stream callback); value = "
                                 "completed / (last completion - first arrival)"},
            "latency_ms": {"p50": st["p50_us"] / 1e3, "p99": st["p99_us"] / 1e3, "mean": st["mean_us"] / 1e3,
                           "max": st["max_us"] / 1e3},
            "mean_batch": st["mean_batch"],
            "per_graph_batches": [x["batches"] for x in info],
            "roofline": None,
            "cpu_baseline": cpu,
            "e2e": {"value": st["completed"] / wall, "unit": UNIT, "h2d_bytes_per_step": 24 * st["mean_batch"],
                    "d2h_bytes_per_step": 0, "note": "host requests in, results resident on the device; wall time "
                                                      "of play + drain"},
            "clocks": clocks,
            # append, classify, update, roster compaction, seal per batch
            "gpu_launches": int(st["batches"]) * (4 + roster_launches(512)),
            "plain_gpu": plain,
            "batched_over_plain": value / plain["value"] if plain and plain["value"] else None,
        }
        print(json.dumps(line), flush=True)


def serve_one(g, roots, reqs, rate, n_warm, n_req, n_plain, max_batch, train, budget, local):
    """One graph through the serving loop: requests arrive as a Poisson
    process of `rate`/s.  Batched form: launch shape tuned on the first batch,
    cost model trained on the costs of the first `train` insertions, then the
    model's schedule; the first n_warm requests (tuning, logging, training)
    are untimed, the next n_req timed.  Plain form: a fresh server applying
    one request at a time (max_batch 1, one batch in flight), n_plain
    requests offered at the same rate."""
    from streamingbc_gb300 import native
    rng = np.random.default_rng(23)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_warm + n_req + n_plain))
    gid = np.zeros(len(t), dtype=np.int32)

    def run(mb, lo, warm_hi, hi, inflight, tune, tr):
        srv = native.DeviceServer(budget_bytes=budget, max_batch=mb, max_inflight=inflight, autotune=tune,
                                  train_insertions=tr)
        srv.add_graph(g, roots)
        srv.drain()
        if warm_hi > lo:
            srv.play(gid[lo:warm_hi], reqs[lo:warm_hi], t[lo:warm_hi] - t[lo])
            srv.drain()
            srv.stats(reset=True)
        clk = ClockSampler(local)
        clk.start()
        t1 = time.perf_counter()
        srv.play(gid[warm_hi:hi], reqs[warm_hi:hi], t[warm_hi:hi] - t[warm_hi])
        srv.drain()
        wall = time.perf_counter() - t1
        clocks = clk.stop()
        st = srv.stats()
        srv.close()
        return st, wall, clocks

    st, wall, clocks = run(max_batch, 0, n_warm, n_warm + n_req, 0, True, train)
    out = {"value": st["throughput"], "unit": UNIT, "offered_rate": rate, "requests": n_req,
           "latency_ms": {"p50": st["p50_us"] / 1e3, "p99": st["p99_us"] / 1e3, "mean": st["mean_us"] / 1e3,
                          "max": st["max_us"] / 1e3},
           "mean_batch": st["mean_batch"], "batches": st["batches"], "wall_s": wall, "clocks": clocks,
           "how": f"sbc_server, one resident graph; first {n_warm} requests untimed (launch shape tuned on the first "
                  f"batch, per-job costs of {train} insertions logged, cost model trained, model schedule after); "
                  f"throughput = completed / (last completion - first arrival); latency = arrival to batch "
                  f"completion"}
    if n_plain:
        lo = n_warm + n_req
        pst, pwall, _ = run(1, lo, lo, lo + n_plain, 1, True, 0)
        out["plain"] = {"value": pst["throughput"], "unit": UNIT, "requests": n_plain,
                        "latency_ms": {"p50": pst["p50_us"] / 1e3, "p99": pst["p99_us"] / 1e3},
                        "how": "same server and arrival process, one request per batch and one batch in flight: the "
                               "unbatched plain GPU path (overloaded at this rate: latency is queueing)"}
        out["served_over_plain"] = out["value"] / pst["throughput"] if pst["throughput"] else None
    return out


def run_group(args):
    """64 R-MAT graphs updated together: one group batch (append, classify,
    update, seal over all graphs) per step."""
    rank, world, local = dist_env()
    import torch
    from streamingbc_gb300 import build as b
    from streamingbc_gb300 import graphs as G
    from streamingbc_gb300 import native
    if not os.path.exists(native.LIB_PATH):
        b.build()
    lib = native.load()
    lib.sbc_set_device(local if world > 1 else 0)
    torch.cuda.set_device(local if world > 1 else 0)
    B = args.group_batch
    n_val = (args.warmup + args.steps) * B
    n_e2e = 0 if args.no_e2e else (1 + args.steps) * B
    t0 = time.time()
    specs = G.rmat_group(insertions=max(512, n_val + n_e2e))
    gen_s = time.time() - t0
    objs = []
    t0 = time.time()
    for g, roots, ins, _ in specs:
        dg = native.DeviceGraph(g.nv, g.off, g.adj)
        f = native.DeviceForest(dg, roots, workers=1)
        dg.reserve(ins[:n_val + n_e2e])
        f.static_init()
        objs.append((dg, f))
    for _, f in objs:
        f.sync()
    static_s = time.time() - t0
    grp = native.DeviceGroup([f for _, f in objs], variant=args.variant)

    def batches(s):
        return [ins[s * B:(s + 1) * B] for _, _, ins, _ in specs]

    tuned = None
    w0 = 0
    if args.variant < 0 and args.warmup > 0:
        chosen, tms = grp.autotune(batches(0), reps=2)
        tuned = {"chosen": chosen, "ms_per_shape": [round(float(x), 3) for x in tms]}
        w0 = 1
    for s in range(w0, args.warmup):
        grp.insert(batches(s))
    grp.counters()
    clk = ClockSampler(local)
    clk.start()
    torch.cuda.synchronize()
    dev_ms = []
    t_wall = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        dev_ms.append(grp.insert(batches(s)))
    wall_ms = (time.perf_counter() - t_wall) * 1e3
    clocks = clk.stop()
    cnt = grp.counters()
    n_step = B * len(specs)
    total_ms = float(np.sum(dev_ms))
    value = args.steps * n_step / (total_ms / 1e3)
    K = sum(len(r) for _, r, _, _ in specs)
    alg_bytes = 8 * cnt["scanned"] + 40 * cnt["vertices"] + 16 * K * B * args.steps
    achieved = alg_bytes / (total_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()

    e2e = None
    if n_e2e:
        base = n_val // B
        grp.insert(batches(base))
        grp.bc()
        lat = []
        t1 = time.perf_counter()
        for s in range(base + 1, base + 1 + args.steps):
            ts = time.perf_counter()
            grp.insert(batches(s))
            grp.bc()  # every member's BC vector, one wait
            lat.append((time.perf_counter() - ts) * 1e3)
        e2e_s = time.perf_counter() - t1
        nv_sum = sum(g.nv for g, _, _, _ in specs)
        e2e = {"value": args.steps * n_step / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 4 * n_step,
               "d2h_bytes_per_step": 8 * nv_sum + 4 * len(specs),
               "p50_step_ms": float(np.percentile(lat, 50)), "p99_step_ms": float(np.percentile(lat, 99))}
    # per-graph correctness, outside the timed region: every member against
    # a static recompute (fresh graph + forest, same roots) of its graph with
    # the insertions applied so far -- incremental must equal static exactly
    n_applied = (args.warmup + args.steps) * B + ((1 + args.steps) * B if n_e2e else 0)
    all_bc = grp.bc()
    passed = 0
    for i, ((g, roots, ins, _), (_, f)) in enumerate(zip(specs, objs)):
        g2 = G.insert_edges(g, ins[:n_applied])
        dg2 = native.DeviceGraph(g2.nv, g2.off, g2.adj)
        f2 = native.DeviceForest(dg2, roots, workers=1)
        f2.static_init()
        d2 = f2.dist()
        reach = d2 != np.iinfo(np.int32).max
        ok = (np.array_equal(f.dist(), d2) and np.array_equal(f.sigma()[reach], f2.sigma()[reach]) and
              float(np.max(np.abs(all_bc[i] - f2.bc()) / np.maximum(np.abs(f2.bc()), 1.0))) <= 1e-9)
        passed += int(ok)
        f2.close()
        dg2.close()
    check = {"graphs": len(specs), "passed": passed, "insertions_per_graph": n_applied,
             "how": "after the timed and e2e steps: each member's dist (all vertices), sigma (reachable) and BC "
                    "(1e-9 relative) against a static init of its updated graph on the same roots; the static "
                    "init is pinned to the reference by the test suite"}
    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = cpu_sample_group(specs, B, args.cpu_insertions // 2 or 4, os.cpu_count() or 1)
    info = grp.info()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64+f64", "data": "synthetic",
            "config": {"workload": GROUP_DESC.format(b=B), "graphs": len(specs), "roots": K,
                       "vertices": sum(g.nv for g, _, _, _ in specs), "batch_per_graph": B,
                       "parallelism": "single GPU", "variant": info["variant"], "workers": info["workers"],
                       "autotune": tuned, "static_init_s": static_s, "generate_s": gen_s,
                       "l2": "per-root state of all graphs on device; no flush (inputs change every step)",
                       "timing": "CUDA events on the group stream around each batch's append..seal launches"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                         "kernel": "k_update_group (whole batch sequence timed)",
                         "alg_bytes_per_launch": alg_bytes / args.steps,
                         "avg_launch_ms": total_ms / args.steps},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clocks,
            # append, classify, update, seal per group batch, and a roster compaction per member
            "gpu_launches": (4 + sum(roster_launches(len(r)) for _, r, _, _ in specs)) * args.steps,
            "latency_ms": {"batch_p50": float(np.percentile(dev_ms, 50)), "wall_ms_timed": wall_ms},
            "work": {"traversed_vertices": cnt["vertices"], "traversed_edges": cnt["edges"],
                     "scanned_slots": cnt["scanned"], "case1_pairs": cnt["case1"], "case2_pairs": cnt["case2"],
                     "insertions": args.steps * n_step},
            "per_graph_check": check,
        }
        print(json.dumps(line), flush=True)
    grp.close()
    for dg, f in objs:
        f.close()
        dg.close()


def run_ours(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from streamingbc_gb300 import build as b
    from streamingbc_gb300 import native
    if not os.path.exists(native.LIB_PATH):
        b.build()
    lib = native.load()
    lib.sbc_set_device(local if world > 1 else 0)

    B = args.batch or (256 if args.workload == "rmat20" else 64)
    # warm-up, the timed `value` pass, then a second pass with per-launch events for the roofline
    n_dev = (args.warmup + 2 * args.steps) * B
    n_e2e = 0 if args.no_e2e else (1 + args.steps) * B
    n_plain = args.plain
    # cost model: log per-job costs over the first `train` insertions, train,
    # then time `compare` batches under both schedules (paired, on copies)
    train = args.train_insertions if args.train_insertions >= 0 else (16384 if args.workload == "rmat20" else 0)
    n_cmp = args.compare_batches * B if train > 0 else 0
    n_pre = train + n_cmp
    t0 = time.time()
    n_served = 0 if (args.workload != "rmat20" or args.no_served) else 16384 + 2 * B + args.served_requests + 2048
    g, roots, ins_all = load_workload(args.workload, max(n_pre + n_dev + n_e2e + n_plain, n_served))
    if args.roots:
        roots = roots[:args.roots]
    if world > 1:
        # weak scaling by roots: K roots per rank out of K * world uniform roots,
        # the graph and the insertion stream replicated on every rank
        from streamingbc_gb300 import graphs as G
        from streamingbc_gb300.sharding import shard_roots
        k_rank = len(roots)
        all_roots = G.pick_roots(g.nv, min(g.nv, k_rank * world), seed=3)
        roots = shard_roots(all_roots, rank, world)
    gen_s = time.time() - t0
    t0 = time.time()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    build_s = time.time() - t0
    f = native.DeviceForest(dg, roots, workers=args.workers, variant=args.variant)
    dg.reserve(ins_all)  # slack for every insertion of the run, planned before timing

    t0 = time.time()
    f.static_init()
    static_s = time.time() - t0
    f.counters()

    model_info = None
    if train > 0:
        K0 = len(roots)
        pre = torch.tensor(ins_all[:train], dtype=torch.int32, device="cuda")
        p_u, p_v = pre[:, 0].contiguous(), pre[:, 1].contiguous()
        f.cost_log_start(min(train * K0, 1 << 26))
        t0 = time.time()
        for s in range(0, train - B + 1, B):
            f.insert_device(B, p_u[s:].data_ptr(), p_v[s:].data_ptr())
        f.sync()
        log_s = time.time() - t0
        samples = f.cost_log_stop()
        tstats = f.train_cost_model(epochs=args.train_epochs, batch=4096, lr=2e-3, val_frac=0.1, seed=1)
        f.set_schedule(native.DeviceForest.SCHED_MODEL)
        ms_s = ms_m = 0.0
        for s in range(train, train + n_cmp, B):
            a, b_ = f.compare_schedules(ins_all[s:s + B], reps=1)
            ms_s += a
            ms_m += b_
        f.counters()
        model_info = {"train_insertions": train, "logged_samples": samples, "logging_s": log_s,
                      "train": {k: tstats[k] for k in ("train_samples", "val_samples", "epochs", "steps",
                                                      "train_ms", "val_mae", "val_rmse", "val_mae_mean")},
                      "target": "log(1 + touched vertices) per (insertion, root) job",
                      "schedule_compare": {"batches": args.compare_batches, "static_ms": ms_s, "model_ms": ms_m,
                                           "static_over_model": ms_s / ms_m if ms_m > 0 else None,
                                           "note": "same batches, each timed under both schedules on copies of "
                                                   "the state (classify/ordering + update)"},
                      "schedule": "model"}
    ins = ins_all[n_pre:]

    # ---------------- device-resident batches (value) ----------------
    d_ins = torch.tensor(ins[:n_dev], dtype=torch.int32, device="cuda")
    d_u = d_ins[:, 0].contiguous()
    d_v = d_ins[:, 1].contiguous()
    torch.cuda.synchronize()
    # the first warm-up batch goes through the launch-shape autotuner (it
    # applies the batch once, after timing its update under every shape that
    # fits on copies of the state), unless a shape was forced
    tuned = None
    w0 = 0
    if args.variant < 0 and args.warmup > 0:
        chosen, tms = f.autotune(ins[:B], reps=2)
        tuned = {"chosen": chosen, "ms_per_shape": [round(float(x), 3) for x in tms]}
        w0 = 1
    for s in range(w0, args.warmup):
        f.insert_device(B, d_u[s * B:].data_ptr(), d_v[s * B:].data_ptr())
    f.sync()
    f.counters()
    # value pass: each batch replays a captured CUDA graph; CUDA events on the
    # library's stream bracket the K batches
    clk = ClockSampler(local)
    clk.start()
    barrier(world)
    torch.cuda.synchronize()
    f.timer_start()
    t_wall = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        f.insert_device(B, d_u[s * B:].data_ptr(), d_v[s * B:].data_ptr())
    total_ms = f.timer_stop()
    wall_ms = (time.perf_counter() - t_wall) * 1e3
    barrier(world)
    clocks = clk.stop()
    cnt_value = f.counters()
    total_ms = barrier_max(total_ms, world)
    n_timed = args.steps * B
    value = n_timed * world / (total_ms / 1e3)

    # roofline pass: the next K batches launched directly with CUDA events
    # around every kernel (graph replay is off while profiling)
    f.reset_profile()
    f.set_profiling(True)
    for s in range(args.warmup + args.steps, args.warmup + 2 * args.steps):
        f.insert_device(B, d_u[s * B:].data_ptr(), d_v[s * B:].data_ptr())
    f.sync()
    f.set_profiling(False)
    prof = f.profile()
    cnt = f.counters()

    # per-batch latency: profiled batch events give each step's device time
    batch_ms = prof["batch_ms"] / max(prof["batches"], 1)

    # Algorithmic bytes of the timed region: 8 B per adjacency slot the kernel
    # scans (neighbour id + neighbour distance), 40 B per traversed vertex
    # (state read + write) and 16 B per (root, insertion) for classification.
    # `alg_bytes_ref` applies the same figures to the reference's traversal
    # counters, i.e. to the edges the reference's traversal scans.
    K = len(roots)
    alg_bytes = 8 * cnt["scanned"] + 40 * cnt["vertices"] + 16 * K * n_timed
    alg_bytes_ref = 8 * cnt["edges"] + 40 * cnt["vertices"] + 16 * K * n_timed
    upd_launches = max(prof["update_launches"], 1)
    upd_ms = prof["update_ms"] / upd_launches
    achieved = (alg_bytes / upd_launches) / (upd_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic, traffic_note = traffic_estimate(args.workload, B, alg_bytes / upd_launches, len(roots),
                                             f.info()["workers"])

    # ---------------- plain path: one insertion per call ----------------
    plain = None
    if n_plain:
        pl = ins[n_dev + n_e2e:n_dev + n_e2e + n_plain]
        lat = []
        for u, v in pl:
            t1 = time.perf_counter()
            f.insert([(u, v)])
            lat.append((time.perf_counter() - t1) * 1e3)
        plain = {"value": 1e3 / float(np.mean(lat)), "unit": UNIT, "insertions": len(lat),
                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                 "note": "sbc_insert_batch with n=1 per call (append + update + stats, synchronous)"}

    # ---------------- e2e through the host C-ABI ----------------
    e2e = None
    if n_e2e:
        base = n_dev
        bc = np.zeros(g.nv, dtype=np.float64)
        ei = np.ascontiguousarray(ins[base:base + n_e2e])
        f.insert(ei[:B])  # warm-up step of this path
        f.bc()
        barrier(world)
        lat = []
        t1 = time.perf_counter()
        for s in range(1, 1 + args.steps):
            ts = time.perf_counter()
            f.insert(ei[s * B:(s + 1) * B])
            bc = f.bc()
            if world > 1:
                from streamingbc_gb300.sharding import reduce_sum
                bc = reduce_sum(bc)  # partial BC of this rank's roots -> BC over all ranks' roots
            lat.append((time.perf_counter() - ts) * 1e3)
        e2e_s = barrier_max(time.perf_counter() - t1, world)
        e2e = {"value": args.steps * B * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 2 * 4 * B,
               "d2h_bytes_per_step": 8 * g.nv + 4 * B + 4 + 32,
               "p50_step_ms": float(np.percentile(lat, 50)), "p99_step_ms": float(np.percentile(lat, 99))}

    # ---------------- deletions (after everything else: they change the graph) ----------------
    deletions = None
    if args.deletions:
        src = np.repeat(np.arange(g.nv), np.diff(g.off))
        sel = src < g.adj
        E = np.stack([src[sel], g.adj[sel]], axis=1)
        pick = E[np.random.default_rng(17).choice(len(E), args.deletions, replace=False)]
        f.delete(pick[:1])  # warm-up deletion
        t1 = time.perf_counter()
        dst = f.delete(pick[1:])
        del_s = time.perf_counter() - t1
        deletions = {"value": (len(pick) - 1) / del_s, "unit": "deletions/s", "deletions": len(pick) - 1,
                     "removed": dst["inserted"], "keep_parent_pairs": dst["case1"],
                     "lost_parent_pairs": dst["case2"],
                     "note": "sbc_delete_batch, host arrays, synchronous, one call and one update launch: removals "
                             "marked in order, every affected root runs the deletions in order (each job sees the "
                             "graph after its deletion): sigma-only update where the deeper endpoint keeps a parent, "
                             "else the affected vertices move down in place (graphs of >= 32768 vertices) or the "
                             "root is recomputed once on the final graph (smaller graphs, or a move-down over "
                             "max(1024, V/16) vertices)"}

    cpu = None
    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        cpu = cpu_sample(g, roots, ins_all, args.cpu_insertions, args.cpu_insertions_nt1, threads)
        if deletions:
            # a deletion on the CPU port is a recompute of every root
            deletions["cpu_port_recompute_s_per_deletion"] = cpu["static_init_s"]

    info = f.info()
    variant_used = f.variant
    served = None
    if args.workload == "rmat20" and not args.no_served and world == 1:
        f.close()
        dg.close()
        served = serve_one(g, roots, ins_all[:n_served], args.served_rate, 16384 + 2 * B, args.served_requests,
                           2048, args.serve_max_batch, 16384, int(args.serve_budget_gb * (1 << 30)), local)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64+f64", "data": "synthetic",
            "config": {"workload": workload_desc(args.workload, g, roots), "roots": K, "batch": B,
                       "parallelism": (f"roots sharded over {world} GPUs ({K} roots per rank, graph and "
                                       f"insertions replicated, one BC all-reduce per e2e step)")
                                      if world > 1 else "single GPU",
                       "l2": f"per-root state {info['bytes'] / 1e9:.1f} GB on device >> 129 MB L2; no flush",
                       "workers": info["workers"], "variant": variant_used, "autotune": tuned,
                       "static_init_s": static_s,
                       "graph_build_s": build_s,
                       "generate_s": gen_s,
                       "timing": "value: K batches replayed from a captured CUDA graph, CUDA events on the "
                                 "library stream; roofline: the next K batches launched directly with events "
                                 "around every kernel"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_note,
                         "peak_source": peak_kind,
                         "kernel": "k_update", "alg_bytes_per_launch": alg_bytes / upd_launches,
                         "alg_bytes_ref_per_launch": alg_bytes_ref / upd_launches,
                         "frac_ref_equivalent": (alg_bytes_ref / upd_launches) / (upd_ms / 1e3) / 1e9 / peak,
                         "avg_launch_ms": upd_ms},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clocks,
            # set_src, stage, append, classify, update, roster compaction, seal per
            # batch; under the model schedule classify becomes features + 3 ordering kernels
            "gpu_launches": ((9 if model_info else 6) + roster_launches(K)) * args.steps,
            "cost_model": model_info,
            "deletions": deletions,
            "plain_gpu": plain,
            "latency_ms": {"batch_p50": batch_ms, "wall_ms_timed": wall_ms,
                           "per_insertion_in_batch": batch_ms},
            "work": {"traversed_vertices": cnt["vertices"], "traversed_edges": cnt["edges"],
                     "scanned_slots": cnt["scanned"], "case1_pairs": cnt["case1"], "case2_pairs": cnt["case2"],
                     "insertions": n_timed},
            "kernel_ms": {k: prof[k] for k in ("append_ms", "classify_ms", "update_ms", "batch_ms")},
            "served": served,
        }
        print(json.dumps(line), flush=True)
    if served is None:
        f.close()
        dg.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == GROUP_WORKLOAD:
        run_group(args)
    elif args.workload == SERVE_WORKLOAD:
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
