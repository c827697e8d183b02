"""Benchmark: GTEPS and HBM-roofline fraction of the five push algorithms on R-MAT scale 22.

Workload (one "step" = one pass of the hot path over the graph, every algorithm once):
  R-MAT scale 22 (4,194,304 vertices), edge factor 16 (67,108,864 edges), a/b/c/d = .57/.19/.19/.05,
  seed 1, uint32 weights uniform in [1,63], Tigr K = 8 (--k 4|8|16).
    BFS, SSSP, SSWP  sync_push_dd from the highest-out-degree vertex
    CC               async_push_dd (every vertex seeded) on the symmetrised arc set (134M arcs)
    PageRank         sync_push_td (Jacobi pull), d = 0.85, stop at ||x-x*||_1/||x||_1 <= 1e-7
  value = sum over the step of TEPS edges (m_r per traversal, m for CC, sweeps*m for PageRank)
          / device time of the step (CUDA events on the launching stream), whole job over all ranks.
  e2e   = the same metric through the C ABI with host buffers, every step: the directed weighted edge
          list copied in once from page-locked memory, the three virtual graphs (forward, symmetrised
          on the device for CC, transposed for PageRank) built from it on the GPU, results copied back.
Inputs are larger than L2 (the part arrays are ~0.7 GB) and L2 is also flushed (256 MB write)
between timed steps.

The default (one GPU) line also carries `grid`, `batch` and `ppr`: the lines of the other workloads
(--workload grid|batch|ppr) measured after the headline with fewer timed steps -- the 4096^2 road-like
grid against one launch per round, the 256-graph query batch against the plain kernel looped per query
(its wall time and the sum of its kernel times), the 64-column personalised-PageRank adjoint against the
single-column kernels looped per teleport vector -- and `stream`: BFS/SSSP/SSWP on the headline graph held in
host memory and streamed through device buffers of a quarter of its parts (eeg_stream_*). --no-extras
leaves them out.

cpu_baseline: the reference's CPU path on one core over the same graph (its seq_cpu sweeps, by the
oracle's C restatement; PageRank: FP64 oracle sweeps, the reference has none); its outputs also check
the GPU's outputs of the timed run (`parity`: integers bit-exact, PageRank normalised L1).

--impl reference: the same CPU path on the same R-MAT scale-22 graph with all host threads, one step =
the headline's five jobs at once (the four seq_cpu traversals on a core each, FP64 PageRank to the same
stop on the remaining threads); the inputs come from the oracle's generator, so that arm loads no
product library.
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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SCALE, EF, SEED = 22, 16, 1
SAMPLE_SCALE = 18
ALGO_PLAN = [("bfs", "sync_push_dd"), ("sssp", "sync_push_dd"), ("sswp", "sync_push_dd"),
             ("cc", "async_push_dd"), ("pr", "sync_push_td")]
PR_TOL = 1e-7
BFS_PUSH_ONLY = False  # --bfs-push-only


def workload_name(scale: int, K: int, pr_k: int = 16) -> str:
    return (f"R-MAT s{scale} ef{EF} a/b/c/d=.57/.19/.19/.05 seed {SEED} w~U[1,63]; BFS/SSSP/SSWP sync_push_dd "
            f"from max-out-degree vertex, CC async_push_dd on the symmetrised graph, PR sync_push_td d=0.85 "
            f"tol 1e-7; K={K} (PageRank's transposed graph K={pr_k})")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# the sources each measured kernel is compiled from (a traffic figure is used only while they are unchanged)
KERNEL_SOURCES = {"k_traverse": ["traverse.cuh", "traverse_host.cu", "common.cuh"],
                  "k_pagerank": ["pagerank.cu", "common.cuh"], "k_ppr_rows": ["ppr.cu", "common.cuh"]}


def kernel_source_sha(kernel: str) -> str:
    """Hash of the kernel's source files with comments and blank lines left out (a comment edit keeps
    a measured figure valid; any code change retires it)."""
    import hashlib
    import re

    h = hashlib.sha1()
    for f in KERNEL_SOURCES[kernel.split("<")[0]]:
        text = (ROOT / "eegraph_gb300" / "csrc" / f).read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        h.update("\n".join(ln.rstrip() for ln in text.splitlines() if ln.strip()).encode())
    return h.hexdigest()[:16]


def load_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary (profiles/traffic.json), or None
    when there is none or it was measured on other sources of the kernel than the ones built here."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        t = json.loads(p.read_text())
        e = t.get(workload, {}).get(kernel)
        if e is None or e.get("source_sha") != kernel_source_sha(kernel):
            return None
        return float(e["dram_bytes_per_launch"])
    except Exception:
        return None


class EnergyMeter:
    """GPU energy (joules) over a timed region from the library's NVML session (eeg_energy_*)."""

    def __init__(self, device: int):
        import eegraph_gb300 as E

        self.session = E.EnergySession(device)

    def summary(self, steps: int, covers: str = "timed steps") -> dict:
        r = self.session.end()
        if r is None:
            return {"unavailable": self.session.reason or "NVML energy counter not available"}
        if r["joules"] <= 0.0:  # the counter did not advance over the region
            return {"joules": None, "note": "below the energy counter's resolution over this region",
                    "seconds": round(r["seconds"], 4), "covers": covers}
        return {"joules": round(r["joules"], 3), "joules_per_step": round(r["joules"] / max(steps, 1), 4),
                "seconds": round(r["seconds"], 4), "avg_watts": round(r["avg_watts"], 1), "covers": covers}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms (each line time-stamped) while the
    sampler is open. summary() keeps the samples inside the window marked by start()/stop() -- the timed
    region -- or every sample when no window was marked or no time stamp could be read."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t0 = self.t1 = None

    def __enter__(self):
        if self.proc is not None:  # already sampling (opened early, then used in a with block)
            return self
        cmd = ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "50"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            import atexit

            atexit.register(self.__exit__, None, None, None)  # no poller outlives the process
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def start(self):
        self.t0 = time.time()

    def stop(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import datetime

        rows = []
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                ts = None
            rows.append((ts, f[1:]))
        window = "whole run"
        if self.t0 is not None and self.t1 is not None:
            inside = [r for r in rows if r[0] is not None and self.t0 - 0.05 <= r[0] <= self.t1 + 0.05]
            if inside:
                rows, window = inside, "timed region"
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, f in rows:
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "window": window}


def reduce_job(total_ms: float, total_edges: float, world: int, device) -> tuple[float, float]:
    """Whole-job time and work over the ranks: the slowest rank's time, the sum of all ranks' edges."""
    if world <= 1:
        return total_ms, total_edges
    import torch
    import torch.distributed as dist

    t = torch.tensor([total_ms, total_edges], dtype=torch.float64, device=device)
    mx, sm = t.clone(), t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(sm[1])


# ---------------------------------------------------------------- workload
def make_inputs(E, scale: int):
    s, d, w = E.gen_rmat(scale, EF, seed=SEED, wmin=1, wmax=63)
    ss, ds, ws = E.symmetrize(s, d, w)
    n = 1 << scale
    return n, (s, d, w), (ss, ds, ws)


def teps_edges(algo: str, res: dict, m: int, m_sym: int) -> float:
    if algo == "pr":
        return float(res["iterations"]) * m
    if algo == "cc":
        return float(m_sym)
    return float(res["reached_edges"])


def run_step(vg, vg_sym, vg_pr, source, outs, stream, results):
    for algo, variant in ALGO_PLAN:
        g = vg_sym if algo == "cc" else (vg_pr if algo == "pr" else vg)
        _, res = g.run(algo, variant, source, out_device_ptr=outs[algo], stream=stream,
                       pr_tolerance=PR_TOL, bfs_push_only=BFS_PUSH_ONLY)
        results[algo] = res


def bench_gpu(args) -> None:
    import torch

    import eegraph_gb300 as E

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    E.lib().eeg_set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    scale = args.scale
    n, (s, d, w), (ss, ds, ws) = make_inputs(E, scale)
    m, m_sym = s.size, ss.size
    stream = torch.cuda.current_stream(dev).cuda_stream

    # BFS pulls in its large rounds over the transposed parts (SSSP and SSWP push only)
    vg = E.VirtualGraph.build(n, s, d, w, K=args.k, reverse=not BFS_PUSH_ONLY, stream=stream)
    vg_sym = E.VirtualGraph.build(n, ss, ds, ws, K=args.k, stream=stream)
    # PageRank pulls over the transposed graph: its own part size (unweighted)
    vg_pr = E.VirtualGraph.build(n, s, d, None, K=args.pr_k, reverse=True, stream=stream)
    info = vg.info()
    source = info["max_degree_vertex"]
    outs_t = {a: torch.empty(n, dtype=torch.int32, device=dev) for a, _ in ALGO_PLAN}
    outs = {a: t.data_ptr() for a, t in outs_t.items()}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    results: dict = {}
    # the clock sampler runs from the warm-up on (nvidia-smi needs a moment to start) and keeps the
    # samples stamped inside the timed region
    clk = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        run_step(vg, vg_sym, vg_pr, source, outs, stream, results)
    torch.cuda.synchronize()

    per_algo = {a: {"ms": [], "edges": [], "bytes": [], "iters": [], "scanned": []} for a, _ in ALGO_PLAN}
    step_ms = []
    launches = 0
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with clk:
        clk.start()
        energy = EnergyMeter(local)
        for i in range(args.steps):
            flush.fill_(float(i))  # L2 flush between timed steps (outside the events)
            starts[i].record()
            run_step(vg, vg_sym, vg_pr, source, outs, stream, results)
            ends[i].record()
            for a, _ in ALGO_PLAN:
                r = results[a]
                per_algo[a]["ms"].append(r["kernel_ms"])
                per_algo[a]["edges"].append(teps_edges(a, r, m, m_sym))
                per_algo[a]["bytes"].append(r["algorithmic_bytes"])
                per_algo[a]["iters"].append(r["iterations"])
                per_algo[a]["scanned"].append(r["edges_scanned"])
                launches += r["launches"]
        torch.cuda.synchronize()
        clk.stop()
        energy_line = energy.summary(args.steps, "timed steps (with their L2 flushes)")
        if world > 1:
            torch.distributed.barrier()
    step_ms = [starts[i].elapsed_time(ends[i]) for i in range(args.steps)]
    # the outputs of the last timed step, for the parity check against the reference CPU path
    gpu_vals = {a: outs_t[a].cpu().numpy().view(np.float32 if a == "pr" else np.uint32).copy() for a, _ in ALGO_PLAN}
    total_ms = sum(step_ms)
    step_edges = sum(per_algo[a]["edges"][-1] for a, _ in ALGO_PLAN)
    total_edges = step_edges * args.steps
    total_ms_all, total_edges_all = reduce_job(total_ms, total_edges, world, dev)
    value = total_edges_all / (total_ms_all * 1e-3) / 1e9

    # ---- end to end through the C ABI with host buffers (timed on the host around the whole step)
    import torch as _t

    pin = {k: _t.from_numpy(v.view(np.int32)).pin_memory() for k, v in {"s": s, "d": d, "w": w}.items()}
    dev_in = {k: _t.empty(v.numel(), dtype=_t.int32, device=dev) for k, v in pin.items()}
    ptr = {k: v.data_ptr() for k, v in dev_in.items()}
    host_out = {a: np.empty(n, np.float32 if a == "pr" else np.uint32) for a, _ in ALGO_PLAN}
    e2e_ms = []
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in pin:  # one upload of the directed edge list; every graph is built from it on the GPU
            dev_in[k].copy_(pin[k], non_blocking=True)
        g1 = E.VirtualGraph.build_device(n, m, ptr["s"], ptr["d"], ptr["w"], K=args.k, stream=stream)
        g2 = E.VirtualGraph.build_device(n, m, ptr["s"], ptr["d"], ptr["w"], K=args.k, symmetrize=True,
                                         stream=stream)
        g3 = E.VirtualGraph.build_device(n, m, ptr["s"], ptr["d"], None, K=args.pr_k, reverse_only=True,
                                         stream=stream)
        src_e2e = g1.info()["max_degree_vertex"]
        for algo, variant in ALGO_PLAN:
            (g2 if algo == "cc" else (g3 if algo == "pr" else g1)).run(algo, variant, src_e2e, out=host_out[algo],
                                                                        stream=stream, pr_tolerance=PR_TOL)
        g1.close()
        g2.close()
        g3.close()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    # the end-to-end path's host outputs equal the device-resident run's (integers exactly, PageRank bitwise:
    # same graph, same kernel)
    e2e_equal = all(np.array_equal(host_out[a], gpu_vals[a]) for a, _ in ALGO_PLAN) if e2e_ms else None
    e2e_total_ms = sum(e2e_ms)
    if world > 1:
        tt = torch.tensor([e2e_total_ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_total_ms = float(tt[0])
    e2e_value = total_edges_all / (e2e_total_ms * 1e-3) / 1e9 if e2e_ms else None
    h2d = 4 * 3 * m
    d2h = 4 * n * len(ALGO_PLAN)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    peak, peak_kind = load_peaks()
    algo_summary = {}
    for a, _ in ALGO_PLAN:
        ms = statistics.median(per_algo[a]["ms"])
        by = statistics.median(per_algo[a]["bytes"])
        ed = statistics.median(per_algo[a]["edges"])
        algo_summary[a] = {"kernel_ms": round(ms, 4), "gteps": round(ed / (ms * 1e-3) / 1e9, 3),
                           "iterations": int(statistics.median(per_algo[a]["iters"])),
                           "edges_scanned": int(statistics.median(per_algo[a]["scanned"])),
                           "algorithmic_GB": round(by / 1e9, 4),
                           "achieved_GBs": round(by / (ms * 1e-3) / 1e9, 1),
                           "roofline_frac": round(by / (ms * 1e-3) / 1e9 / peak, 4)}
    kern_names = {"bfs": "k_traverse<OP_BFS>", "sssp": "k_traverse<OP_SSSP>", "sswp": "k_traverse<OP_SSWP>",
                  "cc": "k_traverse<OP_CC>", "pr": "k_pagerank"}
    for a in algo_summary:  # measured DRAM bytes per launch (profiles/traffic.json), where captured
        tr = load_traffic(kern_names[a], f"s{scale}_k{args.pr_k if a == 'pr' else args.k}")
        algo_summary[a]["dram_GB_per_launch"] = round(tr / 1e9, 3) if tr else None
        # the measured DRAM bytes over this run's kernel time: what the kernel moves, where roofline_frac
        # counts the work-minimal bytes of the reference's push algorithm (BFS's pull rounds skip most)
        ms = algo_summary[a]["kernel_ms"]
        algo_summary[a]["dram_frac"] = round(tr / (ms * 1e-3) / 1e9 / peak, 4) if tr else None
    dom = max(algo_summary, key=lambda a: algo_summary[a]["kernel_ms"])
    kern_name = kern_names[dom]
    ach = algo_summary[dom]["achieved_GBs"]
    line = {
        "metric": "GTEPS (sum over BFS,SSSP,SSWP,CC,PR of TEPS edges / device time)",
        "value": round(value, 3),
        "unit": "GTEPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms_all / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 (BFS/SSSP/SSWP/CC), f32 (PageRank)",
        "data": "synthetic (seeded R-MAT, generated in-process)",
        "config": headline_config(scale, args.k, args.pr_k, n, m, m_sym, source, world),
        "per_algo": algo_summary,
        "roofline": {"bound": "hbm", "kernel": kern_name, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_source": peak_kind,
                     "traffic": load_traffic(kern_name, f"s{scale}_k{args.pr_k if dom == 'pr' else args.k}")},
        "e2e": {"value": round(e2e_value, 3) if e2e_value else None, "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_total_ms / args.steps, 3)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "energy": energy_line,
    }
    if world == 1 and not args.no_extras:
        vg.close()
        vg_sym.close()
        vg_pr.close()
        line.update(extras(args))
    if not args.no_cpu_baseline:
        # the reference's CPU path on the same graph, one core; its outputs check the GPU's
        line["cpu_baseline"], line["parity"] = cpu_baseline(n, (s, d, w), (ss, ds, ws), source, args.k, gpu_vals)
        if e2e_ms:
            line["parity"]["e2e_outputs_equal_device_outputs"] = e2e_equal
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def extras(args) -> dict:
    """Summaries of the other configurations the measurement plan names, measured after the headline in
    the same run (one GPU): the 4096^2 road-like grid (persistent kernel vs one launch per round), the
    256-graph query batch (one launch vs the plain kernel looped per query) and the 64-column personalised
    PageRank adjoint (batched vs looped per teleport vector). Each is the line of its own --workload run
    with fewer timed steps."""
    import argparse as _ap

    ea = _ap.Namespace(**vars(args))
    ea.steps = max(1, min(args.steps, 10))
    ea.no_cpu_baseline = True
    ea.scale = SCALE
    out = {}
    g = bench_grid(ea, emit=False)
    out["grid"] = {k: g[k] for k in ("metric", "value", "unit", "ms_per_step", "per_algo", "config")}
    b = bench_batch(ea, emit=False)
    out["batch"] = {k: b[k] for k in ("metric", "value", "unit", "ms_per_step", "plain_loop", "speedup_vs_plain_loop",
                                       "speedup_vs_plain_kernels", "gteps", "parity_with_plain", "config", "energy")}
    p = bench_ppr(ea, emit=False)
    out["ppr"] = {k: p[k] for k in ("metric", "value", "unit", "ms_per_step", "sweeps", "plain_loop",
                                     "speedup_vs_plain_loop", "parity_batched_vs_loop", "roofline", "e2e", "config",
                                     "energy")}
    out["stream"] = bench_stream(ea)
    out["extras_steps"] = ea.steps
    return out


def bench_stream(args) -> dict:
    """Active-subgraph streaming (eeg_stream_*) on the headline's R-MAT s22 graph held in host memory,
    with partition buffers of a quarter of the graph's parts: BFS/SSSP/SSWP sync from the max-degree
    vertex, checked equal to the in-memory kernels; GTEPS = reached edges / the whole streamed run
    (gathers over the CPU-GPU link included)."""
    import eegraph_gb300 as E

    n, (s, d, w), _ = make_inputs(E, args.scale)
    K = args.k
    parts = int(np.ceil(np.bincount(s, minlength=n) / K).sum())
    budget = 2 * (8 * K + 4) * (parts // 4)
    src = int(np.bincount(s, minlength=n).argmax())
    per = {}
    with E.VirtualGraph.build(n, s, d, w, K=K) as vg, E.StreamGraph.from_arrays(n, s, d, w, K=K,
                                                                               budget_bytes=budget) as sg:
        for algo in ("bfs", "sssp", "sswp"):
            want, ref = vg.run(algo, "sync_push_dd", src)
            sg.run(algo, "sync_push_dd", src)
            runs = [sg.run(algo, "sync_push_dd", src) for _ in range(max(1, min(args.steps, 3)))]
            ms = statistics.median(r["kernel_ms"] for _, r in runs)
            got, r = runs[-1]
            per[algo] = {"ms": round(ms, 3), "rounds": r["iterations"], "partitions": r["partitions"],
                         "gteps": round(r["reached_edges"] / (ms * 1e-3) / 1e9, 3),
                         "in_memory_ms": round(ref["kernel_ms"], 3), "equal_to_in_memory": bool(np.array_equal(got, want)),
                         "edge_bytes_streamed_GB": round(8 * r["edges_scanned"] / 1e9, 3)}
        info = sg.info()
    tot_ms = sum(v["ms"] for v in per.values())
    tot_edges = sum(v["gteps"] * v["ms"] * 1e6 for v in per.values())
    return {"metric": "GTEPS of streamed runs (graph in host memory, device buffers of a quarter of its parts)",
            "value": round(tot_edges / (tot_ms * 1e-3) / 1e9, 3), "unit": "GTEPS", "ms_per_step": round(tot_ms, 3),
            "config": {"workload": f"R-MAT s{args.scale} ef{EF} from the max-out-degree vertex, sync, K={K}",
                       "device_budget_bytes": info["device_budget_bytes"], "host_bytes": info["host_bytes"]},
            "per_algo": per}


def make_batch_inputs(E, num_graphs: int, seed: int = 4):
    """256 graphs, vertex counts log-uniform in [2^10, 2^20], R-MAT edge factor uniform in {8..32}
    (a/b/c/d .57/.19/.19/.05, weights U[1,63]); R-MAT ids of scale ceil(log2 n) are folded mod n. Each graph
    gets 1-8 queries, the algorithm drawn from {BFS, SSSP, SSWP}, the source uniform."""
    rng = np.random.default_rng(seed)
    graphs, queries = [], []
    for gi in range(num_graphs):
        n = int(round(2 ** rng.uniform(10, 20)))
        ef = int(rng.integers(8, 33))
        scale = max(1, int(np.ceil(np.log2(n))))
        s, d, w = E.gen_rmat(scale, ef, seed=1000 + gi, wmin=1, wmax=63)
        m = ef * n
        s, d, w = s[:m] % n, d[:m] % n, w[:m]
        graphs.append((n, s.astype(np.uint32), d.astype(np.uint32), w))
        for _ in range(int(rng.integers(1, 9))):
            queries.append((gi, ["bfs", "sssp", "sswp"][int(rng.integers(0, 3))], int(rng.integers(0, n))))
    return graphs, queries


def bench_batch(args, emit: bool = True):
    """Batched queries: one launch (captured CUDA graph) of the work-queue kernel against the plain
    persistent kernel looped per query, on the same GPU; values compared query by query. With N GPUs
    (torchrun) the queries are split by estimated work (graph edges + vertices; eegraph_gb300.shard_queries,
    the same partition on every rank, no exchange) and each GPU runs its share; the job's time is the
    slowest GPU's (strong scaling: the total work is fixed)."""
    import torch

    import eegraph_gb300 as E

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    E.lib().eeg_set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream().cuda_stream
    all_graphs, all_queries = make_batch_inputs(E, args.batch_graphs)
    costs = [all_graphs[g][1].size + all_graphs[g][0] for g, _, _ in all_queries]
    mine = E.shard_queries(costs, world)[rank]
    used = sorted({all_queries[i][0] for i in mine})
    remap = {g: j for j, g in enumerate(used)}
    graphs = [all_graphs[g] for g in used]
    queries = [(remap[all_queries[i][0]], all_queries[i][1], all_queries[i][2]) for i in mine]
    vgs = [E.VirtualGraph.build(n, s, d, w, K=args.k, stream=stream) for n, s, d, w in graphs]
    total_edges = sum(int(g[1].size) for g in all_graphs)
    with E.Batch(vgs) as b, ClockSampler(local) as clk:
        words = b.set_queries(queries)
        out = torch.zeros(words, dtype=torch.int32, device="cuda")
        cluster, _ = b.autotune(out.data_ptr())
        for _ in range(args.warmup):
            b.run(out.data_ptr())
        energy = EnergyMeter(local)
        clk.start()
        batch_ms = [b.run(out.data_ptr()) for _ in range(args.steps)]
        clk.stop()
        energy_line = energy.summary(args.steps, "timed batch launches")
        batched = out.cpu().numpy().view(np.uint32).copy()
        offs = b.offsets()
        # plain: the single-query persistent kernel, one call per query, into the same layout
        plain_out = torch.zeros(words, dtype=torch.int32, device="cuda")
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        plain_ms, plain_kernel_ms = [], []
        reached = 0
        for rep in range(max(1, min(args.steps, 2)) + 1):
            torch.cuda.synchronize()
            ev0.record()
            kms = 0.0
            for qi, (gi, algo, src) in enumerate(queries):
                _, r = vgs[gi].run(algo, "sync_push_dd", src, out_device_ptr=plain_out.data_ptr() + 4 * offs[qi],
                                   stream=stream)
                kms += r["kernel_ms"]  # the query's own kernel time (CUDA events around its launch)
                if rep == 0:
                    reached += r["reached_edges"]
            ev1.record()
            torch.cuda.synchronize()
            if rep > 0:  # the first pass warms the per-graph workspaces
                plain_ms.append(ev0.elapsed_time(ev1))
                plain_kernel_ms.append(kms)
        same = bool(np.array_equal(batched, plain_out.cpu().numpy().view(np.uint32)))
    for g in vgs:
        g.close()
    bms, pms = statistics.median(batch_ms), statistics.median(plain_ms)
    pkms = statistics.median(plain_kernel_ms)
    # whole job: the slowest GPU's time, the sum of the GPUs' work
    bms, nq = reduce_job(bms, float(len(queries)), world, dev)
    pms, reached = reduce_job(pms, float(reached), world, dev)
    pkms, _ = reduce_job(pkms, 0.0, world, dev)
    _, n_same = reduce_job(0.0, 1.0 if same else 0.0, world, dev)
    same = n_same == world
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    line = {"metric": f"batched queries/s (BFS/SSSP/SSWP mix over {len(all_graphs)} graphs) vs the plain kernel "
                      "looped per query",
            "value": round(nq / (bms * 1e-3), 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(bms, 3), "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT mixture, generated in-process)",
            "config": {"workload": f"{len(all_graphs)} graphs, n log-uniform [2^10, 2^20], ef U{{8..32}}, 1-8 queries each, "
                                   f"K={args.k}, cluster size {cluster} (autotuned)",
                       "graphs": len(all_graphs), "queries": int(nq), "edges": total_edges,
                       "parallelism": f"queries split by estimated work over {world} GPU(s)"},
            "plain_loop": {"ms_per_step": round(pms, 3), "queries_per_s": round(nq / (pms * 1e-3), 1),
                           "kernel_ms_per_step": round(pkms, 3),
                           "note": "ms_per_step: CUDA events around the whole loop (launches and host round trips "
                                   "included); kernel_ms_per_step: the sum of the queries' own kernel times"},
            "speedup_vs_plain_loop": round(pms / bms, 2), "speedup_vs_plain_kernels": round(pkms / bms, 2),
            "gteps": round(reached / (bms * 1e-3) / 1e9, 3),
            "parity_with_plain": same, "clocks": clk.summary(), "energy": energy_line}
    if emit:
        print(json.dumps(line))
    return line


PPR_SCALE, PPR_COLS, PPR_SEEDS = 20, 64, 32


def make_ppr_inputs(E, scale: int, cols: int = PPR_COLS, seed: int = 1):
    """R-MAT (scale, edge factor 16, a/b/c/d .57/.19/.19/.05, seed 1) with FP32 weights U(0,1]; `cols`
    teleport vectors, each uniform over 32 random seed vertices; dLoss/dX = c ~ N(0,1) (loss sum c*x)."""
    n = 1 << scale
    s, d, _ = E.gen_rmat(scale, EF, seed=seed, wmin=1, wmax=63)
    rng = np.random.default_rng(seed)
    w = (1.0 - rng.random(s.size)).astype(np.float32)
    T = np.zeros((n, cols), np.float32)
    for k in range(cols):
        T[rng.choice(n, PPR_SEEDS, replace=False), k] = 1.0 / PPR_SEEDS
    G = rng.standard_normal((n, cols)).astype(np.float32)
    return n, np.asarray(s, np.uint32), np.asarray(d, np.uint32), w, T, G


def ppr_cpu_baseline(budget_s: float, scale: int = 14, cols: int = 64) -> dict:
    """FP64 oracle (one core) on a bounded sample: R-MAT s14 with the same shape of inputs; its
    throughput is scaled to the full workload by the work ratio (edges x sweeps)."""
    import eegraph_gb300 as E

    import oracle

    n, s, d, w, T, G = make_ppr_inputs(E, scale, cols)
    t0 = time.perf_counter()
    r = oracle.ppr(n, s, d, w.astype(np.float64), T, G, tol=1e-7)
    dt = time.perf_counter() - t0
    return {"grads_per_s_sample": cols / dt, "sample_edges": int(s.size), "sample_sweeps": int(sum(r["sweeps"])),
            "seconds": dt}


def bench_ppr(args, emit: bool = True):
    """Differentiable personalised PageRank: forward + adjoint + gradients for 64 teleport vectors in
    one batched call pair, against the single-column kernels looped per teleport vector. With N GPUs
    (torchrun) the columns are split (eegraph_gb300.shard_columns): each GPU solves its columns on the
    whole graph and the per-edge gradients are summed across GPUs with one all-reduce of 2m floats
    inside the timed step; the job's time is the slowest GPU's (strong scaling: the total is fixed)."""
    import torch

    import eegraph_gb300 as E

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    E.lib().eeg_set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    scale = args.scale if args.scale != SCALE else PPR_SCALE
    n, s, d, w, T_all, G_all = make_ppr_inputs(E, scale, cols=args.ppr_columns)
    C_all = T_all.shape[1]
    cols = E.shard_columns(C_all, world)[rank]
    if not cols:
        raise SystemExit(f"rank {rank}: no columns (more GPUs than the {C_all} columns)")
    T, G = np.ascontiguousarray(T_all[:, cols]), np.ascontiguousarray(G_all[:, cols])
    C = T.shape[1]
    m = int(s.size)
    stream = torch.cuda.current_stream().cuda_stream
    vg = E.VirtualGraph.build(n, s, d, None, K=args.k, reverse=True, edge_ids=True, stream=stream)
    dev = torch.device("cuda", local)
    Tt, Gt = torch.from_numpy(T).to(dev), torch.from_numpy(G).to(dev)
    X = torch.empty_like(Tt)
    dT = torch.empty_like(Tt)
    grads = torch.empty(2 * m, dtype=torch.float32, device=dev)  # dLoss/dw and dLoss/dW, reduced together
    dw, dwn = grads[:m], grads[m:]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    outs = {"dw": dw.data_ptr(), "dwn": dwn.data_ptr(), "dt": dT.data_ptr()}
    with E.PPR(vg, C) as pb, ClockSampler(local) as clk:
        pb.set_weights(w)
        step_ms, fwd, adj = [], [], []
        energy = None
        for i in range(args.warmup + args.steps):
            if i == args.warmup:
                energy = EnergyMeter(local)
                clk.start()
            flush.zero_()
            torch.cuda.synchronize()
            ev0.record()
            _, rf = pb.forward(Tt.data_ptr(), X.data_ptr(), stream=stream)
            _, ra = pb.adjoint(Gt.data_ptr(), out_ptrs=outs, stream=stream)
            if dist is not None:
                dist.all_reduce(grads)  # the batch's edge gradients: the sum over the GPUs' columns
            ev1.record()
            torch.cuda.synchronize()
            if i >= args.warmup:
                step_ms.append(ev0.elapsed_time(ev1))
                fwd.append(rf)
                adj.append(ra)
        clk.stop()
        energy_line = energy.summary(args.steps, "timed steps (with their L2 flushes)")
        # duality c^T x = (1-d) t^T lambda over this GPU's columns
        duality = abs(float((Gt.double() * X.double()).sum()) - float((Tt.double() * dT.double()).sum()))
        duality /= float((Gt.double() * X.double()).abs().sum())
        # end to end through the host API: pinned host inputs in, gradients out to host
        Th, Gh = torch.from_numpy(T).pin_memory(), torch.from_numpy(G).pin_memory()
        dw_h = torch.empty(m, dtype=torch.float32).pin_memory()
        dT_h = torch.empty((n, C), dtype=torch.float32).pin_memory()
        e2e_ms = []
        for i in range(0 if args.no_e2e else args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pb.forward(Th.numpy(), False, stream=stream)
            if dist is None:
                pb.adjoint(Gh.numpy(), out_host={"dw": dw_h.numpy(), "dt": dT_h.numpy()}, stream=stream)
            else:  # the edge gradients are summed on the devices, then read back
                pb.adjoint(Gh.numpy(), out_ptrs={"dw": dw.data_ptr(), "dt": dT.data_ptr()}, stream=stream)
                dist.all_reduce(dw)
                dw_h.copy_(dw)
                dT_h.copy_(dT)
            torch.cuda.synchronize()
            if i >= args.warmup:
                e2e_ms.append((time.perf_counter() - t0) * 1e3)
        # plain: the single-column kernels looped over the teleport vectors (inputs pre-split per column)
        Tc = Tt.t().contiguous()
        Gc = Gt.t().contiguous()
        Xc = torch.empty_like(Tc)
        dTc = torch.empty_like(Tc)
        dw1 = torch.empty(m, dtype=torch.float32, device=dev)
        loop_ms = []
        with E.PPR(vg, 1) as p1:
            p1.set_weights(w)
            for rep in range(2):
                flush.zero_()
                torch.cuda.synchronize()
                ev0.record()
                for k in range(C):
                    p1.forward(Tc[k].data_ptr(), Xc[k].data_ptr(), stream=stream)
                    last = {"dw": dw1.data_ptr(), "dt": dTc[k].data_ptr()} if k == C - 1 else {"dt": dTc[k].data_ptr()}
                    p1.adjoint(Gc[k].data_ptr(), out_ptrs=last, accumulate=k > 0, stream=stream)
                ev1.record()
                torch.cuda.synchronize()
                if rep > 0:
                    loop_ms.append(ev0.elapsed_time(ev1))
        def nl1(a, b):
            return float((a - b).abs().sum() / b.abs().sum())
        if dist is not None:
            dist.all_reduce(dw1)  # the loop's edge gradients over all GPUs' columns, as the batch's
        parity = {"X_nl1": nl1(Xc.t().double(), X.double()), "dT_nl1": nl1(dTc.t().double(), dT.double()),
                  "dw_rel_l1": nl1(dw1.double(), dw.double()), "duality_rel": duality}
    vg.close()

    def job_max(x):  # the slowest (or worst) GPU's figure
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t[0])

    bms = job_max(statistics.median(step_ms))
    lms = job_max(statistics.median(loop_ms))
    e2e_med = job_max(statistics.median(e2e_ms)) if e2e_ms else None
    parity = {k: job_max(v) for k, v in parity.items()}
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None
    fkm = statistics.median(r["kernel_ms"] for r in fwd)
    fby = statistics.median(r["algorithmic_bytes"] for r in fwd)
    fit = int(statistics.median(r["iterations"] for r in fwd))
    ait = int(statistics.median(r["iterations"] for r in adj))
    peak, peak_kind = load_peaks()
    ach = fby / (fkm * 1e-3) / 1e9
    traffic = load_traffic("k_ppr_rows", f"ppr_s{scale}_k{args.k}") if C > 32 else None
    h2d = 2 * n * C_all * 4                     # all GPUs: their teleport and dLoss/dX columns
    d2h = world * m * 4 + n * C_all * 4         # each GPU reads the summed dLoss/dw and its dLoss/dT columns
    line = {
        "metric": "PR-grad/s (personalised PageRank forward + implicit adjoint + edge/teleport gradients, "
                  "teleport vectors per second)",
        "value": round(C_all / (bms * 1e-3), 2), "unit": "PR-grad/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(bms, 3), "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32 (FP64 stop-test reduction)",
        "data": "synthetic (seeded R-MAT, weights U(0,1], teleports and c generated in-process)",
        "config": {"workload": f"R-MAT s{scale} ef{EF}, {C_all} teleport vectors x {PPR_SEEDS} seeds, d=0.85, "
                               f"tol 1e-7, K={args.k}", "vertices": n, "edges": m, "columns": C_all,
                   "row_width": 1 if C == 1 else (32 if C <= 32 else 64),
                   "parallelism": f"columns split over {world} GPU(s) ({C} on rank 0), edge gradients all-reduced",
                   "l2": "iterates 2 x n x row width x 4 B larger than L2; 256 MB L2 flush between timed steps"},
        "sweeps": {"forward": fit, "adjoint": ait},
        "plain_loop": {"ms_per_step": round(lms, 3), "grads_per_s": round(C_all / (lms * 1e-3), 2)},
        "speedup_vs_plain_loop": round(lms / bms, 2),
        "parity_batched_vs_loop": parity,
        "roofline": {"bound": "hbm", "kernel": "k_ppr_rows (forward solve)", "achieved": round(ach, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": peak_kind,
                     "traffic": traffic,
                     "dram_achieved": round(traffic / (fkm * 1e-3) / 1e9, 1) if traffic else None,
                     "dram_frac": round(traffic / (fkm * 1e-3) / 1e9 / peak, 4) if traffic else None,
                     "note": "algorithmic bytes count every row gather as DRAM traffic; at 64 columns about "
                             "79 % of them hit L2 (traffic = measured DRAM bytes per launch), so frac can exceed 1; "
                             "dram_frac = measured DRAM bytes per launch / kernel time / peak"},
        "e2e": {"value": round(C_all / (e2e_med * 1e-3), 2) if e2e_med else None, "unit": "PR-grad/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_med, 3) if e2e_med else None},
        "gpu_launches": 5,
        "clocks": clk.summary(),
        "energy": energy_line,
    }
    if not args.no_cpu_baseline:
        cb = ppr_cpu_baseline(args.cpu_budget)
        work_full = m * (fit + ait)
        work_sample = cb["sample_edges"] * cb["sample_sweeps"]
        line["cpu_baseline"] = {"value": round(cb["grads_per_s_sample"] * work_sample / work_full, 4),
                                "unit": "PR-grad/s", "cores": 1, "kind": "port",
                                "sample": f"FP64 oracle, R-MAT s14 x 64 columns ({cb['seconds']:.1f} s), "
                                          "scaled by edges x sweeps to the full workload"}
    if emit:
        print(json.dumps(line))
    return line


GRID_SIDE, GRID_SEED = 4096, 7


def bench_grid(args, emit: bool = True):
    """High-diameter road-like graph: 4096 x 4096 grid, 4-neighbour undirected, 10 % of edges deleted,
    0.1 % long-range shortcuts, weights U[1,1000], seed 7. BFS/SSSP/SSWP sync_push_dd from vertex 0, one
    persistent launch each, against the same kernels run one launch per round with a host round trip
    in between (the reference's loop shape, src/eegraph.cu:89-211). SSSP and SSWP run bucketed rounds
    (--grid-delta-sssp / --grid-delta-sswp; 0 = plain rounds), whose plain-round time is reported too."""
    import torch

    import eegraph_gb300 as E

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    E.lib().eeg_set_device(local)
    side = args.grid_side
    n = side * side
    s, d, w = E.gen_grid(side, 0.1, 0.001, seed=GRID_SEED, wmin=1, wmax=1000)
    stream = torch.cuda.current_stream().cuda_stream
    plan = [("bfs", "sync_push_dd"), ("sssp", "sync_push_dd"), ("sswp", "sync_push_dd")]
    peak, peak_kind = load_peaks()
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    per = {}
    deltas = {"bfs": 0, "sssp": args.grid_delta_sssp, "sswp": args.grid_delta_sswp}
    joules = 0.0
    energy_ok = True
    with E.VirtualGraph.build(n, s, d, w, K=args.k, stream=stream) as vg, ClockSampler(local) as clk:
        for algo, variant in plan:
            dl = deltas[algo]
            for _ in range(args.warmup):
                vg.run(algo, variant, 0, out_device_ptr=out.data_ptr(), stream=stream, delta=dl)
            torch.cuda.synchronize()
            energy = EnergyMeter(local)
            pers = [vg.run(algo, variant, 0, out_device_ptr=out.data_ptr(), stream=stream, delta=dl)[1]
                    for _ in range(args.steps)]
            torch.cuda.synchronize()
            en = energy.summary(args.steps)
            if en.get("joules") is not None:
                joules += en["joules"]
            elif "unavailable" in en:
                energy_ok = False
            hl = vg.run(algo, variant, 0, out_device_ptr=out.data_ptr(), stream=stream, host_loop=True, delta=dl)[1]
            ms = statistics.median(r["kernel_ms"] for r in pers)
            r0 = pers[0]
            per[algo] = {"kernel_ms": round(ms, 3), "rounds": r0["iterations"], "delta": dl,
                         "gteps": round(r0["reached_edges"] / (ms * 1e-3) / 1e9, 3),
                         "roofline_frac": round(r0["algorithmic_bytes"] / (ms * 1e-3) / 1e9 / peak, 4),
                         "edges_scanned_per_reached_edge": round(r0["edges_scanned"] / max(r0["reached_edges"], 1), 2),
                         "host_loop_ms": round(hl["kernel_ms"], 3),
                         "speedup_vs_host_loop": round(hl["kernel_ms"] / ms, 2)}
            if dl:
                plain = vg.run(algo, variant, 0, out_device_ptr=out.data_ptr(), stream=stream)[1]
                per[algo]["plain_rounds_ms"] = round(plain["kernel_ms"], 3)
                per[algo]["plain_rounds"] = plain["iterations"]
    tot_ms = sum(v["kernel_ms"] for v in per.values())
    tot_e = sum(float(r) for r in [per[a]["gteps"] * per[a]["kernel_ms"] * 1e6 for a in per])
    line = {"metric": "GTEPS (BFS+SSSP+SSWP reached edges / device time) on the 4096^2 road-like grid",
            "value": round(tot_e / (tot_ms * 1e-3) / 1e9, 3), "unit": "GTEPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(tot_ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded grid, generated in-process)",
            "config": {"workload": f"grid {side}x{side}, 10% edges deleted, 0.1% shortcuts, w~U[1,1000], seed 7, "
                                   f"source 0, K={args.k}, bucket widths SSSP {deltas['sssp']} SSWP {deltas['sswp']}",
                       "vertices": n, "arcs": int(s.size)},
            "per_algo": per, "peak": peak, "peak_source": peak_kind, "clocks": clk.summary(),
            "energy": ({"joules": round(joules, 3), "joules_per_step": round(joules / args.steps, 4),
                        "covers": "timed persistent runs of the three algorithms"} if energy_ok and joules > 0
                       else {"joules": None, "note": "below the energy counter's resolution over these runs"}
                       if energy_ok else {"unavailable": "NVML energy counter not available"})}
    if emit:
        print(json.dumps(line))
    return line


# ---------------------------------------------------------------- CPU (reference) path
PR_SAMPLE_SWEEPS = 8  # PageRank sweeps the 1-core baseline times (the reference has no CPU PageRank)


def make_inputs_cpu(scale: int):
    """The headline's inputs made by the oracle's generator (identical arrays; no product library)."""
    import oracle

    s, d, w = oracle.gen_rmat(scale, EF, seed=SEED, wmin=1, wmax=63)
    ss, ds, ws = oracle.symmetrize(s, d, w)
    return 1 << scale, (s, d, w), (ss, ds, ws)


def headline_config(scale: int, K: int, pr_k: int, n: int, m: int, m_sym: int, source: int, world: int) -> dict:
    """The `config` object of the headline line; both arms print the same one for the same workload."""
    return {"workload": workload_name(scale, K, pr_k), "scale": scale, "edge_factor": EF, "K": K, "pr_K": pr_k,
            "vertices": n, "edges": m, "cc_arcs": m_sym, "source": source, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (part arrays ~0.7 GB) and 256 MB L2 flush between timed steps"}


class CpuPath:
    """The reference's CPU path on one graph: its seq_cpu topology sweeps (the oracle's restatement of
    src/{bfs,sssp,sswp,cc}.cu seq_cpu, on the lossless layout built once here, outside any timing) and,
    for PageRank, which the reference has no CPU form of, the FP64 oracle's pull sweeps."""

    def __init__(self, n, g, gsym, K: int = 8):
        import oracle

        self.o = oracle
        self.n, self.K = n, K
        s, d, w = g
        self.m, self.m_sym = int(s.size), int(gsym[0].size)
        self.layout = oracle.virtual_graph(n, s, d, w, K)
        self.layout_sym = oracle.virtual_graph(n, *gsym, K)
        self.csr_in = oracle.in_csr(n, s, d)  # in-edges by target, and the out-degrees

    def traverse(self, algo: str, source: int):
        """(values, TEPS edges, seconds of the sweeps)."""
        lay = self.layout_sym if algo == "cc" else self.layout
        vals, _, secs = self.o.seq_sweep_layout(algo, self.n, lay, source, self.K)
        if algo == "cc":
            return vals, float(self.m_sym), secs
        reached = (vals != 0) if algo == "sswp" else (vals != self.o.INF)
        return vals, float(self.csr_in[2][reached].sum()), secs

    def pagerank(self, threads: int = 1, sweeps: int = 0, tol: float = PR_TOL * 0.15 / 0.85):
        """(x, TEPS edges = sweeps * m, seconds); sweeps > 0 runs exactly that many sweeps."""
        t0 = time.perf_counter()
        x, it = self.o.pagerank_pull(self.csr_in, 0.85, 0.0 if sweeps else tol, sweeps or 100000, threads)
        return x, float(it) * self.m, time.perf_counter() - t0


def parity_check(path: CpuPath, source: int, gpu_vals: dict, cpu_vals: dict, threads: int) -> dict:
    """The GPU's outputs of the timed run against the reference CPU path's (bit-exact for the integer
    algorithms) and PageRank against the FP64 oracle solved to 1e-11 (normalised L1)."""
    out = {}
    for a in ("bfs", "sssp", "sswp", "cc"):
        if a in gpu_vals and a in cpu_vals:
            bad = int((gpu_vals[a] != cpu_vals[a]).sum())
            out[a] = "exact" if bad == 0 else f"{bad} vertices differ"
    if "pr" in gpu_vals:
        xr, _, _ = path.pagerank(threads=threads, tol=1e-11)
        x = np.asarray(gpu_vals["pr"], np.float64)
        out["pr_l1"] = float(np.abs(x / x.sum() - xr / xr.sum()).sum())
        out["pr_ok"] = out["pr_l1"] <= 1e-6
    out["against"] = (f"reference seq_cpu sweeps (oracle restatement) from vertex {source}, CC all seeded; "
                      "PageRank FP64 oracle to 1e-11")
    return out


def cpu_baseline(n, g, gsym, source, K, gpu_vals=None) -> tuple[dict, dict | None]:
    """The reference's CPU path on ONE core over the headline's own graph: BFS, SSSP, SSWP (from the
    max-out-degree vertex) and CC (every vertex seeded, symmetrised) by the seq_cpu sweeps, plus
    PR_SAMPLE_SWEEPS PageRank sweeps of the FP64 oracle. Its outputs double as the parity check of the
    GPU's outputs (gpu_vals) when given. Returns (cpu_baseline, parity)."""
    path = CpuPath(n, g, gsym, K)
    tot_e, tot_t, vals = 0.0, 0.0, {}
    for algo in ("bfs", "sssp", "sswp", "cc"):
        v, e, t = path.traverse(algo, source)
        vals[algo] = v
        tot_e += e
        tot_t += t
    _, e, t = path.pagerank(threads=1, sweeps=PR_SAMPLE_SWEEPS)
    tot_e += e
    tot_t += t
    line = {"value": round(tot_e / tot_t / 1e9, 5), "unit": "GTEPS", "cores": 1, "kind": "port",
            "seconds": round(tot_t, 2),
            "sample": f"the headline graph (R-MAT s{int(np.log2(n))}) itself: BFS/SSSP/SSWP/CC by the reference's "
                      f"seq_cpu sweeps (oracle restatement, K={K}), PageRank {PR_SAMPLE_SWEEPS} FP64 sweeps (the "
                      "reference has no CPU PageRank)"}
    par = parity_check(path, source, gpu_vals, vals, threads=os.cpu_count() or 1) if gpu_vals else None
    return line, par


def bench_reference(args) -> None:
    """The reference's CPU path on the headline's own graph with all host threads: one step runs the
    headline's five jobs at once -- the four seq_cpu traversals on a core each and FP64 PageRank to the
    headline's stop on the remaining threads -- and counts TEPS edges as the GPU arm does."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import concurrent.futures as cf

    threads = args.cpu_threads or os.cpu_count() or 1
    scale = args.scale
    n, g, gsym = make_inputs_cpu(scale)
    source = int(np.bincount(g[0], minlength=n).argmax())
    path = CpuPath(n, g, gsym, args.k)
    pr_threads = max(1, threads - 4)
    algos = [a for a, _ in ALGO_PLAN]

    def step():
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(len(algos)) as ex:
            futs = [ex.submit(path.pagerank, pr_threads) if a == "pr" else ex.submit(path.traverse, a, source)
                    for a in algos]
            edges = sum(f.result()[1] for f in futs)
        return edges, time.perf_counter() - t0

    for _ in range(args.warmup):  # warm-up: one BFS job per step (page-in of the layouts)
        path.traverse("bfs", source)
    tot_e, tot_t = 0.0, 0.0
    for _ in range(args.steps):
        e, t = step()
        tot_e += e
        tot_t += t
    value = tot_e / tot_t / 1e9
    line = {
        "impl": "reference",
        "metric": "GTEPS (sum over BFS,SSSP,SSWP,CC,PR of TEPS edges / device time)",
        "value": round(value, 5), "unit": "GTEPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot_t / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 (BFS/SSSP/SSWP/CC), f64 (PageRank oracle)",
        "data": "synthetic (seeded R-MAT, generated in-process by the oracle's generator)",
        "config": headline_config(scale, args.k, args.pr_k, n, path.m, path.m_sym, source, world),
        "cpu_baseline": {"value": round(value, 5), "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"each step the headline's five jobs at once on R-MAT s{scale}: BFS/SSSP/SSWP "
                                   f"from vertex {source} and CC (all seeded, symmetrised) by the reference's seq_cpu "
                                   f"sweeps (oracle restatement; one core each), PageRank by the FP64 oracle to the "
                                   f"headline's stop on {pr_threads} threads (the reference has no CPU PageRank); "
                                   "warm-up steps run one BFS job each"},
        "e2e": {"value": round(value, 5), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--k", type=int, default=8, choices=[4, 8, 16])
    ap.add_argument("--pr-k", type=int, default=16, choices=[4, 8, 16],
                    help="part size of PageRank's graph (pull over the transposed graph)")
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--cpu-budget", type=float, default=30.0)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) measurement")
    ap.add_argument("--pr-variant", default="sync_push_td", choices=["sync_push_td", "async_push_td", "sync_push_dd",
                                                                     "async_push_dd"],
                    help="PageRank variant of the step (profiling; the headline uses sync_push_td)")
    ap.add_argument("--bfs-push-only", action="store_true",
                    help="BFS without pull rounds (the headline graph is then built without transposed parts)")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline only: skip the grid, batch and personalised-PageRank summaries")
    ap.add_argument("--algos", default="bfs,sssp,sswp,cc,pr",
                    help="subset of the step to run (profiling); the headline uses all five")
    ap.add_argument("--workload", default="rmat", choices=["rmat", "grid", "batch", "ppr", "stream"],
                    help="rmat: the headline (R-MAT s22, five algorithms); grid: the 4096^2 high-diameter graph; "
                         "batch: 256-graph query mixture, batched vs looped; "
                         "ppr: personalised PageRank forward + adjoint, 64 teleport vectors, batched vs looped; "
                         "stream: the R-MAT graph in host memory, streamed through device buffers")
    ap.add_argument("--batch-graphs", type=int, default=256)
    ap.add_argument("--ppr-columns", type=int, default=PPR_COLS, help="teleport vectors of the ppr workload (1-64)")
    ap.add_argument("--grid-side", type=int, default=GRID_SIDE)
    ap.add_argument("--grid-delta-sssp", type=int, default=8000, help="SSSP bucket width on the grid (0 = plain)")
    ap.add_argument("--grid-delta-sswp", type=int, default=16, help="SSWP bucket width on the grid (0 = plain)")
    args = ap.parse_args()
    global ALGO_PLAN, BFS_PUSH_ONLY
    ALGO_PLAN = [(a, args.pr_variant if a == "pr" else v) for a, v in ALGO_PLAN if a in args.algos.split(",")]
    BFS_PUSH_ONLY = args.bfs_push_only
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    elif args.workload == "grid":
        bench_grid(args)
    elif args.workload == "batch":
        bench_batch(args)
    elif args.workload == "ppr":
        bench_ppr(args)
    elif args.workload == "stream":
        import torch

        import eegraph_gb300 as E

        torch.cuda.set_device(dist_env()[2])
        E.lib().eeg_set_device(dist_env()[2])
        line = bench_stream(args)
        line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                     "data": "synthetic (seeded R-MAT, generated in-process)"})
        print(json.dumps(line))
    else:
        bench_gpu(args)


if __name__ == "__main__":
    main()
