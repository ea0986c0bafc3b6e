#!/usr/bin/env python
"""LA3 plain-path benchmark on GB300: GTEPS of BFS, SSSP, CC and TC.

Workload (the plain single-query configuration): seeded R-MAT scale 22
(edge factor 16, a/b/c/d = .57/.19/.19/.05, ids 1..2^22, self-loops and
duplicates removed) loaded undirected for BFS and CC and directed with
uint32 weights in [1, 128] for SSSP, and R-MAT scale 20 loaded as the
reference's TC loads it (directed, cycles removed).  One step = BFS and SSSP
from the step's root (drawn by seed from the non-isolated vertices), CC, and
TC, each through the C ABI.  GTEPS numerators: BFS = undirected edges with
both endpoints reached, SSSP = directed edges whose source is reachable,
CC = stored symmetric entries, TC = undirected edges; `value` is the sum of
the four numerators over the timed steps divided by the timed device time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl la3g|reference]

Multi-GPU runs are replicas (one process per GPU, launched by torchrun):
each rank runs the whole workload on its own copy of the graphs with its own
roots; `value` is the sum over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS per app on 1 GB300 (plain vs batched/served); p50/p99 query latency"
SCALE, TC_SCALE = 22, 20
GRAPH_SEED, WEIGHT_SEED, TC_SEED = 22, 23, 20
CPU_SAMPLE_SCALE, CPU_SAMPLE_TC_SCALE = 18, 16


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["la3g", "reference"], default="la3g")
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--tc-scale", type=int, default=TC_SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args(argv)


# ---------------------------------------------------------------- distributed

def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def reduce_results(edges: float, seconds: float, group=None, device=None):
    """Whole-job aggregation over replicas: edges summed, time = max."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return edges, seconds
    t = torch.tensor([edges, seconds], dtype=torch.float64, device=device)
    e = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(e, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(s, op=dist.ReduceOp.MAX, group=group)
    return float(e.item()), float(s.item())


def rank_roots(candidates, k: int, rank: int, seed: int = 99):
    """Roots of replica `rank`: a seeded draw from the non-isolated vertices."""
    import numpy as np
    rng = np.random.default_rng(seed + 1000 * rank)
    return [int(x) for x in rng.choice(candidates, size=k, replace=len(candidates) < k)]


# ---------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up can stall the driver: wait for its first
            # sample before the caller starts timing.
            t0 = time.time()
            while not self.lines and time.time() - t0 < 10 and self.proc.poll() is None:
                time.sleep(0.05)
            self.mark = len(self.lines)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def start_timed(self):
        self.mark = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[getattr(self, "mark", 0):] or self.lines[-1:]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return d.get(kernel)


# ---------------------------------------------------------------- CPU baseline

def ref_bench_bin() -> Path:
    return ROOT / "oracle" / "_ref" / "bin" / "bench_ref"


def run_reference_sample(steps: int, scale: int, tc_scale: int, nroots: int = 4, seed: int = 99) -> dict:
    """Runs the reference's own CPU implementation (built from its sources with
    the single-rank MPI stand-in; np = 1, OMP_NUM_THREADS = 2) on a seeded
    R-MAT sample, ingest untimed, execute() windows timed."""
    import numpy as np
    import la3_gb300 as L
    exe = ref_bench_bin()
    if not exe.exists():
        raise FileNotFoundError(str(exe))
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        n, ntc = 1 << scale, 1 << tc_scale
        e = L.EdgeList.rmat(scale, 16, seed=GRAPH_SEED)
        e.write(d / "g.bin")
        ew = L.EdgeList.rmat(scale, 16, seed=GRAPH_SEED, weighted=True, wseed=WEIGHT_SEED)
        ew.write(d / "g.w.bin")
        L.EdgeList.rmat(tc_scale, 16, seed=TC_SEED).write(d / "t.bin")
        src, dst, _ = e.arrays()
        # roots with out-edges, so that the directed SSSP from them does work too
        cand = np.unique(src[src != dst])
        roots = rank_roots(cand, nroots, 0, seed)
        env = dict(os.environ, OMP_NUM_THREADS="2")
        t0 = time.time()
        r = subprocess.run([str(exe), str(d / "g.bin"), str(d / "g.w.bin"), str(n), str(d / "t.bin"), str(ntc),
                            str(steps)] + [str(x) for x in roots], capture_output=True, text=True, env=env, check=True)
        wall = time.time() - t0
    out = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    summ = [o for o in out if o.get("summary")][-1]
    per_step = [o for o in out if "step" in o]
    return {"summary": summ, "steps": per_step, "wall_s": wall, "roots": roots}


def cpu_threads_note() -> str:
    try:
        import platform
        return f"{platform.machine()} x{os.cpu_count()}"
    except Exception:
        return "unknown"


def reference_line(args) -> dict:
    """--impl reference: the reference CPU path on a bounded sample."""
    res = run_reference_sample(args.warmup + args.steps, CPU_SAMPLE_SCALE, CPU_SAMPLE_TC_SCALE)
    steps = res["steps"][args.warmup:]
    e = sum(s["bfs_e"] + s["sssp_e"] + s["cc_e"] + s["tc_e"] for s in steps)
    t = sum(s["bfs_s"] + s["sssp_s"] + s["cc_s"] + s["tc_s"] for s in steps)
    v = e / t / 1e9
    apps = {a: sum(s[f"{a}_e"] for s in steps) / max(1e-12, sum(s[f"{a}_s"] for s in steps)) / 1e9
            for a in ("bfs", "sssp", "cc", "tc")}
    sample = (f"reference apps (np=1, OMP_NUM_THREADS=2; one tile so SpMV runs on one thread) on R-MAT "
              f"s{CPU_SAMPLE_SCALE} (BFS/SSSP/CC) + s{CPU_SAMPLE_TC_SCALE} (TC); execute() windows only; "
              f"host {cpu_threads_note()}")
    return {"metric": METRIC, "value": v, "unit": "GTEPS", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded R-MAT)",
            "config": {"workload": f"plain BFS+SSSP+CC R-MAT s{CPU_SAMPLE_SCALE} + TC s{CPU_SAMPLE_TC_SCALE} "
                                   f"(bounded CPU sample of the s{SCALE}/s{TC_SCALE} workload)",
                       "apps_gteps": apps},
            "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": 2, "kind": "reference", "sample": sample},
            "e2e": {"value": v, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- GPU arm

def gpu_line(args, rank: int, world: int, local: int) -> dict | None:
    import numpy as np
    import torch
    import la3_gb300 as L

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    t_setup = time.time()
    e = L.EdgeList.rmat(args.scale, 16, seed=GRAPH_SEED)
    ew = L.EdgeList.rmat(args.scale, 16, seed=GRAPH_SEED, weighted=True, wseed=WEIGHT_SEED)
    et = L.EdgeList.rmat(args.tc_scale, 16, seed=TC_SEED)
    GU = L.Graph.from_edges(e, 0)
    GW = L.Graph.from_edges(ew, L.DIRECTED | L.WEIGHTED)
    GT = L.Graph.from_edges(et, L.DIRECTED | L.ACYCLIC)
    pos, ids = GU.positions()
    nonisolated = ids[: GU.info.nregular + GU.info.nsink]
    # SSSP roots: vertices with out-edges in the directed graph (regular and
    # source positions); a sink root reaches nothing
    _, wids = GW.positions()
    iw = GW.info
    with_out = np.concatenate([wids[: iw.nregular], wids[iw.nregular + iw.nsink: iw.nregular + iw.nsink + iw.nsource]])
    del e, ew, et
    K, W = args.steps, args.warmup
    roots = rank_roots(np.sort(nonisolated), K + W, rank)
    sroots = rank_roots(np.sort(with_out), K + W, rank, seed=98)
    for g in (GU, GW, GT):
        g.set_stream(stream.cuda_stream)
    setup_s = time.time() - t_setup

    # TEPS numerators per root (computed once, outside every timed region)
    teps_b, teps_s = {}, {}
    for r in set(roots):
        _, _, sb = L.bfs(GU, r, False, False)
        teps_b[r] = sb.teps_edges
    for r in set(sroots):
        _, ss = L.sssp(GW, r, False)
        teps_s[r] = ss.teps_edges
    _, sc = L.cc(GU, False)
    _, _, stc = L.tc(GT, False)
    cc_e, tc_e = sc.teps_edges, stc.teps_edges

    def step(k):
        L.N.check(L.N.lib().la3g_bfs(GU._h, roots[k], None, None, None))
        L.N.check(L.N.lib().la3g_sssp(GW._h, sroots[k], None, None))
        L.N.check(L.N.lib().la3g_cc(GU._h, None, None))
        L.N.check(L.N.lib().la3g_tc(GT._h, None, None, None))

    # warm-up
    for k in range(W):
        step(k)
    torch.cuda.synchronize()

    # L2: every step's inputs (s22 CSR ~ 0.5 GB) are larger than the 129 MB L2;
    # additionally the L2 is flushed before each step by writing 256 MB.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    flush.fill_(1)  # first touch maps the pages (hundreds of ms): keep it out of the timed region
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    app_ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(K)]
    edges = 0.0
    app_edges = {"bfs": 0, "sssp": 0, "cc": 0, "tc": 0}
    lib = L.N.lib()
    with ClockSampler(local) as clocks:
        step(0)  # one more untimed step with the sampler running
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks.start_timed()
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for k in range(K):
                r, rs = roots[W + k], sroots[W + k]
                flush.fill_(k & 0xFF)
                a = app_ev[k]
                a[0].record(stream)
                L.N.check(lib.la3g_bfs(GU._h, r, None, None, None))
                a[1].record(stream)
                L.N.check(lib.la3g_sssp(GW._h, rs, None, None))
                a[2].record(stream)
                L.N.check(lib.la3g_cc(GU._h, None, None))
                a[3].record(stream)
                L.N.check(lib.la3g_tc(GT._h, None, None, None))
                a[4].record(stream)
                app_edges["bfs"] += teps_b[r]
                app_edges["sssp"] += teps_s[rs]
                app_edges["cc"] += cc_e
                app_edges["tc"] += tc_e
            ev[1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    region_ms = ev[0].elapsed_time(ev[1])
    app_ms = {"bfs": 0.0, "sssp": 0.0, "cc": 0.0, "tc": 0.0}
    for a in app_ev:
        for i, nm in enumerate(("bfs", "sssp", "cc", "tc")):
            app_ms[nm] += a[i].elapsed_time(a[i + 1])
    edges = float(sum(app_edges.values()))
    tot_edges, tot_s = reduce_results(edges, region_ms / 1e3, device=dev)
    value = tot_edges / tot_s / 1e9

    # end-to-end through the public API with host buffers (pinned outputs)
    N, NT = GU.nslots, GT.nslots
    pin = lambda n, dt: torch.empty(n, dtype=dt, pin_memory=True).numpy()
    hops, par, dist, lab, ntri = (pin(N, torch.uint8), pin(N, torch.int32).view(np.uint32),
                                  pin(N, torch.int32).view(np.uint32), pin(N, torch.int32).view(np.uint32),
                                  pin(NT, torch.int32).view(np.uint32))
    roots_h = pin(2 * K, torch.int32).view(np.uint32)
    roots_h[:K] = roots[W:W + K]
    roots_h[K:] = sroots[W:W + K]
    import ctypes as C
    u8p, u32p = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32)
    tot = C.c_uint64()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(K):
        r, rs = int(roots_h[k]), int(roots_h[K + k])
        L.N.check(lib.la3g_bfs(GU._h, r, hops.ctypes.data_as(u8p), par.ctypes.data_as(u32p), None))
        L.N.check(lib.la3g_sssp(GW._h, rs, dist.ctypes.data_as(u32p), None))
        L.N.check(lib.la3g_cc(GU._h, lab.ctypes.data_as(u32p), None))
        L.N.check(lib.la3g_tc(GT._h, C.byref(tot), ntri.ctypes.data_as(u32p), None))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_edges, e2e_s = reduce_results(edges, e2e_s, device=dev)
    e2e = {"value": e2e_edges / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 16,
           "d2h_bytes_per_step": N * (1 + 4 + 4 + 4) + NT * 4 + 8}

    # roofline of the dominant kernel: per-launch CUDA events inside the library
    L.profile_reset()
    L.profile(True)
    with torch.cuda.stream(stream):
        for k in range(min(K, 2)):
            step(W + k)
    torch.cuda.synchronize()
    L.profile(False)
    prof = L.profile_report()
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peaks = measured_peaks()
    achieved = dom[1]["bytes"] / (dom[1]["ms"] / 1e3) / 1e9
    launches = dom[1]["launches"]
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": ncu_traffic(dom[0]), "algo_bytes_per_launch": dom[1]["bytes"] / launches,
                "ms_per_launch": dom[1]["ms"] / launches,
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 4),
                                "gbs": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["ms"] > 0 else None}
                            for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}
    launches_per_step = None

    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": region_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT, generated in-process)",
        "config": {"workload": f"plain BFS+SSSP+CC on R-MAT s{args.scale} (ef 16) + TC on R-MAT s{args.tc_scale}",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (s22 CSR ~0.5 GB) and 256 MB L2 flush before every step",
                   "apps_gteps": {a: app_edges[a] / (app_ms[a] / 1e3) / 1e9 for a in app_ms},
                   "apps_ms_per_step": {a: app_ms[a] / K for a in app_ms},
                   "nentries": {"undirected_s22": GU.info.nentries, "directed_s22": GW.info.nentries,
                                "tc_s20": GT.info.nentries},
                   "setup_s": round(setup_s, 2)},
        "roofline": roofline,
        "e2e": e2e,
        "clocks": clocks.summary(),
    }
    # kernels of this library per step (counted by the library)
    st = [L.Stats() for _ in range(4)]
    lib.la3g_bfs(GU._h, roots[W], None, None, C.byref(st[0]))
    lib.la3g_sssp(GW._h, sroots[W], None, C.byref(st[1]))
    lib.la3g_cc(GU._h, None, C.byref(st[2]))
    lib.la3g_tc(GT._h, None, None, C.byref(st[3]))
    launches_per_step = sum(s.kernel_launches for s in st)
    line["gpu_launches"] = launches_per_step * K
    line["config"]["iterations"] = {"bfs": st[0].iterations, "bfs_bottom_up": st[0].pull_iterations,
                                    "sssp": st[1].iterations}
    if not args.no_cpu_baseline:
        try:
            res = run_reference_sample(2, CPU_SAMPLE_SCALE, CPU_SAMPLE_TC_SCALE)
            s = res["summary"]
            e_ = s["bfs_e"] + s["sssp_e"] + s["cc_e"] + s["tc_e"]
            t_ = s["bfs_s"] + s["sssp_s"] + s["cc_s"] + s["tc_s"]
            line["cpu_baseline"] = {
                "value": e_ / t_ / 1e9, "unit": "GTEPS", "cores": 2, "kind": "reference",
                "sample": (f"2 steps of BFS+SSSP+CC on R-MAT s{CPU_SAMPLE_SCALE} + TC on s{CPU_SAMPLE_TC_SCALE}, "
                           f"reference apps np=1 OMP_NUM_THREADS=2 (one tile: SpMV on one thread), execute() "
                           f"windows only, host {cpu_threads_note()}, {res['wall_s']:.1f} s wall incl. ingest")}
        except Exception as ex:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": "GTEPS", "cores": 0, "kind": "reference",
                                    "sample": f"unavailable: {type(ex).__name__}: {ex}"}
    return line


def main(argv=None) -> int:
    args = parse_args(argv)
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank == 0:
            try:
                print(json.dumps(reference_line(args)), flush=True)
            except Exception as ex:
                print(json.dumps({"impl": "reference", "unavailable": f"{type(ex).__name__}: {ex}"}), flush=True)
        return 0
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    line = gpu_line(args, rank, world, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
