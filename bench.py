#!/usr/bin/env python
"""LA3 plain-path benchmark on GB300: GTEPS of BFS, SSSP, CC and TC.

Workload (the plain single-query configuration): seeded R-MAT scale 22
(edge factor 16, a/b/c/d = .57/.19/.19/.05, ids 1..2^22, self-loops and
duplicates removed) loaded undirected for BFS and CC and directed with
uint32 weights in [1, 128] for SSSP, and R-MAT scale 20 loaded as the
reference's TC loads it (directed, cycles removed).  One step = BFS and SSSP
from the step's root (drawn by seed from the non-isolated vertices), CC, and
TC (both of its passes: the list building and the counting), each through
the C ABI.  GTEPS numerators: BFS = undirected edges with both endpoints
reached, SSSP = directed edges whose source is reachable, CC = stored
symmetric entries, TC = undirected edges; `value` is the sum of the four
numerators over the timed steps divided by the timed device time.

The same line carries, outside the timed region: the first timed step's
results checked against the C oracle on the same inputs ("parity") and the
oracle's own times as the CPU baseline; per-app fractions of the HBM
roofline; and the systems forms on their configurations ("systems":
batched BFS/SSSP with 64/256/1024 roots on R-MAT s22 and ER 2^22, the
served stream's saturation rate and p50/p99, PageRank FP64 on R-MAT s16
and FP32 vs FP64 on R-MAT s24).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl la3g|reference]

The reference arm (--impl reference) runs the reference's own CPU build on
the same workload (inputs written by the host-only generator tool, so no
library of this project is loaded): every graph ingested once, untimed;
warm-up BFS runs, one CC and one TC run, then steps alternating BFS and
SSSP from the same roots as the GPU arm; `value` = sum over apps of the
mean numerator / sum over apps of the mean execute() time, i.e. the GTEPS
of one step of the same composition.

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


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["la3g", "reference"], default="la3g")
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--tc-scale", type=int, default=TC_SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the oracle parity check and CPU baseline")
    ap.add_argument("--no-systems", action="store_true", help="skip the batched / served / PageRank sub-results")
    ap.add_argument("--workload", choices=["plain", "batched", "precision", "serve", "next"], default="plain",
                    help="plain (default): the single-query BFS/SSSP/CC/TC step; batched: multi-source BFS/SSSP; "
                         "precision: FP32 vs FP64 PageRank on s24; serve: Poisson query stream over resident graphs; "
                         "next: LM queries, the degree app and graph simulation")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window per offered rate")
    ap.add_argument("--serve-rates", default="1000,5000,20000,50000")
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
                                          "--format=csv,noheader,nounits", "-lms", "20"],
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


# ---------------------------------------------------------------- workload

def workload_config(args) -> dict:
    """The workload's description, identical in both arms' lines."""
    return {"workload": f"plain BFS+SSSP+CC on R-MAT s{args.scale} (ef 16) + TC on R-MAT s{args.tc_scale}",
            "graphs": {"bfs_cc": f"R-MAT s{args.scale} ef 16 seed {GRAPH_SEED}, undirected",
                       "sssp": f"R-MAT s{args.scale} ef 16 seed {GRAPH_SEED}, directed, u32 weights in [1, 128] "
                               f"seed {WEIGHT_SEED}",
                       "tc": f"R-MAT s{args.tc_scale} ef 16 seed {TC_SEED}, directed acyclic (lower id -> higher id)"},
            "roots": "seeded draws: BFS from the non-isolated vertices, SSSP from the vertices with out-edges"}


def candidate_roots(pairs_path: Path, triples_path: Path, n: int):
    """Root candidates from the edge files (sorted ids): vertices with an
    edge (BFS) and vertices with an out-edge (SSSP) - the same sets the GPU
    arm reads off the loaded graphs' vertex classes."""
    import numpy as np
    a = np.fromfile(pairs_path, np.uint32)
    nonisolated = np.nonzero(np.bincount(a, minlength=n + 1))[0].astype(np.uint32)
    del a
    w = np.fromfile(triples_path, np.uint32).reshape(-1, 3)
    with_out = np.nonzero(np.bincount(w[:, 0], minlength=n + 1))[0].astype(np.uint32)
    return nonisolated, with_out


# ---------------------------------------------------------------- reference arm

def ref_bench_bin() -> Path:
    return ROOT / "oracle" / "_ref" / "bin" / "bench_ref"


def gen_tool() -> Path:
    return ROOT / "la3_gb300" / "bin" / "la3g_gen"


def cpu_threads_note() -> str:
    import platform
    return f"{platform.machine()} x{os.cpu_count()}"


def reference_line(args) -> dict:
    """--impl reference: the reference's own CPU build on the same workload
    (inputs from the host-only generator tool; no library of this project
    is loaded in this process or its children)."""
    exe, gen = ref_bench_bin(), gen_tool()
    for f in (exe, gen):
        if not f.exists():
            raise FileNotFoundError(f"{f} (run __graft_entry__.build() first)")
    K, W = args.steps, args.warmup
    threads = os.cpu_count() or 1
    n, ntc = 1 << args.scale, 1 << args.tc_scale
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        g, gw, gt = d / "g.bin", d / "g.w.bin", d / "t.bin"
        t0 = time.time()
        subprocess.run([str(gen), "rmat", str(args.scale), "16", str(GRAPH_SEED), str(g)], check=True,
                       capture_output=True)
        subprocess.run([str(gen), "rmat", str(args.scale), "16", str(GRAPH_SEED), str(gw), str(WEIGHT_SEED)],
                       check=True, capture_output=True)
        subprocess.run([str(gen), "rmat", str(args.tc_scale), "16", str(TC_SEED), str(gt)], check=True,
                       capture_output=True)
        gen_s = time.time() - t0
        nonisolated, with_out = candidate_roots(g, gw, n)
        roots = rank_roots(nonisolated, K + W, 0)
        sroots = rank_roots(with_out, K + W, 0, seed=98)
        npairs = max(1, (K + 1) // 2)
        pair_args = []
        for i in range(npairs):
            pair_args += [str(roots[W + i]), str(sroots[W + i])]
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        t0 = time.time()
        r = subprocess.run([str(exe), str(g), str(gw), str(n), str(gt), str(ntc), str(W), str(K), "1", "1"] + pair_args,
                           capture_output=True, text=True, env=env, check=True)
        wall = time.time() - t0
    out = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    summ = [o for o in out if o.get("summary")][-1]
    runs = summ["runs"]
    mean_e = {a: summ[f"{a}_e"] / max(1, runs[a]) for a in ("bfs", "sssp", "cc", "tc")}
    mean_s = {a: summ[f"{a}_s"] / max(1, runs[a]) for a in ("bfs", "sssp", "cc", "tc")}
    v = sum(mean_e.values()) / sum(mean_s.values()) / 1e9
    apps = {a: mean_e[a] / max(1e-12, mean_s[a]) / 1e9 for a in mean_e}
    sample = (f"reference apps built from their sources (np=1, OMP_NUM_THREADS={threads}; one tile, so the SpMV runs on "
              f"one thread) on the same inputs: {W} untimed BFS runs, then {runs['cc']} CC, {runs['tc']} TC (both "
              f"passes), {runs['bfs']} BFS and {runs['sssp']} SSSP execute() windows; value = sum of per-app mean "
              f"numerators / sum of per-app mean times (one step's composition); ingest {summ['ingest_s']:.0f} s "
              f"untimed; host {cpu_threads_note()}")
    cfg = workload_config(args)
    cfg.update({"apps_gteps": apps, "apps_s_per_run": mean_s, "runs": runs, "ingest_s": summ["ingest_s"],
                "generate_s": round(gen_s, 1), "wall_s": round(wall, 1)})
    return {"metric": METRIC, "value": v, "unit": "GTEPS", "impl": "reference", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": 1e3 * sum(mean_s.values()),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded R-MAT, written by the host-only generator tool)",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": threads, "kind": "reference", "sample": sample},
            "e2e": {"value": v, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- GPU arm

def gpu_line(args, rank: int, world: int, local: int) -> dict | None:
    import ctypes as C
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
    check = rank == 0 and not args.no_cpu_baseline
    tmpdir = tempfile.TemporaryDirectory() if check else None
    if check:
        # the same records for the oracle (written outside every timed region)
        d = Path(tmpdir.name)
        e.write(d / "g.bin")
        ew.write(d / "g.w.bin")
        et.write(d / "t.bin")
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

    # TEPS numerators and algorithmic bytes per root (outside every timed region)
    teps_b, teps_s, bytes_b, bytes_s = {}, {}, {}, {}
    for r in set(roots):
        _, _, sb = L.bfs(GU, r, False, False)
        teps_b[r], bytes_b[r] = sb.teps_edges, sb.algo_bytes
    for r in set(sroots):
        _, ss = L.sssp(GW, r, False)
        teps_s[r], bytes_s[r] = ss.teps_edges, ss.algo_bytes
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
    app_edges = {"bfs": 0, "sssp": 0, "cc": 0, "tc": 0}
    app_bytes = {"bfs": 0.0, "sssp": 0.0, "cc": 0.0, "tc": 0.0}
    lib = L.N.lib()
    with ClockSampler(local) as clocks:
        step(0)  # one more untimed step with the sampler running
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks.start_timed()
        # an NVTX range around the timed steps lets a profiler capture exactly them
        torch.cuda.nvtx.range_push("bench_timed_steps")
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
                app_bytes["bfs"] += bytes_b[r]
                app_bytes["sssp"] += bytes_s[rs]
                app_bytes["cc"] += sc.algo_bytes
                app_bytes["tc"] += stc.algo_bytes
            ev[1].record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
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
    e2e = {"value": e2e_edges / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 8,
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
                            for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])},
                # each app's algorithmic bytes over the timed steps / its timed device time / peak
                "apps": {a: {"gbs": app_bytes[a] / (app_ms[a] / 1e3) / 1e9,
                             "frac": app_bytes[a] / (app_ms[a] / 1e3) / 1e9 / peaks["hbm_gbs"],
                             "bytes_per_step": app_bytes[a] / K}
                         for a in app_ms}}

    line = None
    if rank == 0:
        cfg = workload_config(args)
        cfg.update({"parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                    "l2": "inputs larger than L2 (s22 CSR ~0.5 GB) and 256 MB L2 flush before every step",
                    "apps_gteps": {a: app_edges[a] / (app_ms[a] / 1e3) / 1e9 for a in app_ms},
                    "apps_ms_per_step": {a: app_ms[a] / K for a in app_ms},
                    "nentries": {"undirected": GU.info.nentries, "directed": GW.info.nentries,
                                 "tc": GT.info.nentries},
                    "setup_s": round(setup_s, 2)})
        line = {
            "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": region_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32", "data": "synthetic (seeded R-MAT, generated in-process)",
            "config": cfg, "roofline": roofline, "e2e": e2e, "clocks": clocks.summary(),
        }
        # kernels of this library per step (counted by the library)
        st = [L.Stats() for _ in range(4)]
        lib.la3g_bfs(GU._h, roots[W], None, None, C.byref(st[0]))
        lib.la3g_sssp(GW._h, sroots[W], None, C.byref(st[1]))
        lib.la3g_cc(GU._h, None, C.byref(st[2]))
        lib.la3g_tc(GT._h, None, None, C.byref(st[3]))
        line["gpu_launches"] = sum(x.kernel_launches for x in st) * K
        cfg["iterations"] = {"bfs": st[0].iterations, "bfs_bottom_up": st[0].pull_iterations,
                             "sssp": st[1].iterations}
        if check:
            try:
                par_, cpu = oracle_check(Path(tmpdir.name), args, GU, GW, GT, roots[W], sroots[W])
                line["parity"] = par_
                line["cpu_baseline"] = cpu
            except Exception as ex:  # reported, never required
                line["parity"] = {"checked": False, "error": f"{type(ex).__name__}: {ex}"}
            tmpdir.cleanup()
        if not args.no_systems:
            line["systems"] = systems_results(args, GU, GW, stream, dev)
    return line


def oracle_check(d: Path, args, GU, GW, GT, root: int, sroot: int):
    """The first timed step's results against the C oracle on the same
    records, every vector compared in full (bit-exact); the oracle's own
    execution times form the CPU baseline (kind "port")."""
    import numpy as np
    import la3_gb300 as L
    from oracle import oracle as O
    O.build()
    n, ntc = 1 << args.scale, 1 << args.tc_scale
    hops, parent, sb = L.bfs(GU, root)
    dist, ss = L.sssp(GW, sroot)
    lab, sc = L.cc(GU)
    tot, ntri, stc = L.tc(GT)
    res, times, edges = {}, {}, {}
    og = O.OracleGraph(d / "g.bin", n, 0)
    t0 = time.perf_counter()
    oh, op, _ = og.bfs(root)
    times["bfs"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ol, _ = og.cc()
    times["cc"] = time.perf_counter() - t0
    del og
    res["bfs"] = bool(np.array_equal(hops, oh) and np.array_equal(parent, op))
    res["cc"] = bool(np.array_equal(lab, ol))
    ow = O.OracleGraph(d / "g.w.bin", n, O.DIRECTED | O.WEIGHTED)
    t0 = time.perf_counter()
    od, _ = ow.sssp(sroot)
    times["sssp"] = time.perf_counter() - t0
    del ow
    res["sssp"] = bool(np.array_equal(dist, od))
    ot = O.OracleGraph(d / "t.bin", ntc, O.DIRECTED | O.ACYCLIC)
    t0 = time.perf_counter()
    otot, oper = ot.tc()
    times["tc"] = time.perf_counter() - t0
    del ot
    res["tc"] = bool(otot == tot and np.array_equal(ntri, oper))
    edges = {"bfs": sb.teps_edges, "sssp": ss.teps_edges, "cc": sc.teps_edges, "tc": stc.teps_edges}
    parity = {"checked": True, "bit_exact": all(res.values()), "apps": res,
              "case": f"BFS root {root} (hops + parent), SSSP root {sroot} (distances), CC (labels), TC (total "
                      f"{tot} and per-vertex counts): full vectors against the C oracle on the same records"}
    omp = os.environ.get("OMP_NUM_THREADS")
    threads = int(omp) if omp and omp.isdigit() else (os.cpu_count() or 1)
    cpu = {"value": sum(edges.values()) / sum(times.values()) / 1e9, "unit": "GTEPS", "cores": threads,
           "kind": "port",
           "sample": (f"one step of the same workload (BFS root {root}, SSSP root {sroot}, CC, TC) through the C "
                      f"restatement of the reference's path: BFS/SSSP/CC single-threaded, TC's intersections over "
                      f"{threads} OpenMP threads; execute windows only (ingest untimed); host {cpu_threads_note()}; "
                      f"per app s: " + ", ".join(f"{a} {t:.2f}" for a, t in times.items()))}
    return parity, cpu


def systems_results(args, GU, GW, stream, dev) -> dict:
    """The systems forms on their configurations, for the default line:
    batched BFS/SSSP (64/256/1024 roots) on the plain step's R-MAT graphs and
    on ER 2^22, PageRank (FP64 s16 with oracle parity, FP32 vs FP64 on
    R-MAT and ER 2^24), the served stream at 1k/s offered and at
    saturation (20k/s offered), and the generic engine (graph simulation and
    TC on the TC graph's size).  Each part carries its own clock record;
    a part that fails reports its error instead."""
    import torch
    out = {}
    idx = torch.cuda.current_device()

    def batched():
        graphs = batched_graphs(args, rmat=(GU, GW))
        for gu, gw in graphs.values():
            gu.set_stream(stream.cuda_stream)
            gw.set_stream(stream.cuda_stream)
        r = batched_measure(args, 0, graphs, stream, dev)
        for gu, gw in (graphs["er"],):
            gu.free()
            gw.free()
        return r

    parts = (("batched", batched),
             ("pagerank", lambda: pagerank_measure(args, stream, dev)),
             ("served", lambda: serve_measure(args, [1000.0, 20000.0], 1.0)),
             ("engine", lambda: engine_measure(args, stream)))
    for name, fn in parts:
        t0 = time.time()
        try:
            with ClockSampler(idx) as clocks:
                clocks.start_timed()
                r = fn()
            r["clocks"] = clocks.summary()
        except Exception as ex:  # reported, never required
            r = {"error": f"{type(ex).__name__}: {ex}"}
        r["wall_s"] = round(time.time() - t0, 1)
        out[name] = r
        torch.cuda.synchronize()
    return out


def engine_measure(args, stream) -> dict:
    """The generic vertex-program engine (include/la3g_vp.cuh) on the plain
    bench's TC graph size: graph simulation (graphsim.cpp:45-90; a 5-vertex
    query with a cycle, 6 labels, the data graph reversed) and TC written as
    the reference writes it (tc.cpp:11-52; neighbour lists as variable-size
    messages), each call timed on the host clock (median of three), results
    checked: TC's total against la3g_tc."""
    import ctypes as C
    import numpy as np
    import la3_gb300 as L
    import la3_gb300.build as B
    progs = C.CDLL(str(B.PROGRAMS_LIB))
    u32p = C.POINTER(C.c_uint32)
    progs.la3gp_graphsim.argtypes = [C.c_void_p, u32p, C.c_uint32, u32p, u32p, C.c_uint32, C.POINTER(C.c_uint8),
                                     C.c_char_p, u32p, u32p]
    progs.la3gp_tc.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64), u32p]
    sc = args.tc_scale
    rng = np.random.default_rng(501)
    gr = L.Graph.from_edges(L.EdgeList.rmat(sc, 16, seed=GRAPH_SEED + 7), L.DIRECTED | L.REVERSE)
    gr.set_stream(stream.cuda_stream)
    vlab = np.zeros(gr.nslots, np.uint32)
    vlab[: 1 << sc] = rng.integers(1, 7, 1 << sc)
    qlab = np.array([1, 2, 3, 2, 4], np.uint32)
    qedges = np.array([[0, 1], [1, 2], [2, 3], [3, 1], [1, 4]], np.uint32).reshape(-1)
    matched = np.empty(gr.nslots, np.uint8)

    def gs():
        nm, it = C.c_uint32(), C.c_uint32()
        t0 = time.perf_counter()
        L.N.check(progs.la3gp_graphsim(gr._h, vlab.ctypes.data_as(u32p), qlab.size, qlab.ctypes.data_as(u32p),
                                       qedges.ctypes.data_as(u32p), qedges.size // 2,
                                       matched.ctypes.data_as(C.POINTER(C.c_uint8)), None, C.byref(nm), C.byref(it)))
        return time.perf_counter() - t0, nm.value, it.value

    gs()
    g_runs = [gs() for _ in range(3)]
    gr.free()
    et = L.EdgeList.rmat(sc, 16, seed=TC_SEED)
    gt = L.Graph.from_edges(et, L.DIRECTED | L.ACYCLIC)
    gtr = L.Graph.from_edges(et, L.DIRECTED | L.ACYCLIC | L.REVERSE)
    del et
    gt.set_stream(stream.cuda_stream)
    gtr.set_stream(stream.cuda_stream)

    def tce():
        tot = C.c_uint64()
        t0 = time.perf_counter()
        L.N.check(progs.la3gp_tc(gt._h, gtr._h, C.byref(tot), None))
        return time.perf_counter() - t0, tot.value

    tce()
    t_runs = [tce() for _ in range(3)]
    lib_total = L.tc(gt, False)[0]
    gt.free()
    gtr.free()
    return {"graph": f"R-MAT s{sc} (edge factor 16)",
            "graphsim": {"ms": statistics.median(r[0] for r in g_runs) * 1e3, "matches": g_runs[-1][1],
                         "iterations": g_runs[-1][2], "query": "5 vertices, a cycle, 6 labels"},
            "tc_through_engine": {"ms": statistics.median(r[0] for r in t_runs) * 1e3, "triangles": t_runs[-1][1],
                                  "equals_la3g_tc": t_runs[-1][1] == lib_total},
            "timing": "host clock around each call (engine set-up and result copy included), median of 3"}


# ---------------------------------------------------------------- other workloads

def _pct(xs, q):
    import numpy as np
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else None


def _timed(stream, fn):
    """Device time (ms) of a synchronous library call on `stream`, by events."""
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def _flush_fn(dev):
    """A function that writes 256 MB (twice the L2) on the current stream."""
    import torch
    buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    buf.fill_(1)  # first touch maps the pages: keep it out of any timed region
    torch.cuda.synchronize()
    count = [0]

    def flush():
        count[0] += 1
        buf.fill_(count[0] & 0xFF)
        torch.cuda.synchronize()  # done before the next timed call starts on its own stream

    return flush


def batched_measure(args, rank: int, graphs: dict, stream, dev, sizes_b=(64, 256, 1024), sizes_s=(64, 256, 1024),
                    parity_roots: int = 8) -> dict:
    """Batched multi-source BFS / SSSP (64 roots per frontier word): per
    graph and batch size, batch time after an L2 flush, GTEPS = sum over
    roots of the single-root numerator / batch time, and its ratio to the
    plain per-root rate (single-root calls of the same roots, timed alike).
    Parity: for the 64-root batches, `parity_roots` sampled roots' full hop /
    distance vectors equal the single-root calls'."""
    import numpy as np
    import la3_gb300 as L
    flush = _flush_fn(dev)
    sweep, depth_hist, tune, parity = {}, {}, {}, {}
    for name, (gu, gw) in graphs.items():
        _, ids = gu.positions()
        cand_b = np.sort(ids[: gu.info.nregular])
        _, wids = gw.positions()
        iw = gw.info
        cand_s = np.sort(np.concatenate([wids[: iw.nregular],
                                         wids[iw.nregular + iw.nsink: iw.nregular + iw.nsink + iw.nsource]]))
        rb = rank_roots(cand_b, max(sizes_b), rank, seed=7)
        rs = rank_roots(cand_s, max(sizes_s), rank, seed=8)
        # the project autotuner picks level mode, block size and push threshold
        # for this graph and each batch size (untimed, separate root draws)
        tune[name] = {R: min(L.batch_autotune(gu, rank_roots(cand_b, R, rank, seed=17 + R)), key=lambda c: c["ms"])
                      for R in sizes_b}
        # single-root numerators and times (outside every timed batch)
        tb, ts, eb, es, lv = [], [], {}, {}, []
        for r in rb:
            st = L.Stats()
            flush()
            ms = _timed(stream, lambda: L.N.check(L.N.lib().la3g_bfs(gu._h, r, None, None, L.C.byref(st))))
            tb.append(ms)
            eb[r] = st.teps_edges
            lv.append(st.iterations)
        for r in rs:
            st = L.Stats()
            flush()
            ms = _timed(stream, lambda: L.N.check(L.N.lib().la3g_sssp(gw._h, r, None, L.C.byref(st))))
            ts.append(ms)
            es[r] = st.teps_edges
        h = np.bincount(np.asarray(lv))
        depth_hist[name] = {int(i): int(c) for i, c in enumerate(h) if c}
        ent = {"bfs": {}, "sssp": {}}
        plain_b = sum(eb[r] for r in rb) / (sum(tb) / 1e3) / 1e9
        plain_s = sum(es[r] for r in rs) / (sum(ts) / 1e3) / 1e9
        for R in sizes_b:
            rr = rb[:R]
            L.bfs_batch(gu, rr, want_hops=False)  # warm (allocations, graph capture)
            flush()
            ms = _timed(stream, lambda: L.bfs_batch(gu, rr, want_hops=False))
            g_ = sum(eb[r] for r in rr) / (ms / 1e3) / 1e9
            ent["bfs"][R] = {"ms": round(ms, 3), "gteps": g_, "x_plain": g_ / plain_b}
        for R in sizes_s:
            rr = rs[:R]
            L.sssp_batch(gw, rr, want_dist=False)
            flush()
            ms = _timed(stream, lambda: L.sssp_batch(gw, rr, want_dist=False))
            g_ = sum(es[r] for r in rr) / (ms / 1e3) / 1e9
            ent["sssp"][R] = {"ms": round(ms, 3), "gteps": g_, "x_plain": g_ / plain_s}
        ent["plain"] = {"bfs_gteps": plain_b, "sssp_gteps": plain_s, "bfs_ms_per_root": statistics.mean(tb),
                        "sssp_ms_per_root": statistics.mean(ts)}
        sweep[name] = ent
        if parity_roots:
            R = min(sizes_b)
            hb, _ = L.bfs_batch(gu, rb[:R], want_hops=True)
            ds, _ = L.sssp_batch(gw, rs[:R], want_dist=True)
            pick = np.linspace(0, R - 1, parity_roots).astype(int)
            ok_b = all(np.array_equal(hb[i], L.bfs(gu, rb[i], True, False)[0]) for i in pick)
            ok_s = all(np.array_equal(ds[i], L.sssp(gw, rs[i])[0]) for i in pick)
            parity[name] = {"bfs": ok_b, "sssp": ok_s,
                            "case": f"{parity_roots} of the {R} roots of each batch, full vectors vs single-root calls"}
            del hb, ds
    return {"sweep": sweep, "bfs_depth_histogram": depth_hist, "autotune_best": tune, "parity": parity,
            "l2": "256 MB L2 flush before every batch and every single-root call"}


def batched_line(args, rank, world, local) -> dict | None:
    """Batched multi-source BFS / SSSP on R-MAT s22 and Erdos-Renyi 2^22
    (BFS: 8 n undirected pairs, average degree 16; SSSP: 16 n directed
    pairs): the sweep above, then timed steps of one BFS batch of 1024 roots
    and one SSSP batch of 1024 roots on R-MAT."""
    import numpy as np
    import torch
    import la3_gb300 as L
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    graphs = batched_graphs(args)
    for gu, gw in graphs.values():
        gu.set_stream(stream.cuda_stream)
        gw.set_stream(stream.cuda_stream)
    res = batched_measure(args, rank, graphs, stream, dev)
    gu, gw = graphs["rmat"]
    _, ids = gu.positions()
    rb = rank_roots(np.sort(ids[: gu.info.nregular]), 1024, rank, seed=7)
    _, wids = gw.positions()
    iw = gw.info
    rs = rank_roots(np.sort(np.concatenate([wids[: iw.nregular],
                                            wids[iw.nregular + iw.nsink: iw.nregular + iw.nsink + iw.nsource]])),
                    1024, rank, seed=8)
    eb = sum(L.bfs(gu, r, False, False)[2].teps_edges for r in rb)
    es = sum(L.sssp(gw, r, False)[1].teps_edges for r in rs)
    flush = _flush_fn(dev)

    def step():
        L.bfs_batch(gu, rb, want_hops=False)
        L.sssp_batch(gw, rs, want_dist=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        clocks.start_timed()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
        tot = 0.0
        for k in range(args.steps):
            flush()
            ev[2 * k].record(stream)
            step()
            ev[2 * k + 1].record(stream)
            torch.cuda.synchronize()
            tot += ev[2 * k].elapsed_time(ev[2 * k + 1])
    e_all, t_all = reduce_results((eb + es) * args.steps, tot / 1e3, device=dev)
    # end to end: roots from pinned host memory in, hops / distances out
    pin_roots = torch.tensor(rb, dtype=torch.int64).to(torch.int32).pin_memory().numpy().view(np.uint32)
    t0 = time.perf_counter()
    hb, _ = L.bfs_batch(gu, pin_roots, want_hops=True)
    ds, _ = L.sssp_batch(gw, rs, want_dist=True)
    e2e_s = time.perf_counter() - t0
    if rank != 0:
        return None
    res["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
    res["workload"] = (f"batched BFS (1024 roots) + SSSP (1024 roots) on R-MAT s{args.scale}; sweep on R-MAT and "
                       f"ER 2^{args.scale}")
    return {
        "metric": METRIC, "value": e_all / t_all / 1e9, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 frontier words / u32 distances", "data": "synthetic (seeded R-MAT and ER)",
        "config": res,
        "e2e": {"value": (eb + es) / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 4 * (len(rb) + len(rs)),
                "d2h_bytes_per_step": int(hb.nbytes + ds.nbytes)},
        "clocks": clocks.summary(),
    }


def batched_graphs(args, rmat=None) -> dict:
    import la3_gb300 as L
    n = 1 << args.scale
    if rmat is None:
        rmat = (L.Graph.from_edges(L.EdgeList.rmat(args.scale, 16, seed=GRAPH_SEED), 0),
                L.Graph.from_edges(L.EdgeList.rmat(args.scale, 16, seed=GRAPH_SEED, weighted=True, wseed=WEIGHT_SEED),
                                   L.DIRECTED | L.WEIGHTED))
    return {"rmat": rmat,
            "er": (L.Graph.from_edges(L.EdgeList.er(n, 8 * n, seed=GRAPH_SEED + 100), 0),
                   L.Graph.from_edges(L.EdgeList.er(n, 16 * n, seed=GRAPH_SEED + 101, weighted=True, wseed=WEIGHT_SEED),
                                      L.DIRECTED | L.WEIGHTED))}


def pagerank_measure(args, stream, dev, include_er: bool = True) -> dict:
    """PageRank: (1) the plain-method configuration - FP64, 20 iterations on
    R-MAT s16 (edge factor 16), ranks compared bit for bit with the C
    oracle on the same records; (2) the precision study - FP32 SpMV with FP32
    accumulation vs the FP64 path on R-MAT s24 (and ER 2^24 x16 directed):
    50 iterations or FP64 L1 residual < 1e-9, L1 and max-abs error, GTEPS."""
    import numpy as np
    import la3_gb300 as L
    from oracle import oracle as O
    out = {}
    flush = _flush_fn(dev)
    # (1) s16 FP64, 20 iterations
    e = L.EdgeList.rmat(16, 16, seed=GRAPH_SEED + 1)
    G = L.Graph.from_edges(e, L.DIRECTED)
    G.set_stream(stream.cuda_stream)
    L.pagerank(G, 20, False, False)
    ts = []
    for _ in range(5):
        flush()
        st = L.Stats()
        ts.append(_timed(stream, lambda: L.N.check(L.N.lib().la3g_pr(G._h, 20, None, None, L.C.byref(st)))))
    m16 = G.info.nentries
    rank16, deg16, _ = L.pagerank(G, 20)
    with tempfile.TemporaryDirectory() as d:
        e.write(Path(d) / "p.bin")
        O.build()
        og = O.OracleGraph(Path(d) / "p.bin", 1 << 16, O.DIRECTED)
        orank, odeg = og.pagerank(20)
    G.free()
    del e
    out["s16_fp64"] = {"m": m16, "iterations": 20, "ms": statistics.median(ts),
                       "gteps": 20 * m16 / statistics.median(ts) / 1e6,
                       "bit_exact_vs_oracle": bool(np.array_equal(rank16.view(np.uint64), orank.view(np.uint64))
                                                   and np.array_equal(deg16, odeg)),
                       "max_abs_vs_oracle": float(np.abs(rank16 - orank).max())}
    # (2) precision study
    scale = 24 if args.scale == SCALE else args.scale + 2
    n = 1 << scale
    iters, tol = 50, 1e-9
    for name in (("rmat", "er") if include_er else ("rmat",)):
        if name == "rmat":
            e = L.EdgeList.rmat(scale, 16, seed=GRAPH_SEED + 2)
        else:
            e = L.EdgeList.er(n, 16 * n, seed=GRAPH_SEED + 3)
        G = L.Graph.from_edges(e, L.DIRECTED)
        del e
        G.set_stream(stream.cuda_stream)
        m = G.info.nentries
        L.pagerank(G, 2, False, False)
        L.pagerank_f32(G, 2)
        st64, st32 = L.Stats(), L.Stats()
        res = L.C.c_double()
        flush()
        t64 = _timed(stream, lambda: L.N.check(L.N.lib().la3g_pr(G._h, iters, None, None, L.C.byref(st64))))
        flush()
        t32 = _timed(stream, lambda: L.N.check(L.N.lib().la3g_pr_f32(G._h, iters, tol, None, L.C.byref(res),
                                                                     L.C.byref(st32))))
        # the FP32 study over the tiled DCSC layout (built by the first call, untimed)
        t0 = time.time()
        L.pagerank_f32(G, 2, tiled=True)
        tile_build_s = time.time() - t0
        stt = L.Stats()
        flush()
        tt = _timed(stream, lambda: L.N.check(L.N.lib().la3g_pr_f32_tiled(G._h, iters, tol, None, L.C.byref(res),
                                                                          L.C.byref(stt))))
        r64 = L.pagerank(G, iters, True, False)[0]
        r32, res32, _ = L.pagerank_f32(G, iters, tol)
        rt, rest, _ = L.pagerank_f32(G, iters, tol, tiled=True)
        d_ = np.abs(r32 - r64)
        dt = np.abs(rt - r64)
        out[f"s{scale}_{name}"] = {
            "m": m, "n": n, "dangling_frac": G.info.nsink / max(1, G.info.nvertices),
            "fp64": {"iterations": st64.iterations, "ms": t64, "gteps": st64.iterations * m / t64 / 1e6},
            "fp32": {"iterations": st32.iterations, "ms": t32, "gteps": st32.iterations * m / t32 / 1e6,
                     "l1_residual": res32},
            "fp32_tiled": {"iterations": stt.iterations, "ms": tt, "gteps": stt.iterations * m / tt / 1e6,
                           "x_flat": t32 / tt if tt else None, "l1_residual": rest,
                           "l1_rel_vs_fp64": float(dt.sum() / r64.sum()), "max_abs_vs_fp64": float(dt.max()),
                           "layout_build_s": round(tile_build_s, 2)},
            "l1_abs": float(d_.sum()), "l1_rel": float(d_.sum() / r64.sum()), "max_abs": float(d_.max()),
            "max_rel": float((d_ / np.maximum(1.0, r64)).max())}
        G.free()
    return out


def precision_line(args, rank, world, local) -> dict | None:
    """The PageRank configurations alone (see pagerank_measure)."""
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    with ClockSampler(local) as clocks:
        clocks.start_timed()
        out = pagerank_measure(args, stream, dev)
    if rank != 0:
        return None
    key = [k for k in out if k.endswith("_rmat")][0]
    return {
        "metric": METRIC, "value": out[key]["fp32"]["gteps"], "unit": "GTEPS", "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": out[key]["fp32"]["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (SpMV and accumulation); f64 residual", "data": "synthetic (seeded R-MAT and ER)",
        "config": {"workload": "PageRank: FP64 20 iterations on R-MAT s16; FP32 vs FP64 on R-MAT and ER 2^24, "
                               "50 iterations or L1 residual < 1e-9", "results": out,
                   "l2": "256 MB L2 flush before every timed call"},
        "e2e": None, "clocks": clocks.summary(),
    }


def serve_measure(args, rates, seconds: float) -> dict:
    """Served query stream: BFS / SSSP from random roots over R-MAT s18, s21
    and s23 (undirected for BFS, directed weighted for SSSP) and BM25 top-10
    over a bipartite corpus (8M docs, 1M terms, ~50 terms per doc, Zipf 1.1),
    Poisson arrivals at each offered rate; latency from submit to result.
    The plain arm runs the same stream one query at a time through the
    single-query entry points (same arrival times).  Both arms leave the
    BFS / SSSP vectors on the device and copy the BM25 top-10 out."""
    import numpy as np
    import la3_gb300 as L
    small = args.scale != SCALE  # reduced sizes for quick runs
    scales = (12, 14, 16) if small else (18, 21, 23)
    D, T, tpd = (100_000, 20_000, 30) if small else (8_000_000, 1_000_000, 50)
    t_setup = time.time()
    graphs = []
    for sc in scales:
        gu = L.Graph.from_edges(L.EdgeList.rmat(sc, 16, seed=100 + sc), 0)
        gw = L.Graph.from_edges(L.EdgeList.rmat(sc, 16, seed=100 + sc, weighted=True, wseed=200 + sc),
                                L.DIRECTED | L.WEIGHTED)
        graphs.append((sc, gu, gw))
    eb = L.EdgeList.bipartite(D, T, tpd, seed=300)
    postings = eb.m
    gb = L.Graph.from_edges(eb, L.BIPARTITE | L.WEIGHTED, D, T)
    del eb
    bm = L.BM25(gb)
    setup_s = time.time() - t_setup
    rng = np.random.default_rng(400)
    cands = []
    for sc, gu, gw in graphs:
        _, ids = gu.positions()
        _, wids = gw.positions()
        iw = gw.info
        cands.append((np.sort(ids[: gu.info.nregular]),
                      np.sort(np.concatenate([wids[: iw.nregular],
                                              wids[iw.nregular + iw.nsink: iw.nregular + iw.nsink + iw.nsource]]))))
    zipf_w = 1.0 / np.arange(1, T + 1) ** 1.1
    zipf_w /= zipf_w.sum()

    def make_stream(rate, nq):
        gaps = rng.exponential(1.0 / rate, nq)
        arr = np.cumsum(gaps)
        qs = []
        for i in range(nq):
            u = rng.random()
            if u < 0.4:
                gi = int(rng.integers(0, 3))
                qs.append(("bfs", gi, int(rng.choice(cands[gi][0]))))
            elif u < 0.8:
                gi = int(rng.integers(0, 3))
                qs.append(("sssp", gi, int(rng.choice(cands[gi][1]))))
            else:
                k = int(rng.integers(2, 9))
                terms = sorted(set(int(D + 1 + t) for t in rng.choice(T, k, p=zipf_w)))
                qs.append(("bm25", 0, terms))
        return arr, qs

    budget = int(200e9)
    S = L.Server(budget)  # default lanes: 256 BFS (four 64-lane words), 256 SSSP
    gid = []
    for sc, gu, gw in graphs:
        gid.append((S.add_graph(gu), S.add_graph(gw)))
    gid_b = S.add_graph(gb)
    lanes = {f"s{sc}": {"bfs": S.lanes(a), "sssp": S.lanes(b)} for (sc, _, _), (a, b) in zip(graphs, gid)}
    lib = L.N.lib()

    def served(arr, qs):
        n = len(qs)
        tickets = [None] * n
        ids_out = np.zeros((n, 10), np.uint32)
        sc_out = np.zeros((n, 10), np.float32)
        term_arrs = [np.asarray(q[2], np.uint32) if q[0] == "bm25" else None for q in qs]
        t0 = time.perf_counter()
        for i, (kind, gi, x) in enumerate(qs):
            while time.perf_counter() - t0 < arr[i]:
                pass
            if kind == "bfs":
                q = L.N.Query(kind=1, graph=gid[gi][0], root=x)
            elif kind == "sssp":
                q = L.N.Query(kind=2, graph=gid[gi][1], root=x)
            else:
                ta = term_arrs[i]
                q = L.N.Query(kind=3, graph=gid_b, k=10, terms=ta.ctypes.data_as(L.C.POINTER(L.C.c_uint32)),
                              nterms=ta.size, out=ids_out[i].ctypes.data,
                              scores_out=sc_out[i].ctypes.data_as(L.C.POINTER(L.C.c_float)))
            t = L.C.c_uint64()
            L.N.check(lib.la3g_server_submit(S._h, L.C.byref(q), L.C.byref(t)))
            tickets[i] = t.value
        t_sub = time.perf_counter() - t0
        lat, qlat, by = [], [], {"bfs": [], "sssp": [], "bm25": []}
        r = L.N.QueryResult()
        for i, t in enumerate(tickets):
            st = lib.la3g_server_poll(S._h, t, 600000, L.C.byref(r))
            L.N.check(st)
            if r.status != 0:
                raise RuntimeError(f"query {i} failed: {r.status}")
            lat.append(r.latency_ms)
            qlat.append(r.queue_ms)
            by[qs[i][0]].append(r.latency_ms)
        t_end = time.perf_counter() - t0
        return {"qps": n / t_end, "offered_qps": n / arr[-1], "submitted_qps": n / t_sub,
                "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99), "queue_p50_ms": _pct(qlat, 50),
                "by_kind_p50_ms": {k: _pct(v, 50) for k, v in by.items()},
                "by_kind_p99_ms": {k: _pct(v, 99) for k, v in by.items()}}, (ids_out, sc_out)

    def plain(arr, qs):
        n = len(qs)
        lat = []
        ids = np.zeros(10, np.uint32)
        sc = np.zeros(10, np.float32)
        nout = L.C.c_uint32()
        t0 = time.perf_counter()
        for i, (kind, gi, x) in enumerate(qs):
            now = time.perf_counter() - t0
            if now < arr[i]:
                while time.perf_counter() - t0 < arr[i]:
                    pass
            if kind == "bfs":
                L.N.check(lib.la3g_bfs(graphs[gi][1]._h, x, None, None, None))
            elif kind == "sssp":
                L.N.check(lib.la3g_sssp(graphs[gi][2]._h, x, None, None))
            else:
                ta = np.asarray(x, np.uint32)
                L.N.check(lib.la3g_bm25_query(gb._h, ta.ctypes.data_as(L.C.POINTER(L.C.c_uint32)), ta.size, 10,
                                              ids.ctypes.data_as(L.C.POINTER(L.C.c_uint32)),
                                              sc.ctypes.data_as(L.C.POINTER(L.C.c_float)), L.C.byref(nout),
                                              None, None, None))
            lat.append((time.perf_counter() - t0 - arr[i]) * 1e3)
        t_end = time.perf_counter() - t0
        return {"qps": n / t_end, "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99)}

    # BM25 alone: device time per query and the term kernel's algorithmic
    # GB/s (postings' doc id + tf, touched docs' K(d) and score) vs the peak
    bm_q = [sorted(set(int(D + 1 + t) for t in rng.choice(T, int(rng.integers(2, 9)), p=zipf_w))) for _ in range(300)]
    for q in bm_q[:20]:
        bm.query(q, 10)
    L.profile_reset()
    L.profile(True)
    bm_ms, bm_post = [], 0
    for q in bm_q:
        _, _, _, st = bm.query(q, 10)
        bm_ms.append(st.device_ms)
        bm_post += st.edges_examined
    L.profile(False)
    prof = L.profile_report().get("bm25_term", {"ms": 0.0, "bytes": 0.0, "launches": 0})
    peaks = measured_peaks()
    bm25_gbs = prof["bytes"] / (prof["ms"] / 1e3) / 1e9 if prof["ms"] else None
    bm25 = {"queries": len(bm_q), "device_ms_mean": statistics.mean(bm_ms), "device_ms_p50": _pct(bm_ms, 50),
            "postings_per_query": bm_post / len(bm_q), "term_kernel_gbs": bm25_gbs,
            "term_kernel_frac": (bm25_gbs / peaks["hbm_gbs"]) if bm25_gbs else None,
            "term_kernel_launches": prof["launches"]}

    # warm both arms (allocations, first launches)
    arr, qs = make_stream(2000.0, 200)
    served(arr, qs)
    plain(arr, qs)
    results = []
    for rate in rates:
        nq = int(min(max(rate * seconds, 200), 20_000))
        arr, qs = make_stream(rate, nq)
        sv, _ = served(arr, qs)
        pl = plain(arr, qs)
        results.append({"offered_rate": rate, "queries": nq, "served": sv, "plain": pl,
                        "x_plain_qps": sv["qps"] / pl["qps"],
                        "mix": {k: sum(1 for q in qs if q[0] == k) for k in ("bfs", "sssp", "bm25")}})
    info = S.info()
    S.free()
    top = results[-1]
    return {"workload": f"served stream: BFS/SSSP over R-MAT s{scales[0]}/s{scales[1]}/s{scales[2]} + BM25 top-10 "
                        f"over {D} docs x {T} terms ({postings} postings); Poisson arrivals",
            "rates": results, "lanes": lanes, "hbm_budget_bytes": budget, "hbm_used_bytes": info["used_bytes"],
            "bm25_alone": bm25, "setup_s": round(setup_s, 1),
            "qps_at_top_rate": top["served"]["qps"], "x_plain_at_top_rate": top["x_plain_qps"],
            "p50_ms_at_top_rate": top["served"]["p50_ms"], "p99_ms_at_top_rate": top["served"]["p99_ms"]}


def serve_line(args, rank, world, local) -> dict | None:
    """The served stream alone at the offered rates of --serve-rates."""
    import torch
    torch.cuda.set_device(local)
    rates = [float(x) for x in args.serve_rates.split(",")]
    with ClockSampler(local) as clocks:
        clocks.start_timed()
        res = serve_measure(args, rates, args.serve_seconds)
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": res["qps_at_top_rate"], "unit": "queries/s", "n_gpus": world,
        "steps": len(rates), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 frontier words / u32 distances / f32 BM25",
        "data": "synthetic (seeded R-MAT, Zipf corpus)", "config": res, "e2e": None, "clocks": clocks.summary(),
    }


def next_line(args, rank, world, local) -> dict | None:
    """The widened apps: LM top-10 queries over the serve line's corpus (8M
    docs x 1M terms, ~50 terms per doc, Zipf 1.1 queries of 2-8 terms), the
    degree app on R-MAT s22 (directed), graph simulation on R-MAT s20 (data
    graph reversed, 6 labels, a 5-vertex query with a cycle).  A step = 100
    LM queries + one degree call + one graph simulation.  value = LM queries/s
    from device time; e2e = the same calls timed on the host clock."""
    import ctypes as C
    import numpy as np
    import torch
    import la3_gb300 as L
    import la3_gb300.build as B
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    small = args.scale != SCALE
    D, T, tpd = (100_000, 20_000, 30) if small else (8_000_000, 1_000_000, 50)
    t_setup = time.time()
    eb = L.EdgeList.bipartite(D, T, tpd, seed=300)
    postings = eb.m
    gb = L.Graph.from_edges(eb, L.BIPARTITE | L.WEIGHTED, D, T)
    del eb
    gb.set_stream(stream.cuda_stream)
    t0 = time.time()
    lm = L.LM(gb)
    lm_prepare_s = time.time() - t0
    lm.query([], 0)  # the first query's leftover term activity
    rng = np.random.default_rng(500 + rank)
    zipf_w = 1.0 / np.arange(1, T + 1) ** 1.1
    zipf_w /= zipf_w.sum()

    def queries(n):
        return [sorted(set(int(D + 1 + t) for t in rng.choice(T, int(rng.integers(2, 9)), p=zipf_w)))
                for _ in range(n)]

    gd = L.Graph.from_edges(L.EdgeList.rmat(args.scale, 16, seed=GRAPH_SEED), L.DIRECTED)
    gd.set_stream(stream.cuda_stream)
    gs_scale = args.tc_scale
    gr = L.Graph.from_edges(L.EdgeList.rmat(gs_scale, 16, seed=GRAPH_SEED + 7), L.DIRECTED | L.REVERSE)
    gr.set_stream(stream.cuda_stream)
    vlab = np.zeros(gr.nslots, np.uint32)
    vlab[: 1 << gs_scale] = rng.integers(1, 7, 1 << gs_scale)  # 6 labels, vertex n unlabelled
    qlab = np.array([1, 2, 3, 2, 4], np.uint32)
    qedges = np.array([[0, 1], [1, 2], [2, 3], [3, 1], [1, 4]], np.uint32).reshape(-1)
    progs = C.CDLL(str(B.PROGRAMS_LIB))
    u32p = C.POINTER(C.c_uint32)
    progs.la3gp_graphsim.argtypes = [C.c_void_p, u32p, C.c_uint32, u32p, u32p, C.c_uint32, C.POINTER(C.c_uint8),
                                     C.c_char_p, u32p, u32p]
    matched = np.empty(gr.nslots, np.uint8)
    # TC as the reference writes it, through the generic engine (neighbour
    # lists as variable-size messages), on the plain bench's TC graph
    et = L.EdgeList.rmat(args.tc_scale, 16, seed=TC_SEED)
    gt = L.Graph.from_edges(et, L.DIRECTED | L.ACYCLIC)
    gtr = L.Graph.from_edges(et, L.DIRECTED | L.ACYCLIC | L.REVERSE)
    del et
    gt.set_stream(stream.cuda_stream)
    gtr.set_stream(stream.cuda_stream)
    progs.la3gp_tc.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    setup_s = time.time() - t_setup

    def tc_engine():
        tot = C.c_uint64()
        th = time.perf_counter()
        L.N.check(progs.la3gp_tc(gt._h, gtr._h, C.byref(tot), None))
        return tot.value, time.perf_counter() - th

    def graphsim():
        nm, it = C.c_uint32(), C.c_uint32()
        L.N.check(progs.la3gp_graphsim(gr._h, vlab.ctypes.data_as(u32p), qlab.size, qlab.ctypes.data_as(u32p),
                                       qedges.ctypes.data_as(u32p), qedges.size // 2,
                                       matched.ctypes.data_as(C.POINTER(C.c_uint8)), None, C.byref(nm), C.byref(it)))
        return nm.value, it.value

    def step(qs):
        lm_dev, lm_post = [], 0
        th = time.perf_counter()
        for q in qs:
            _, _, _, st = lm.query(q, 10)
            lm_dev.append(st.device_ms)
            lm_post += st.edges_examined
        lm_host = time.perf_counter() - th
        _, _, _, dst = L.degree(gd, 3)
        th = time.perf_counter()
        nm, it = graphsim()
        gs_s = time.perf_counter() - th
        return lm_dev, lm_post, lm_host, dst.device_ms, gs_s, nm, it

    for _ in range(args.warmup):
        step(queries(20))
    tc_engine()
    tc_runs = [tc_engine() for _ in range(3)]
    tc_lib, _, _ = L.tc(gt, False)
    torch.cuda.synchronize()
    L.profile_reset()
    L.profile(True)
    res = []
    with ClockSampler(local) as clocks:
        clocks.start_timed()
        for _ in range(args.steps):
            res.append(step(queries(100)))
    L.profile(False)
    prof = L.profile_report().get("lm_term", {"ms": 0.0, "bytes": 0.0, "launches": 0})
    peaks = measured_peaks()
    lm_dev = [x for r in res for x in r[0]]
    lm_host = sum(r[2] for r in res)
    lm_gbs = prof["bytes"] / (prof["ms"] / 1e3) / 1e9 if prof["ms"] else None
    deg_ms = statistics.median(r[3] for r in res)
    gs_s = statistics.median(r[4] for r in res)
    nq = len(lm_dev)
    if rank != 0:
        return None
    return {
        "metric": "LM queries/s on 1 GB300 (8M-doc corpus); degree and graph-simulation rates", "value": nq /
        (sum(lm_dev) / 1e3), "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(lm_dev) / args.steps + deg_ms + gs_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 LM scores / u32 degrees / u32 masks", "data": "synthetic (seeded)",
        "config": {"workload": f"LM top-10 over {D} docs x {T} terms ({postings} postings); degree on R-MAT "
                               f"s{args.scale}; graph simulation on R-MAT s{gs_scale} (5-vertex query, 6 labels)",
                   "lm": {"queries": nq, "device_ms_mean": statistics.mean(lm_dev),
                          "device_ms_p50": _pct(lm_dev, 50), "device_ms_p99": _pct(lm_dev, 99),
                          "postings_per_query": sum(r[1] for r in res) / nq, "term_kernel_gbs": lm_gbs,
                          "term_kernel_frac": (lm_gbs / peaks["hbm_gbs"]) if lm_gbs else None,
                          "prepare_s": round(lm_prepare_s, 2)},
                   "degree": {"device_ms": deg_ms, "gteps": gd.info.nentries / (deg_ms / 1e3) / 1e9},
                   "graphsim": {"ms": gs_s * 1e3, "iterations": res[-1][6], "matches": res[-1][5],
                                "edge_passes_per_s": res[-1][6] * gr.info.nentries / gs_s},
                   "tc_engine": {"ms": statistics.median(t for _, t in tc_runs) * 1e3,
                                 "triangles": tc_runs[-1][0], "equals_la3g_tc": tc_runs[-1][0] == tc_lib,
                                 "graph": f"R-MAT s{args.tc_scale}, host clock incl. the Gn list build"},
                   "setup_s": round(setup_s, 1), "peak_source": peaks.get("source", "measured")},
        "e2e": {"value": nq / lm_host, "unit": "queries/s", "h2d_bytes_per_step": 4 * 5 * 100,
                "d2h_bytes_per_step": 8 * 10 * 100},
        "clocks": clocks.summary(),
    }


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
    fn = {"plain": gpu_line, "batched": batched_line, "precision": precision_line, "serve": serve_line,
          "next": next_line}[args.workload]
    line = fn(args, rank, world, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
