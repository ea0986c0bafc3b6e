"""Generates the golden vectors under tests/golden from the LA3 reference itself.

The reference is built from its own sources with the single-rank MPI
stand-in (`make -C oracle stage ref`, needs the reference checkout); its
dump drivers (oracle/refdump) replay each app's run() and write every
per-vertex result.  This script:

  1. copies the reference's own sample graphs (data/graph_analytics/g1_*,
     data/information_retrieval/g2_*) — the only known-answer inputs it
     ships — into tests/golden/data/;
  2. writes small seeded synthetic inputs (R-MAT, Erdos-Renyi, a bipartite
     corpus, and edge cases: duplicates, self-loops, vertex 0 with edges,
     a path deeper than 255 hops) with the la3_gb300 generators;
  3. runs the reference dump drivers on every case and stores the outputs as
     <case>.npz plus a manifest (golden.json).

Run it from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
GOLD = ROOT / "tests" / "golden"
DATA = GOLD / "data"
# the reference checkout whose sample data are copied (LA3_REFERENCE overrides it)
REFDATA = Path(os.environ.get("LA3_REFERENCE", "/root/reference")) / "data"
REF_BIN = ROOT / "oracle" / "_ref" / "bin"

sys.path.insert(0, str(ROOT))


def run_dump(args: list[str]) -> dict:
    r = subprocess.run([str(a) for a in args], capture_output=True, text=True, check=True,
                       env={"OMP_NUM_THREADS": "2", "PATH": "/usr/bin:/bin"})
    for line in reversed(r.stdout.splitlines()):
        if line.startswith("{"):
            return json.loads(line)
    raise RuntimeError("no JSON line from " + " ".join(map(str, args)))


def load(prefix: Path, suffix: str, dtype) -> np.ndarray:
    return np.fromfile(str(prefix) + suffix, dtype=dtype)


def write_records(path: Path, recs: list[tuple], weighted: bool) -> None:
    a = np.array(recs, dtype=np.uint32).reshape(-1, 3 if weighted else 2)
    a.tofile(path)


def main() -> None:
    only_lm = "--only-lm" in sys.argv  # regenerate the LM cases alone (other fixtures untouched)
    only_gs = "--only-gs" in sys.argv  # regenerate the graph-simulation cases alone
    if not (REF_BIN / "dump_pr").exists():
        sys.exit("build the reference first: make -C oracle stage ref")
    from la3_gb300 import EdgeList  # host-side generators; no GPU needed
    DATA.mkdir(parents=True, exist_ok=True)
    for f in ["graph_simulation/g3_13_13_20.bin", "graph_simulation/g3_13_13_20.labels"] + \
             [f"graph_simulation/{q}.{x}" for q in ("q1_4_4_6", "q2_4_4_4", "q3_4_4_6") for x in ("labels", "mtx")]:
        shutil.copy(REFDATA / f, DATA / Path(f).name)
    for f in ["graph_analytics/g1_8_8_13.bin", "graph_analytics/g1_8_8_13.w.bin",
              "information_retrieval/g2_7_7_17.w.bp.bin", "information_retrieval/g2_7_7_17.term.labels",
              "information_retrieval/g2_7_7_17.queries"]:
        shutil.copy(REFDATA / f, DATA / Path(f).name)

    # synthetic inputs
    EdgeList.rmat(10, 16, seed=11).write(DATA / "rmat10.bin")
    EdgeList.rmat(10, 16, seed=11, weighted=True, wseed=12).write(DATA / "rmat10.w.bin")
    EdgeList.rmat(12, 8, seed=21).write(DATA / "rmat12.bin")
    EdgeList.rmat(12, 8, seed=21, weighted=True, wseed=22).write(DATA / "rmat12.w.bin")
    EdgeList.er(1024, 8 * 1024, seed=31).write(DATA / "er10.bin")
    EdgeList.er(1024, 16 * 1024, seed=31, weighted=True, wseed=32).write(DATA / "er10.w.bin")
    EdgeList.bipartite(2000, 400, 12, seed=41).write(DATA / "bip.w.bp.bin")
    # edge cases
    rng = np.random.default_rng(5)
    recs = []
    for _ in range(600):
        s, d = rng.integers(0, 64, 2)
        recs.append((int(s), int(d), int(rng.integers(1, 50))))
    recs += [(3, 3, 7), (5, 9, 100), (5, 9, 1), (9, 5, 2), (0, 1, 4)]  # self-loop, dups, id 0
    write_records(DATA / "dups.w.bin", recs, True)
    write_records(DATA / "dups.bin", [r[:2] for r in recs], False)
    write_records(DATA / "path300.bin", [(i, i + 1) for i in range(1, 300)], False)
    write_records(DATA / "zero.bin", [(0, 5), (5, 3), (3, 7), (0, 2), (2, 9), (9, 1), (4, 6), (8, 8), (10, 4)],
                  False)
    # queries for the synthetic corpus: sorted unique, plus unsorted / duplicate ones
    ndocs, nterms = 2000, 400
    labels = DATA / "bip.term.labels"
    labels.write_text("".join(f"t{i} {i}\n" for i in range(1, nterms + 1)))
    qrng = np.random.default_rng(7)
    qlines = []
    for i in range(24):
        k = int(qrng.integers(2, 9))
        t = sorted(set(int(x) for x in qrng.integers(1, nterms + 1, k)))
        qlines.append(" ".join(f"t{x}" for x in t))
    qlines += ["t9 t3", "t3 t9", "t5 t5 t2", "t400 t1 t200", "tnope t7"]
    (DATA / "bip.queries").write_text("\n".join(qlines) + "\n")

    # LM corpus whose doc and term token sums pass 2^24, where the order of
    # the float additions shows in the result
    brng = np.random.default_rng(13)
    brecs = []
    for d in range(1, 61):
        for t in sorted(set(int(x) for x in brng.integers(1, 25, 9))):
            brecs.append((d, t, int(brng.integers(1, 3_000_000))))
    write_records(DATA / "bigtf.w.bp.bin", brecs, True)
    (DATA / "bigtf.term.labels").write_text("".join(f"b{i} {i}\n" for i in range(1, 25)))
    (DATA / "bigtf.queries").write_text("b1 b2\nb24 b7 b3\nb5\nb9 b9 b11\nb20 b1 b14 b6\n")

    # graph-simulation inputs: JSON-line labels over a small alphabet (vertex 0
    # without a label in one file), random small queries, some label files
    # ending in a newline (the reference then reads one more, empty, label)
    grng = np.random.default_rng(17)
    alphabet = ["A", "B", "C", "D", "E"]
    for gname, n, null0 in (("rmat10", 1024, False), ("er10", 1024, True)):
        lines = ["["]
        for i in range(n):
            lines.append("null," if (null0 and i == 0) else '{"t":"%s"},' % alphabet[int(grng.integers(0, 5))])
        lines.append("]")
        (DATA / f"{gname}.gs.labels").write_text("\n".join(lines) + "\n")
    gs_queries = []
    for qi in range(6):
        qn = int(grng.integers(3, 7))
        labs = [alphabet[int(grng.integers(0, 5))] for _ in range(qn)]
        if qi == 4:
            labs[1] = "Z"  # not in the data
        edges = sorted({(int(grng.integers(0, qn)), int(grng.integers(0, qn))) for _ in range(qn + 2)})
        edges = [e for e in edges if e[0] != e[1]] or [(0, 1)]
        trail = "\n" if qi % 2 else ""
        (DATA / f"gsq{qi}.labels").write_text("\n".join(labs) + trail)
        (DATA / f"gsq{qi}.mtx").write_text("\n".join(f"{a} {b}" for a, b in edges) + "\n")
        gs_queries.append(f"gsq{qi}")

    cases = {}
    tmp = Path(tempfile.mkdtemp())

    def gs_case(name, labels_f, f, n, ql_f, qm_f):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_graphsim", DATA / labels_f, DATA / f, n, DATA / ql_f, DATA / qm_f, o])
        q = meta["qsize"]
        res = np.fromfile(str(o) + ".res.u8", dtype=np.uint8).reshape(-1, q)
        np.savez_compressed(GOLD / f"{name}.npz", res=res, matched=load(o, ".matched.u8", np.uint8))
        cases[name] = {"app": "graphsim", "file": f, "labels": labels_f, "n": n, "qlabels": ql_f, "qmtx": qm_f,
                       **meta}

    def gs_cases():
        for q in ("q1_4_4_6", "q2_4_4_4", "q3_4_4_6"):
            gs_case(f"g3_{q}_gs", "g3_13_13_20.labels", "g3_13_13_20.bin", 13, f"{q}.labels", f"{q}.mtx")
        for k, qn in enumerate(gs_queries):
            gname = "rmat10" if k % 2 == 0 else "er10"
            gs_case(f"{gname}_{qn}_gs", f"{gname}.gs.labels", f"{gname}.bin", 1024, f"{qn}.labels", f"{qn}.mtx")

    if only_gs:
        gs_cases()
        old = json.loads((GOLD / "golden.json").read_text())
        old.update(cases)
        (GOLD / "golden.json").write_text(json.dumps(old, indent=1, sort_keys=True) + "\n")
        shutil.rmtree(tmp)
        print(f"{len(cases)} graph-simulation cases written to {GOLD}")
        return

    def pr_case(name, f, n, iters):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_pr", DATA / f, n, iters, o])
        np.savez_compressed(GOLD / f"{name}.npz", rank=load(o, ".rank.f64", np.float64),
                            degree=load(o, ".degree.u32", np.uint32))
        cases[name] = {"app": "pr", "file": f, "n": n, "iters": iters, **meta}

    def bfs_case(name, f, n, root):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_bfs", DATA / f, n, root, o])
        np.savez_compressed(GOLD / f"{name}.npz", hops=load(o, ".hops.u8", np.uint8),
                            parent=load(o, ".parent.u32", np.uint32))
        cases[name] = {"app": "bfs", "file": f, "n": n, "root": root, **meta}

    def sssp_case(name, f, n, root):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_sssp", DATA / f, n, root, o])
        np.savez_compressed(GOLD / f"{name}.npz", dist=load(o, ".dist.u32", np.uint32))
        cases[name] = {"app": "sssp", "file": f, "n": n, "root": root, **meta}

    def cc_case(name, f, n):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_cc", DATA / f, n, o])
        np.savez_compressed(GOLD / f"{name}.npz", label=load(o, ".label.u32", np.uint32))
        cases[name] = {"app": "cc", "file": f, "n": n, **meta}

    def tc_case(name, f, n):
        o = tmp / name
        meta = run_dump([REF_BIN / "dump_tc", DATA / f, n, o])
        np.savez_compressed(GOLD / f"{name}.npz", ntri=load(o, ".ntri.u32", np.uint32))
        cases[name] = {"app": "tc", "file": f, "n": n, **meta}

    def bm25_case(name, f, labels_f, ndocs, nterms, queries_f, k, app="bm25"):
        o = tmp / name
        meta = run_dump([REF_BIN / f"dump_{app}", DATA / f, DATA / labels_f, ndocs, nterms, DATA / queries_f, k, o])
        raw = np.fromfile(str(o) + ".queries.bin", dtype=np.uint32)
        i = 0
        arrays = {"length": load(o, ".length.f32", np.float32)}
        nq = 0
        while i < raw.size:
            na = int(raw[i]); i += 1
            pairs = raw[i:i + 2 * na].reshape(-1, 2); i += 2 * na
            nk = int(raw[i]); i += 1
            tk = raw[i:i + 2 * nk].reshape(-1, 2); i += 2 * nk
            arrays[f"q{nq}_ids"] = pairs[:, 0].copy()
            arrays[f"q{nq}_scores"] = pairs[:, 1].copy().view(np.float32)
            arrays[f"q{nq}_topk_ids"] = tk[:, 0].copy()
            arrays[f"q{nq}_topk_scores"] = tk[:, 1].copy().view(np.float32)
            nq += 1
        np.savez_compressed(GOLD / f"{name}.npz", **arrays)
        cases[name] = {"app": app, "file": f, "labels": labels_f, "queries": queries_f, "ndocs": ndocs,
                       "nterms": nterms, "k": k, **meta}

    def lm_cases():
        bm25_case("g2_lm", "g2_7_7_17.w.bp.bin", "g2_7_7_17.term.labels", 7, 7, "g2_7_7_17.queries", 3, app="lm")
        bm25_case("bip_lm", "bip.w.bp.bin", "bip.term.labels", ndocs, nterms, "bip.queries", 10, app="lm")
        bm25_case("bigtf_lm", "bigtf.w.bp.bin", "bigtf.term.labels", 60, 24, "bigtf.queries", 8, app="lm")

    if only_lm:
        lm_cases()
        old = json.loads((GOLD / "golden.json").read_text())
        old.update(cases)
        (GOLD / "golden.json").write_text(json.dumps(old, indent=1, sort_keys=True) + "\n")
        shutil.rmtree(tmp)
        print(f"{len(cases)} LM cases written to {GOLD}")
        return

    pr_case("g1_pr", "g1_8_8_13.bin", 8, 20)
    pr_case("g1_pr_conv", "g1_8_8_13.bin", 8, 0)
    bfs_case("g1_bfs", "g1_8_8_13.bin", 8, 5)
    sssp_case("g1_sssp", "g1_8_8_13.w.bin", 8, 5)
    cc_case("g1_cc", "g1_8_8_13.bin", 8)
    tc_case("g1_tc", "g1_8_8_13.bin", 8)
    bm25_case("g2_bm25", "g2_7_7_17.w.bp.bin", "g2_7_7_17.term.labels", 7, 7, "g2_7_7_17.queries", 3)

    pr_case("rmat10_pr", "rmat10.bin", 1024, 20)
    pr_case("rmat12_pr", "rmat12.bin", 4096, 20)
    pr_case("rmat12_pr_conv", "rmat12.bin", 4096, 0)
    for r in (1, 77, 1000):
        bfs_case(f"rmat10_bfs_{r}", "rmat10.bin", 1024, r)
        sssp_case(f"rmat10_sssp_{r}", "rmat10.w.bin", 1024, r)
    for r in (5, 4000):
        bfs_case(f"rmat12_bfs_{r}", "rmat12.bin", 4096, r)
        sssp_case(f"rmat12_sssp_{r}", "rmat12.w.bin", 4096, r)
    bfs_case("er10_bfs", "er10.bin", 1024, 3)
    sssp_case("er10_sssp", "er10.w.bin", 1024, 3)
    cc_case("rmat10_cc", "rmat10.bin", 1024)
    cc_case("rmat12_cc", "rmat12.bin", 4096)
    cc_case("er10_cc", "er10.bin", 1024)
    tc_case("rmat10_tc", "rmat10.bin", 1024)
    tc_case("rmat12_tc", "rmat12.bin", 4096)
    tc_case("er10_tc", "er10.bin", 1024)
    pr_case("dups_pr", "dups.bin", 64, 20)
    sssp_case("dups_sssp", "dups.w.bin", 64, 5)
    sssp_case("dups_sssp_root0", "dups.w.bin", 64, 0)
    bfs_case("dups_bfs", "dups.bin", 64, 9)
    cc_case("dups_cc", "dups.bin", 64)
    tc_case("dups_tc", "dups.bin", 64)
    cc_case("zero_cc", "zero.bin", 10)
    bfs_case("zero_bfs", "zero.bin", 10, 0)
    bfs_case("path300_bfs", "path300.bin", 300, 1)
    bfs_case("isolated_root_bfs", "rmat10.bin", 1024, 0)
    sssp_case("isolated_root_sssp", "rmat10.w.bin", 1024, 0)
    bm25_case("bip_bm25", "bip.w.bp.bin", "bip.term.labels", ndocs, nterms, "bip.queries", 10)
    lm_cases()
    gs_cases()

    (GOLD / "golden.json").write_text(json.dumps(cases, indent=1, sort_keys=True) + "\n")
    shutil.rmtree(tmp)
    print(f"{len(cases)} cases written to {GOLD}")


if __name__ == "__main__":
    main()
