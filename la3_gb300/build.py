"""Builds the native library and the app drivers in-tree.

    python -m la3_gb300.build            # libla3g.so + drivers
    python -m la3_gb300.build --clean

Everything is compiled for sm_103a only (`-gencode arch=compute_103a,
code=sm_103a`); translation units compile in parallel and link into
`la3_gb300/_build/libla3g.so`; the vertex programs of `la3_gb300/programs/`
(written against `include/la3g_vp.cuh`) link into `libla3g_programs.so`.  The drivers (`pr`, `bfs`, `sssp`, `cc`, `tc`,
`bm25`, `la3g_tool`) go to `la3_gb300/bin/`, and so does the host-only input
generator `la3g_gen` (`la3_gb300/tools/`, no CUDA and no libla3g).  Floating-point contraction is
disabled library-wide (`--fmad=false`, `-ffp-contract=off`) because the apps
reproduce the reference's arithmetic operation by operation.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
DRIVERS = PKG / "drivers"
TOOLS = PKG / "tools"
PROGRAMS = PKG / "programs"
BUILD = PKG / "_build"
BIN = PKG / "bin"
INCLUDE = ROOT / "include"
LIB = BUILD / "libla3g.so"
PROGRAMS_LIB = BUILD / "libla3g_programs.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]
CXX_FLAGS = ["-O3", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-pthread",
             "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def cuda_lib_dir() -> Path:
    root = Path(nvcc()).resolve().parent.parent
    for d in (root / "lib64", root / "targets" / "sbsa-linux" / "lib", root / "targets" / "x86_64-linux" / "lib"):
        if (d / "libcudart_static.a").exists() or (d / "libcudart.so").exists():
            return d
    return root / "lib64"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    if _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"])
    build_programs()
    build_drivers()
    build_tools()
    return LIB


def build_programs() -> None:
    """Vertex programs written against include/la3g_vp.cuh, linked to libla3g."""
    srcs = sorted(PROGRAMS.glob("*.cu"))
    if not srcs:
        return
    deps = srcs + [LIB, INCLUDE / "la3g.h", INCLUDE / "la3g_vp.cuh", INCLUDE / "la3g_programs.h"]
    if _stale(PROGRAMS_LIB, deps):
        _run([nvcc()] + NVCC_FLAGS + ["-shared", "-o", str(PROGRAMS_LIB)] + [str(x) for x in srcs]
             + ["-L", str(BUILD), "-lla3g", "-Xlinker", "-rpath,$ORIGIN"])


def build_drivers() -> None:
    BIN.mkdir(exist_ok=True)
    srcs = sorted(DRIVERS.glob("*.cpp"))
    common = [p for p in srcs if p.stem == "driver_common"]
    jobs = []
    for src in srcs:
        if src.stem == "driver_common":
            continue
        out = BIN / src.stem
        deps = [src, LIB] + common + sorted(DRIVERS.glob("*.h")) + [INCLUDE / "la3g.h"]
        # drivers of apps written as vertex programs link libla3g_programs too
        progs = "la3g_programs.h" in src.read_text()
        if progs:
            deps += [PROGRAMS_LIB, INCLUDE / "la3g_programs.h"]
        if _stale(out, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-I", str(INCLUDE), "-I", str(DRIVERS), str(src)]
                        + [str(c) for c in common]
                        + ["-o", str(out), "-L", str(BUILD)] + (["-lla3g_programs"] if progs else [])
                        + ["-lla3g", "-Wl,-rpath,$ORIGIN/../_build", "-pthread"])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for f in [ex.submit(_run, c) for c in jobs]:
            f.result()


def build_tools() -> None:
    """Host-only tools: compiled from their own sources (and the generator's),
    linked to neither CUDA nor libla3g."""
    BIN.mkdir(exist_ok=True)
    gen = CSRC / "gen.cpp"
    for src in sorted(TOOLS.glob("*.cpp")):
        out = BIN / src.stem
        deps = [src, gen, INCLUDE / "la3g.h", CSRC / "la3g_internal.h"]
        if _stale(out, deps):
            _run(["g++"] + CXX_FLAGS + [str(src), str(gen), "-o", str(out)])


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(BIN, ignore_errors=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    if a.clean:
        clean()
    else:
        print(build(verbose=a.verbose))
