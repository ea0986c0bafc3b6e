"""Golden outputs of the reference's format tools (tools/mtx2bin.cpp,
tools/bin2mtx.cpp), built from its sources by `make -C oracle stage ref`.
Writes tests/golden/tools/: the inputs, then one output per (tool, flags)
case, named <case>.out, plus cases.json.  Run here (where the reference
checkout is); the fixtures are committed and the tests only read them."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = ROOT / "tests" / "golden" / "tools"
BIN = ROOT / "oracle" / "_ref" / "bin"


def main() -> int:
    OUT.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(11)
    n, m = 40, 120
    src = rng.integers(1, n + 1, m)
    dst = rng.integers(1, n + 1, m)
    w = rng.integers(1, 200, m)
    # Matrix Market-like text inputs
    pairs = "".join(f"{a} {b}\n" for a, b in zip(src, dst))
    triples = "".join(f"{a} {b} {c}\n" for a, b, c in zip(src, dst, w))
    (OUT / "pairs.mtx").write_text("% a comment\n# another\n" + pairs)
    (OUT / "pairs_hdr.mtx").write_text(f"{n} {n} {m}\n" + pairs)
    (OUT / "triples.mtx").write_text("%%MatrixMarket coordinate\n" + triples)
    (OUT / "triples_dbl.mtx").write_text("".join(f"{a} {b} {c / 4}\n" for a, b, c in zip(src, dst, w)))
    # binary inputs
    np.stack([src, dst], 1).astype(np.uint32).tofile(OUT / "pairs.bin")
    np.stack([src, dst, w], 1).astype(np.uint32).tofile(OUT / "triples.bin")
    hdr = np.array([n, n], np.uint32).tobytes() + np.array([m], np.uint64).tobytes()
    (OUT / "pairs_hdr.bin").write_bytes(hdr + np.stack([src, dst], 1).astype(np.uint32).tobytes())
    cases = {
        "m2b_pairs": ["mtx2bin", "pairs.mtx", []],
        "m2b_pairs_woi": ["mtx2bin", "pairs.mtx", ["-woi"]],
        "m2b_pairs_wod": ["mtx2bin", "pairs.mtx", ["-wod"]],
        "m2b_hdr_hio": ["mtx2bin", "pairs_hdr.mtx", ["-hio"]],
        "m2b_hdr_hi": ["mtx2bin", "pairs_hdr.mtx", ["-hi"]],
        "m2b_triples_wi_woi": ["mtx2bin", "triples.mtx", ["-wi", "-woi"]],
        "m2b_triples_wi": ["mtx2bin", "triples.mtx", ["-wi"]],
        "m2b_dbl_wi_wod": ["mtx2bin", "triples_dbl.mtx", ["-wi", "-wod"]],
        "m2b_dbl_wi_woi": ["mtx2bin", "triples_dbl.mtx", ["-wi", "-woi"]],
        "b2m_pairs": ["bin2mtx", "pairs.bin", []],
        "b2m_pairs_wo": ["bin2mtx", "pairs.bin", ["-wo"]],
        "b2m_pairs_wor": ["bin2mtx", "pairs.bin", ["-wor"]],
        "b2m_triples_wi_wo": ["bin2mtx", "triples.bin", ["-wi", "-wo"]],
        "b2m_triples_wi": ["bin2mtx", "triples.bin", ["-wi"]],
        "b2m_hdr_hio": ["bin2mtx", "pairs_hdr.bin", ["-hio"]],
        "b2m_hdr_hi_wo": ["bin2mtx", "pairs_hdr.bin", ["-hi", "-wo"]],
    }
    for name, (tool, inp, flags) in cases.items():
        out = OUT / f"{name}.out"
        subprocess.run([str(BIN / tool), str(OUT / inp), str(out)] + flags, check=True, capture_output=True)
    (OUT / "cases.json").write_text(json.dumps(cases, indent=1))
    print(f"{len(cases)} cases written to {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
