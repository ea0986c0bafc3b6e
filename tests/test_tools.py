"""mtx2bin / bin2mtx keep the reference tools' options and output bytes
(tools/mtx2bin.cpp:11-116, tools/bin2mtx.cpp:11-96): every committed case
produced by the reference tool is reproduced byte for byte.  No GPU."""
import json
import subprocess

import pytest

from conftest import GOLD

TOOLS = GOLD / "tools"


@pytest.fixture(scope="module")
def bins(native):
    import la3_gb300.build as B
    return B.BIN


@pytest.mark.parametrize("name", sorted(json.loads((TOOLS / "cases.json").read_text())))
def test_tool_matches_reference(bins, name, tmp_path):
    tool, inp, flags = json.loads((TOOLS / "cases.json").read_text())[name]
    out = tmp_path / "out"
    r = subprocess.run([str(bins / tool), str(TOOLS / inp), str(out)] + flags, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == (TOOLS / f"{name}.out").read_bytes(), name


def test_header_after_comments(bins, tmp_path):
    """The header line may follow comment lines (read from the first
    non-comment line)."""
    src = tmp_path / "g.mtx"
    src.write_text("% comment\n3 3 2\n1 2\n2 3\n")
    out = tmp_path / "g.bin"
    assert subprocess.run([str(bins / "mtx2bin"), str(src), str(out), "-hio"], capture_output=True).returncode == 0
    import numpy as np
    b = out.read_bytes()
    assert np.frombuffer(b[:8], np.uint32).tolist() == [3, 3] and np.frombuffer(b[8:16], np.uint64)[0] == 2
    assert np.frombuffer(b[16:], np.uint32).tolist() == [1, 2, 2, 3]


def test_usage(bins):
    r = subprocess.run([str(bins / "mtx2bin")], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout
