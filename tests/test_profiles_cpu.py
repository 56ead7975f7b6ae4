"""The ncu summaries under profiles/: each carries the per-launch DRAM traffic
bench.py reads for its roofline, and every ncu command in them leaves the GPU
clocks alone (--clock-control none) and runs committed files only."""
import glob
import os

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FILES = sorted(glob.glob(os.path.join(REPO, "profiles", "*.txt")))


def _ncu_commands(text):
    """The ncu command lines of a summary, backslash continuations joined."""
    cmds, cur = [], None
    for raw in text.splitlines():
        line = raw.lstrip("#").strip()
        if cur is None and not (line.startswith("ncu --") or "&& ncu --" in line):
            continue
        piece = line[:-1].strip() if line.endswith("\\") else line
        cur = piece if cur is None else cur + " " + piece
        if not line.endswith("\\"):
            cmds.append(cur)
            cur = None
    return cmds


def test_there_are_summaries():
    assert len(FILES) >= 10


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_summary_traffic_and_commands(path):
    text = open(path).read()
    traffic = [l for l in text.splitlines() if l.startswith("traffic_bytes_per_launch:")]
    assert len(traffic) == 1, "one traffic line"
    assert int(float(traffic[0].split(":", 1)[1])) > 0
    cmds = _ncu_commands(text)
    assert cmds, "the command that made the summary"
    for c in cmds:
        assert "--clock-control none" in c, c
        assert "_work" not in c and "/root/" not in c, c
        assert "bench.py" in c, c
