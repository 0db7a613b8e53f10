"""Kernel choices persisted across processes (the JSON file of
fdtd2d_clear_kernel_choices' header note): a first process times the shot's
class at create and writes the file; a second process reads it and creates
the same kind of shot without timing, with the same kernel choice."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = """
import fdtd_2d_gb300 as F
p = F.Problem.from_spec(nx=2304, ny=1536, npml=20, n_steps=40, src_i=60, src_j=700, det_i=62, det_j=700)
for k in range(2):
    with F.Shot(p, 0) as s:
        s.run(1, 40)
        s.synchronize()
        print(s.choice_source(), s.kernel_name())
"""


def _run(env):
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln.split(" ", 1) for ln in r.stdout.strip().splitlines()]


def test_choices_persist_across_processes(gpu, tmp_path):
    cache = tmp_path / "sub" / "choices.json"
    env = {k: v for k, v in os.environ.items() if not k.startswith("FDTD2D_")}
    env["FDTD2D_TUNE_CACHE"] = str(cache)
    first = _run(env)
    assert first[0][0] == "0"            # timed at create, file written
    assert first[1][0] == "1"            # the same process keeps it
    doc = json.loads(cache.read_text())
    assert doc["fdtd2d_kernel_choices"] == 1 and doc["choices"]
    second = _run(env)
    assert second[0][0] == "2"           # a new process reads the file
    assert second[0][1] == first[0][1]   # and makes the same choice
    # an entry written by another version of the timing is not used
    text = cache.read_text()
    assert "|v2|" in text
    cache.write_text(text.replace("|v2|", "|v1|"))
    assert _run(env)[0][0] == "0"
    env["FDTD2D_TUNE_CACHE"] = "0"       # memory only: timed again
    assert _run(env)[0][0] == "0"
