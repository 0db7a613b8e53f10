"""The host code under AddressSanitizer and UndefinedBehaviorSanitizer: the
problem builders, the Settings.ini parser and medium producers, the TOF and
wave-front post-processing, and the oracle, built from their sources with
-fsanitize=address,undefined and driven by tests/sanitize/harness.cpp over
edge sizes and the golden Settings.ini cases.  No GPU."""
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "fdtd_2d_gb300" / "csrc"
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.slow
def test_host_code_sanitized(tmp_path):
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compiler")
    flags = ["-O1", "-g", "-fsanitize=address,undefined,float-cast-overflow", "-fno-omit-frame-pointer", "-fopenmp",
             "-fno-sanitize-recover=undefined,float-cast-overflow"]
    obj = tmp_path / "oracle.o"
    r = subprocess.run(["gcc", "-std=c11", *flags, "-c", str(ROOT / "oracle" / "oracle.c"), f"-I{ROOT / 'include'}",
                        f"-I{ROOT / 'oracle'}", "-o", str(obj)], capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in (r.stderr or ""):
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    exe = tmp_path / "harness"
    r = subprocess.run(["g++", "-std=c++17", *flags, f"-I{CSRC}", str(Path(__file__).parent / "sanitize" / "harness.cpp"),
                        str(obj), str(CSRC / "problem.cpp"), str(CSRC / "ini.cpp"), str(CSRC / "processing.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in (r.stderr or "") or "ubsan" in (r.stderr or "")):
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    (tmp_path / "sanitize_out").mkdir()
    inis = [str(GOLDEN / c / "Settings.ini") for c in ("sphere_fluc_chirp", "torus_wall_tof", "tof_line")]
    # degenerate files: a sphere semi-axis of 0 (an infinite level, converted
    # as the reference's x86 build converts it) and a zero TOF window with the
    # processing switch commented out (refused by fdtd2d_write_tof)
    for name, case, edits in (("zero_axis.ini", "sphere_fluc_chirp", {"A": "0"}),
                              ("zero_window.ini", "tof_line", {"FilterWin": "0", "Perform": None})):
        text = (GOLDEN / case / "Settings.ini").read_text()
        for key, val in edits.items():
            repl = f";{key} = 1" if val is None else f"{key} = {val}"
            text, n = re.subn(rf"(?m)^{key}\s*=.*$", repl, text)
            assert n == 1, (name, key)
        (tmp_path / name).write_text(text)
        inis.append(str(tmp_path / name))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", OMP_NUM_THREADS="4")
    r = subprocess.run([str(exe), *inis], capture_output=True, text=True, cwd=tmp_path, env=env, timeout=600)
    out = r.stdout + r.stderr
    assert "AddressSanitizer" not in out and "runtime error" not in out, out[-4000:]
    assert r.returncode == 0 and "SANITIZE OK" in r.stdout, out[-4000:]


@pytest.mark.slow
def test_driver_host_code_sanitized(tmp_path):
    """fdtd2d_run_settings end to end under ASan/UBSan on golden Settings.ini
    cases (wave-front lines, TOF window, torus and wall, S2D second shot),
    with the device entry points replaced by a host stand-in
    (tests/sanitize/driver_harness.cpp): the parsing, the run schedule and
    every writer of the drop-in driver."""
    if not shutil.which("g++"):
        pytest.skip("no host compiler")
    exe = tmp_path / "driver_harness"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
                        "-fno-sanitize-recover=undefined", "-fopenmp", f"-I{CSRC}",
                        str(Path(__file__).parent / "sanitize" / "driver_harness.cpp"), str(CSRC / "driver.cpp"),
                        str(CSRC / "problem.cpp"), str(CSRC / "ini.cpp"), str(CSRC / "processing.cpp"), "-lpthread",
                        "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in (r.stderr or "") or "ubsan" in (r.stderr or "")):
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", OMP_NUM_THREADS="4")
    for case in ("long_rc", "tof_line", "torus_wall_tof", "s2d_sphere"):
        out = tmp_path / case
        out.mkdir()
        r = subprocess.run([str(exe), str(GOLDEN / case / "Settings.ini"), str(out)], capture_output=True, text=True,
                           env=env, timeout=600)
        log = r.stdout + r.stderr
        assert "AddressSanitizer" not in log and "runtime error" not in log, (case, log[-4000:])
        assert r.returncode == 0 and "DRIVER OK" in r.stdout, (case, log[-4000:])
        assert (out / "Detect.txt").exists() and (out / "log.txt").exists(), case
