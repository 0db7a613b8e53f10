"""In-tree build of the native pieces (no cmake): the CUDA library
``fdtd_2d_gb300/libfdtd2d.so`` (sm_103a kernels + C ABI + host setup), the
drop-in executable ``fdtd_2d_gb300/fdtd2d``, and the CPU oracle
``oracle/liboracle.so`` used by the tests and the CPU baseline.

Run ``python -m fdtd_2d_gb300.build`` or call :func:`build`.  Translation units
compile in parallel; objects go to ``_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "fdtd_2d_gb300"
CSRC = PKG / "csrc"
ORACLE = ROOT / "oracle"
OBJ = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["step_kernels.cu", "step_tma.cu", "step_tmat.cu", "api.cu", "batch.cu", "noalloc.cu"]
HOST_SOURCES = ["problem.cpp", "ini.cpp", "driver.cpp", "processing.cpp"]
HOST_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fdtd_2d_gb300")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> dict[str, Path]:
    OBJ.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "fdtd2d.h"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = OBJ / (s.stem + ".cu.o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include"),
                         "-c", str(s), "-o", str(o)])
    for src in HOST_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", *HOST_FLAGS, "-I", str(ROOT / "include"), "-I",
                         "/usr/local/cuda/include", "-c", str(s), "-o", str(o)])
    oracle_so = ORACLE / "liboracle.so"
    oracle_deps = [ORACLE / "oracle.c", ORACLE / "oracle_impl.h", ROOT / "include" / "fdtd2d.h"]
    if force or _stale(oracle_so, oracle_deps):
        jobs.append(["gcc", "-std=c11", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
                     str(ORACLE / "oracle.c"), "-o", str(oracle_so), "-lm"])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for fut in [ex.submit(_run, j) for j in jobs]:
                fut.result()
    lib = PKG / "libfdtd2d.so"
    if force or jobs or not lib.exists():
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(lib), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    exe = PKG / "fdtd2d"
    main = CSRC / "main.cpp"
    if main.exists() and (force or _stale(exe, [main, lib])):
        _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(main), "-o", str(exe),
              "-L", str(PKG), "-lfdtd2d", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}, {exe}, {oracle_so}")
    return {"lib": lib, "exe": exe, "oracle": oracle_so}


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
