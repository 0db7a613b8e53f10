#!/usr/bin/env python
"""Build the reference program for the CPU -- TEST INFRASTRUCTURE.

Compiles the reference's own sources where they lie (FDTD_2D_Full/kernel.cu,
FDTD_cuda.cu, processing.cu, INIlib/*) with g++ against the CUDA stand-in in
oracle/ref_shim/, plus oracle/ref_harness.cpp, into oracle/_ref/ref_fdtd2d.
Nothing is copied into the repository: two mechanical rewrites are generated
into oracle/_ref/ (git-ignored) because the sources do not compile as shipped:

  * kernel.cu: each launch `name<<<grid, block>>>(args);` becomes
    `EMU_LAUNCH(grid, block, name(args));` (serial loop over the threads);
  * Ext_kernel.cuh: `extern struct X {...};` (an MSVC extension) becomes
    `struct X {...};`.

Usage: python oracle/ref_build.py [/path/to/reference]
The reference tree is the argument, else $FDTD2D_REFERENCE, else the build
container's read-only mount point below.  It needs the reference sources, so
it runs only where they are mounted; build_if_present() (called by the
package build) skips it quietly elsewhere.
"""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
MOUNT_POINT = Path("/root/reference")   # where the build container mounts the reference


def reference_root(arg: str | None = None) -> Path:
    """The reference tree: `arg`, else $FDTD2D_REFERENCE, else the mount point."""
    import os

    if arg:
        return Path(arg)
    env = os.environ.get("FDTD2D_REFERENCE")
    return Path(env) if env else MOUNT_POINT


def strip_comments(src: str) -> str:
    """Drop // and /* */ comments outside string and character literals."""
    out = []
    i, n = 0, len(src)
    in_str = None
    while i < n:
        c = src[i]
        if in_str:
            out.append(c)
            if c == "\\" and i + 1 < n:
                out.append(src[i + 1])
                i += 2
                continue
            if c == in_str:
                in_str = None
            i += 1
        elif c in "\"'":
            in_str = c
            out.append(c)
            i += 1
        elif src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            i = n if j < 0 else j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def rewrite_launches(src: str) -> str:
    src = strip_comments(src)
    out = []
    i = 0
    while True:
        k = src.find("<<<", i)
        if k < 0:
            out.append(src[i:])
            break
        # kernel name: identifier right before <<<
        m = re.search(r"([A-Za-z_]\w*)\s*$", src[i:k])
        name_start = i + m.start(1)
        name = m.group(1)
        e = src.index(">>>", k)
        cfg = src[k + 3:e]
        p = src.index("(", e)
        depth, q = 0, p
        while True:
            if src[q] == "(":
                depth += 1
            elif src[q] == ")":
                depth -= 1
                if depth == 0:
                    break
            q += 1
        args = src[p + 1:q]
        semi = src.index(";", q)
        line_start = src.rfind("\n", 0, name_start) + 1
        prefix = src[line_start:name_start]
        commented = "//" in prefix
        out.append(src[i:name_start])
        if commented:
            out.append(src[name_start:semi + 1])
        else:
            parts = cfg.split(",")
            assert len(parts) == 2, cfg
            out.append(f"EMU_LAUNCH({parts[0].strip()}, {parts[1].strip()}, {name}({args}));")
        i = semi + 1
    return "".join(out)


def build_if_present() -> Path | None:
    """Build oracle/_ref/ref_fdtd2d when the reference sources are present
    and the binary is missing or older than the harness; None when absent."""
    ref = reference_root() / "FDTD_2D_Full"
    if not (ref / "kernel.cu").exists():
        return None
    exe = OUT / "ref_fdtd2d"
    deps = [HERE / "ref_harness.cpp", HERE / "ref_build.py", *(HERE / "ref_shim").glob("*.h")]
    if exe.exists() and all(d.stat().st_mtime <= exe.stat().st_mtime for d in deps):
        return exe
    return exe if compile_reference(ref) == 0 else None


def main() -> int:
    ref = reference_root(sys.argv[1] if len(sys.argv) > 1 else None) / "FDTD_2D_Full"
    if not (ref / "kernel.cu").exists():
        print(f"reference sources not found under {ref}", file=sys.stderr)
        return 1
    return compile_reference(ref)


def compile_reference(ref: Path) -> int:
    OUT.mkdir(exist_ok=True)
    (OUT / "kernel_emu.cu").write_text(rewrite_launches((ref / "kernel.cu").read_text(errors="replace")),
                                       errors="replace")
    ext = (ref / "Ext_kernel.cuh").read_text(errors="replace")
    (OUT / "Ext_kernel.cuh").write_text(re.sub(r"extern\s+struct", "struct", ext), errors="replace")
    common = ["-O2", "-ffp-contract=off", "-w", "-fpermissive", "-include", "cuda_runtime.h", f"-I{HERE}/ref_shim", f"-I{ref}",
              f"-I{ref}/INIlib"]
    jobs = [
        ["g++", "-x", "c++", "-std=c++14", *common, "-c", str(OUT / "kernel_emu.cu"), "-o", str(OUT / "kernel.o")],
        ["g++", "-x", "c++", "-std=c++14", *common, "-Dmain=ref_program_main", "-c", str(ref / "FDTD_cuda.cu"),
         "-o", str(OUT / "fdtd.o")],
        ["g++", "-x", "c++", "-std=c++14", *common, "-c", str(ref / "processing.cu"), "-o", str(OUT / "processing.o")],
        ["gcc", "-O2", "-w", "-c", str(ref / "INIlib" / "ini.c"), "-o", str(OUT / "ini.o")],
        ["g++", "-std=c++14", *common, "-c", str(ref / "INIlib" / "INIReader.cpp"), "-o", str(OUT / "inireader.o")],
        ["g++", "-std=c++14", "-O2", f"-I{HERE}", "-c", str(HERE / "ref_harness.cpp"), "-o", str(OUT / "harness.o")],
    ]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    ok = True
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            ok = False
            print(" ".join(j), "\n", out[-4000:], file=sys.stderr)
    if not ok:
        return 1
    objs = [str(OUT / n) for n in ("harness.o", "kernel.o", "fdtd.o", "processing.o", "ini.o", "inireader.o")]
    subprocess.run(["g++", *objs, "-o", str(OUT / "ref_fdtd2d")], check=True)
    print(OUT / "ref_fdtd2d")
    return 0


if __name__ == "__main__":
    sys.exit(main())
