#!/usr/bin/env python
"""Generate the golden fixtures in tests/golden/<case>/ from the reference
program itself.

Runs oracle/_ref/ref_fdtd2d (the reference's own sources built for the CPU by
oracle/ref_build.py; needs the reference tree, so this runs only where it is
mounted) on each case's Settings.ini and keeps:

  Settings.ini     the input
  setup.npz        setup tables and maps the reference computed (CPML b/c,
                   denominators, material tables, ID maps, array positions,
                   SourceP, dt, chirp parameters)
  state.npz        final Ez/Hx/Hy/Jz, CPML psi arrays, detector traces and the
                   wave-front tracker rows, in the reference's layouts
  *.txt            the output files the reference wrote

Usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))
from refdump import read_dump  # noqa: E402

REF_BIN = ROOT / "oracle" / "_ref" / "ref_fdtd2d"

KEEP_TEXT = ["Detect.txt", "detAll.txt", "detEz.txt", "detHx.txt", "detHy.txt", "RC_Line.txt",
             "TAU_Line.txt", "SourceP.txt", "FieldSaveDat.txt", "Ez.txt", "RcDet_data.txt",
             "SD.txt", "CF.txt", "ARC.txt", "det_SD.txt", "det_CF.txt", "det_ARC.txt",
             "Detect_S2D.txt", "detAll_S2D.txt", "detEz_S2D.txt", "detHx_S2D.txt", "detHy_S2D.txt",
             "DifDetEx.txt"]

BASE = """;golden case {name}
[hardware]
GPU_device=0
[regimes]
SourceToDetect = {s2d}
[grid]
Use_Exp_time = 1
Imax = {imax}
Jmax = {jmax}
Max_time = 400
Exp_time = {exp}
ds = {ds}
dt_coef = 0.5
Isource = {isrc}
Jsource = 10
Idetect = {isrc}
Jdetect = 14
[AESA]
SIsize = 10
SAutoDelta = 0
SIdelta = 2
SPAngle = {angle}
DIsize = 10
DAutoDelta = 0
DIdelta = 2
[PulseParam]
Chirp={chirp}
FreqA=38
FreqB=30
Fronts_ns=0.05
Plato_ns=0.05
Pulse_amp = 1881
[2Dsave]
From=0
To={save_to}
TimeSieve={sieve}
GridSieve=3
[medium]
Build={build}
Icen={isrc}
Jcen={jcen}
A=2
B=1
C=1
P=1
Q=1
N=1
Radius=25
Alpha=2.0
Beta=1.0
ne0=5.5e+19
neA=0
TorusBR=20
[mediumFluc]
FlucBuild={fluc}
FlucIcen={fluci}
FlucJcen={flucj}
FlucAngleK=30
FlucRadius=8
FlucAlpha=2
FlucBeta=1
FlucNe0=1.028e+19
[KameraConf]
DrawWall={wall}
WallPos={wallpos}
[RC_calc]
Iline = {isrc}
LIsize = 10
LIdelta = 5
FilterWindow = 20
Rlevel = 0.07
{extra}
"""

PROCESSING = """[Processing]
Perform = 1
SecDer = 1
SDFType = 1
SDFRuns = 1
CF = 1
CFTau = 30
CFK = -0.5
ARC = 1
ARCTau = 20
ARCK = -0.6
FilterType = 1
FilterRuns = 2
FilterWin = 9
SaveFiltered = 1
SaveOriginal = 1
PosI = 0
PosJ = 1
SizeI = 30
TauThreshold = 0.25
DetSize = 6
DetSim = 1
DetSave = 1
DetWLoad = 0
DimSieve = 2
TimeSieve = 5
BeginAfter = 0
FinishAt = 1
"""

CASES = {
    # sphere + rotated fluctuation, chirped source, steered array, small grid
    # (the reference's launch grids leave CPML cells out here)
    "sphere_fluc_chirp": dict(imax=60, jmax=110, exp=0.25, isrc=30, angle=5, chirp=1, save_to=300,
                              sieve=150, build=1, jcen=80, fluc=2, fluci=25, flucj=70, wall=0,
                              wallpos=950, extra=""),
    # torus medium, steel wall, unchirped, TOF post-processing on
    "torus_wall_tof": dict(imax=64, jmax=128, exp=0.3, isrc=32, angle=0, chirp=0, save_to=-1,
                           sieve=100, build=2, jcen=90, fluc=0, fluci=0, flucj=0, wall=1,
                           wallpos=220, extra=PROCESSING),
    # longer run on a wider grid (full launch coverage) so the wave-front
    # tracker and TAU search (which starts at step 2000) see a real front
    "long_rc": dict(imax=100, jmax=220, exp=1.2, isrc=50, angle=0, chirp=0, save_to=-1, sieve=100,
                    build=1, jcen=190, fluc=0, fluci=0, flucj=0, wall=0, wallpos=950, extra=""),
    # ds = 1 mm so PosJ = 1 is cell row 1, the only row Dev_SaveLine copies:
    # the TOF estimators run on a real saved line
    "tof_line": dict(ds=1.0, imax=80, jmax=120, exp=0.6, isrc=40, angle=0, chirp=0, save_to=-1,
                     sieve=100, build=1, jcen=100, fluc=0, fluci=0, flucj=0, wall=0, wallpos=950,
                     extra=PROCESSING),
    # SourceToDetect: a vacuum run (no medium, no wall) then the run with the
    # medium; the wall is asked for but the reference never builds it in this
    # mode; difference traces in DifDetEx.txt
    "s2d_sphere": dict(s2d=1, imax=60, jmax=110, exp=0.3, isrc=30, angle=5, chirp=0, save_to=-1,
                       sieve=100, build=1, jcen=70, fluc=2, fluci=25, flucj=60, wall=1,
                       wallpos=180, extra=""),
}


def make_case(name: str, params: dict) -> None:
    out = HERE / name
    out.mkdir(exist_ok=True)
    ini = BASE.format(name=name, **{"ds": 0.5, "s2d": 0, **params})
    with tempfile.TemporaryDirectory() as td:
        run = Path(td)
        (run / "Settings.ini").write_text(ini)
        subprocess.run([str(REF_BIN), str(run)], check=True, stdout=subprocess.DEVNULL)
        d = read_dump(run / "ref_dump.bin")
        imax, jmax, nmax, _ = (int(v) for v in d["scalars"])
        setup_keys = [k for k in d if k not in ("detect", "det_Ez", "det_Hx", "det_Hy", "PspdLine", "Ez", "Hx",
                                                 "Hy", "Jz") and not k.startswith("psi_")]
        setup = {k: d[k] for k in setup_keys}
        for k in ("ID1", "ID2", "ID3"):
            setup[k] = d[k].astype(np.int16).reshape(jmax, imax)
        np.savez_compressed(out / "setup.npz", **setup)
        P = 11
        state = {"Ez": d["Ez"].reshape(jmax, imax), "Hx": d["Hx"].reshape(jmax - 1, imax),
                 "Hy": d["Hy"].reshape(jmax, imax - 1), "Jz": d["Jz"].reshape(jmax, imax),
                 "psi_Ezx_1": d["psi_Ezx_1"].reshape(jmax, P), "psi_Ezx_2": d["psi_Ezx_2"].reshape(jmax, P),
                 "psi_Hyx_1": d["psi_Hyx_1"].reshape(jmax, P - 1), "psi_Hyx_2": d["psi_Hyx_2"].reshape(jmax, P - 1),
                 "psi_Ezy_1": d["psi_Ezy_1"].reshape(P, imax), "psi_Ezy_2": d["psi_Ezy_2"].reshape(P, imax),
                 "psi_Hxy_1": d["psi_Hxy_1"].reshape(P - 1, imax), "psi_Hxy_2": d["psi_Hxy_2"].reshape(P - 1, imax),
                 "detect": d["detect"].reshape(nmax, -1), "det_Ez": d["det_Ez"].reshape(nmax, -1),
                 "det_Hx": d["det_Hx"].reshape(nmax, -1), "det_Hy": d["det_Hy"].reshape(nmax, -1),
                 "PspdLine": d["PspdLine"].reshape(nmax, -1)}
        np.savez_compressed(out / "state.npz", **state)
        (out / "Settings.ini").write_text(ini)
        for f in KEEP_TEXT:
            if name in ("long_rc", "s2d_sphere") and f in ("detEz.txt", "detHx.txt", "detHy.txt"):
                continue  # the same samples are in state.npz; keeps the fixture small
            src = run / f
            if src.exists() and src.stat().st_size > 0:
                shutil.copy(src, out / f)
    print(f"{name}: {imax}x{jmax}, {nmax} steps")


def main() -> int:
    if not REF_BIN.exists():
        print("build the reference first: python oracle/ref_build.py", file=sys.stderr)
        return 1
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make_case(n, CASES[n])
    return 0


if __name__ == "__main__":
    sys.exit(main())
