"""The drop-in program (fdtd2d_run_settings: Settings.ini in, the reference's
files out) on the GPU against the reference program's own output files for
the same Settings.ini (tests/golden/, from the reference built for the CPU).

Text files are compared number by number: trace columns within relative L2
1e-5 (the reference's FP32 kernels and ours round differently, and both are
printed with 6 decimals); step counts, indices and layouts agree exactly.
"""
import re
from pathlib import Path

import numpy as np
import pytest

import fdtd_2d_gb300 as F
from helpers import FIELDS, PSI_FIELDS

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.name for p in GOLDEN.iterdir() if (p / "Settings.ini").exists())
NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?|nan|inf")


def numbers(path: Path) -> np.ndarray:
    return np.array([float(x) for x in NUM.findall(path.read_text())])


def table(path: Path) -> list[list[float]]:
    return [[float(x) for x in NUM.findall(line)] for line in path.read_text().splitlines() if line.strip()]


@pytest.fixture(scope="module", params=CASES)
def run(request, tmp_path_factory, gpu):
    case = request.param
    out = tmp_path_factory.mktemp(case)
    F.run_settings(GOLDEN / case / "Settings.ini", out, gpu)
    return case, out


def test_trace_files(run):
    case, out = run
    st = np.load(GOLDEN / case / "state.npz")
    # Column sums over the elements can nearly cancel (Hy is odd about the
    # array centre), so their error is scaled by the sum of |element samples|.
    mag = {"detect": np.abs(st["detect"]).sum(axis=1) * 1000, "Ez": np.abs(st["det_Ez"]).sum(axis=1) * 1000,
           "Hx": np.abs(st["det_Hx"]).sum(axis=1) * 1000, "Hy": np.abs(st["det_Hy"]).sum(axis=1) * 1000}
    for f in ("Detect.txt", "detAll.txt", "detEz.txt", "detHx.txt", "detHy.txt"):
        ref_f = GOLDEN / case / f
        if not ref_f.exists():
            continue
        mine, ref = table(out / f), table(ref_f)
        assert len(mine) == len(ref), f
        m = np.array([r for r in mine if r], dtype=float)
        r = np.array([r for r in ref if r], dtype=float)
        if f == "Detect.txt":
            m, r = m[:, :2], r[:, :2]   # third column: no argument in the reference's printf
        assert m.shape == r.shape, f
        den = np.linalg.norm(r, axis=0)
        if f == "Detect.txt":
            den[1] = np.linalg.norm(mag["detect"])
        if f == "detAll.txt":
            den[3], den[4], den[5] = (np.linalg.norm(mag[k]) for k in ("Ez", "Hx", "Hy"))
        # per column relative L2 (the trace tolerance); all-zero columns exact
        err = np.where(den > 0, np.linalg.norm(m - r, axis=0) / np.maximum(den, 1e-300),
                       np.abs(m - r).max(axis=0))
        assert np.all(err <= 1e-5), (f, err)
        if f in ("Detect.txt", "detAll.txt"):
            # time column: equal up to printf rounding
            assert np.allclose(m[:, 0], r[:, 0], rtol=0, atol=1.5e-6 * max(1.0, abs(r[:, 0]).max()))


def test_setup_files_exact(run):
    case, out = run
    for f in ("SourceP.txt", "FieldSaveDat.txt"):
        assert (out / f).read_text() == (GOLDEN / case / f).read_text(), f
    ref = (GOLDEN / case / "RcDet_data.txt").read_text().split()
    assert (out / "RcDet_data.txt").read_text().split() == ref


def test_field_slices(run):
    case, out = run
    ref_f = GOLDEN / case / "Ez.txt"
    if not ref_f.exists():
        pytest.skip("case saves no slices")
    m, r = numbers(out / "Ez.txt"), numbers(ref_f)
    assert m.shape == r.shape
    assert np.abs(m - r).max() <= 2e-5 * np.abs(r).max() + 2e-6


def test_wavefront_files(run):
    case, out = run
    m, r = table(out / "RC_Line.txt"), table(GOLDEN / case / "RC_Line.txt")
    assert len(m) == len(r)
    for a, b in zip(m, r):
        assert abs(a[0] - b[0]) <= 1 and abs(a[1] - b[1]) <= 1.0 + 1e-3 * abs(b[1])
    assert (out / "TAU_Line.txt").read_text() == (GOLDEN / case / "TAU_Line.txt").read_text()


def test_tof_files(run):
    case, out = run
    for f in ("SD.txt", "CF.txt", "ARC.txt", "det_SD.txt", "det_CF.txt", "det_ARC.txt"):
        ref_f = GOLDEN / case / f
        if not ref_f.exists():
            continue
        m, r = np.loadtxt(out / f), np.loadtxt(ref_f)
        assert m.shape == r.shape and np.array_equal(m[:, 0], r[:, 0]), f
        assert np.mean(np.abs(m[:, 1] - r[:, 1]) <= 1) >= 0.95, f


def test_source_to_detect_files(run):
    """SourceToDetect cases: the vacuum shot's *_S2D.txt files and the
    main - vacuum DifDetEx.txt against the reference's (per-element samples
    relative L2 <= 1e-5; sum columns within 1e-5 of the summed element
    magnitudes)."""
    case, out = run
    g = GOLDEN / case
    if not (g / "Detect_S2D.txt").exists():
        pytest.skip("not a SourceToDetect case")
    per = {}
    for f in ("detEz_S2D.txt", "detHx_S2D.txt", "detHy_S2D.txt"):
        m, r = numbers(out / f), numbers(g / f)
        assert m.shape == r.shape, f
        assert np.linalg.norm(m - r) <= 1e-5 * np.linalg.norm(r), f
        per[f[3:5]] = r.reshape(len(table(g / "Detect_S2D.txt")), -1)
    m, r = np.array(table(out / "Detect_S2D.txt")), np.array(table(g / "Detect_S2D.txt"))
    assert m.shape == r.shape
    assert np.abs(m[:, 0] - r[:, 0]).max() <= 1.5e-6 * max(1.0, np.abs(r[:, 0]).max())
    assert np.linalg.norm(m[:, 1] - r[:, 1]) <= 1e-5 * np.linalg.norm(np.abs(per["Ez"]).sum(1))
    m, r = np.array(table(out / "detAll_S2D.txt")), np.array(table(g / "detAll_S2D.txt"))
    assert m.shape == r.shape
    for c, k in ((3, "Ez"), (4, "Hx"), (5, "Hy")):
        assert np.linalg.norm(m[:, c] - r[:, c]) <= 1e-5 * np.linalg.norm(np.abs(per[k]).sum(1)), c
    st = np.load(g / "state.npz")
    main = {"Ez": st["det_Ez"] * 1000, "Hx": st["det_Hx"] * 1000, "Hy": st["det_Hy"] * 1000}
    m, r = np.array(table(out / "DifDetEx.txt")), np.array(table(g / "DifDetEx.txt"))
    assert m.shape == r.shape and not m[:, [1, 2, 6]].any()
    for c, k in ((3, "Ez"), (4, "Hx"), (5, "Hy")):
        mag = (np.abs(main[k]) + np.abs(per[k])).sum(1)
        assert np.linalg.norm(m[:, c] - r[:, c]) <= 1e-5 * np.linalg.norm(mag), c
    assert np.linalg.norm(m[:, 7] - r[:, 7]) <= 1e-5 * np.linalg.norm(r[:, 7])


def test_material_medium_as_uniform(gpu, monkeypatch, tmp_path):
    """A Settings.ini medium whose materials share CA/CB/DA/DB, with no PEC
    cell and the reference's launch coverage reaching every cell (the golden
    sphere-and-fluctuation case enlarged to 500 x 1200 cells) runs as the
    uniform medium on the staged kernels, with the material kernel's bits:
    fields, psi, detector traces and the wave-front tracker rows."""
    ini = (GOLDEN / "sphere_fluc_chirp" / "Settings.ini").read_text()
    for key, val in (("Imax", "250"), ("Jmax", "600"), ("Use_Exp_time", "0"), ("Max_time", "300")):
        ini = re.sub(rf"(?m)^{key}\s*=.*$", f"{key} = {val}", ini)
    path = tmp_path / "Settings.ini"
    path.write_text(ini)
    prob = F.Problem.from_ini(path)
    s = prob.setup
    assert (s.nx, s.ny) == (500, 1200) and s.n_rc > 0

    def stepped():
        with F.Shot(prob, gpu) as shot:
            name = shot.kernel_name()
            shot.run(1, prob.n_steps)
            out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
            out["det"] = shot.traces()["det_ez"]
            out["rc"] = shot.rc()
        return name, out

    monkeypatch.setenv("FDTD2D_PERSIST", "0")
    monkeypatch.setenv("FDTD2D_MATERIAL_AS_UNIFORM", "0")
    name0, ref = stepped()
    assert name0 == "step_stream_kernel<1>", name0
    monkeypatch.delenv("FDTD2D_MATERIAL_AS_UNIFORM")
    name1, got = stepped()
    assert name1.startswith("step_tma"), name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), k


def test_persistent_settings_ini(gpu, monkeypatch, tmp_path):
    """The persistent kernel on a Settings.ini shot (the golden
    sphere-and-fluctuation case at 500 x 1200 cells, 21 tracker lines, a
    line-probe window), in the material medium and as the uniform medium:
    fields, psi, traces, tracker rows and probe rows are the streaming
    material kernel's bits, the tracker and the probe running on service
    warps beside the next step.  Run calls of 1 to 170 steps."""
    ini = (GOLDEN / "sphere_fluc_chirp" / "Settings.ini").read_text()
    for key, val in (("Imax", "250"), ("Jmax", "600"), ("Use_Exp_time", "0"), ("Max_time", "300")):
        ini = re.sub(rf"(?m)^{key}\s*=.*$", f"{key} = {val}", ini)
    path = tmp_path / "Settings.ini"
    path.write_text(ini)
    prob = F.Problem.from_ini(path)
    s = prob.setup
    assert (s.nx, s.ny) == (500, 1200) and s.n_rc > 0
    s.line_n, s.line_i0, s.line_j, s.line_first, s.line_last = 400, 50, 700, 120, 180
    chunks = (1, 118, 3, 170, prob.n_steps - 292)
    assert chunks[-1] >= 1

    def stepped():
        with F.Shot(prob, gpu) as shot:
            name = shot.kernel_name()
            n = 1
            for c in chunks:
                shot.run(n, n + c - 1)
                n += c
            out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
            out["det"] = shot.traces()["det_ez"]
            out["rc"] = shot.rc()
            out["line"] = shot.line(120, 180)
        return name, out

    monkeypatch.setenv("FDTD2D_MATERIAL_AS_UNIFORM", "0")
    monkeypatch.setenv("FDTD2D_PERSIST", "0")
    name0, ref = stepped()
    assert name0 == "step_stream_kernel<1>", name0
    monkeypatch.setenv("FDTD2D_PERSIST", "1")
    name1, got = stepped()
    assert name1 == "step_persist_kernel<1>", name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), ("material", k)
    monkeypatch.delenv("FDTD2D_MATERIAL_AS_UNIFORM")
    name2, got = stepped()
    assert name2 == "step_persist_kernel<0>", name2
    for k in ref:
        assert np.array_equal(ref[k], got[k]), ("as uniform", k)
