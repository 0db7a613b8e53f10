"""Pins against the reference program itself (tests/golden/, generated by
tests/golden/make_golden.py from the reference's own sources built for the CPU).

* The setup precompute (Settings.ini -> CPML tables, denominators, material
  tables, medium ID maps, array positions, SourceP) is bitwise identical.
* The FP64 oracle's final fields and detector traces match the reference's
  FP32 run within the 1e-5 field tolerance.
* The wave-front tracker restated per step on the oracle's fields gives the
  reference's tracker rows, and the host post-processing (RC_Line.txt,
  TAU_Line.txt, TOF files) reproduces the reference's files from the
  reference's own inputs.
"""
import re
from pathlib import Path

import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.name for p in GOLDEN.iterdir() if (p / "Settings.ini").exists())
FIELD_NAMES = {"Ez": F.FIELD_EZ, "Hx": F.FIELD_HX, "Hy": F.FIELD_HY, "Jz": F.FIELD_JZ}
PSI_NAMES = {"psi_Ezx_1": F.FIELD_PSI_EZX_1, "psi_Ezx_2": F.FIELD_PSI_EZX_2,
             "psi_Hyx_1": F.FIELD_PSI_HYX_1, "psi_Hyx_2": F.FIELD_PSI_HYX_2,
             "psi_Ezy_1": F.FIELD_PSI_EZY_1, "psi_Ezy_2": F.FIELD_PSI_EZY_2,
             "psi_Hxy_1": F.FIELD_PSI_HXY_1, "psi_Hxy_2": F.FIELD_PSI_HXY_2}


def load(case):
    g = GOLDEN / case
    return F.Problem.from_ini(g / "Settings.ini"), np.load(g / "setup.npz"), np.load(g / "state.npz")


def arr(p, name, n, dtype=np.float32):
    return np.ctypeslib.as_array(getattr(p.setup, name), shape=(n,)).astype(dtype)


@pytest.mark.parametrize("case", CASES)
def test_setup_bitwise_equal_to_reference(case):
    p, su, _ = load(case)
    s = p.setup
    imax, jmax, nmax, nmat = (int(v) for v in su["scalars"])
    assert (s.nx, s.ny, s.n_steps, s.n_materials) == (imax, jmax, nmax, nmat)
    assert s.dt == su["dt_dx_dy"][0] and s.dx == su["dt_dx_dy"][1] and s.dy == su["dt_dx_dy"][2]
    for name in ("be_x_1", "ce_x_1", "be_x_2", "ce_x_2", "bh_x_1", "ch_x_1", "bh_x_2", "ch_x_2",
                 "be_y_1", "ce_y_1", "be_y_2", "ce_y_2", "bh_y_1", "ch_y_1", "bh_y_2", "ch_y_2",
                 "den_ex", "den_hx", "den_ey", "den_hy"):
        ref = su[name]
        assert np.array_equal(arr(p, name, ref.size), ref), name
    for ref_name, name in (("CA", "mat_ca"), ("CB", "mat_cb"), ("DA", "mat_da"), ("DB", "mat_db"),
                           ("pne", "mat_ne")):
        assert np.array_equal(arr(p, name, nmat), su[ref_name]), ref_name
    for k in ("ID1", "ID2", "ID3"):
        mine = arr(p, k.lower(), imax * jmax, np.int32).reshape(jmax, imax)
        assert np.array_equal(mine, su[k].astype(np.int32)), k
    env = arr(p, "envelope", nmax + 1)
    assert np.array_equal(env[:nmax], su["SourceP"]) and env[nmax] == 0.0
    f0, f1, t1 = su["fcoef_fcoef2_pulsew"]
    assert (np.float32(s.f0), np.float32(s.f1), np.float32(s.t1)) == (f0, f1, t1)
    # element cells: column arrayI[e] + e, row J + arrayK[0]
    src_i = [s.src[e].i for e in range(s.n_src)]
    assert src_i == [int(a) + e for e, a in enumerate(su["arrayI"])]
    det_i = [s.det[e].i for e in range(s.n_det)]
    assert det_i == [int(a) + e for e, a in enumerate(su["det_arrayI"])]
    rc_scan = [s.rc_scan_i[l] for l in range(s.n_rc)]
    assert rc_scan == [int(a) + l for l, a in enumerate(su["RCdetArrayI"])]


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_state(case):
    p, su, st = load(case)
    nmax = p.n_steps
    o = O.Oracle(p.setup_ptr)
    # Final-state errors are normalised by each field's peak norm over the run
    # (the pulse decays in the CPML; FP32 rounding in the reference is then a
    # larger fraction of what is left).
    peak = {w: 0.0 for w in FIELD_NAMES.values()}
    for n in sorted(set(list(range(100, nmax, 100)) + [nmax])):
        o.run(o.step + 1, n)
        for w in peak:
            peak[w] = max(peak[w], float(np.linalg.norm(o.read_field(w))))
    for name, w in FIELD_NAMES.items():
        ref = st[name].astype(np.float64)
        err = float(np.linalg.norm(o.read_field(w) - ref)) / peak[w]
        assert err <= 1e-5, (name, err)
    tr = o.traces(1, nmax)
    # reference row n = sample at step n; row 0 is zero, step nMax is not kept
    assert not st["detect"][0].any()
    for mine, ref in (("det_ez", "detect"), ("comp_ez", "det_Ez"), ("comp_hx", "det_Hx"),
                      ("comp_hy", "det_Hy")):
        err = O.rel_l2(tr[mine][: nmax - 1], st[ref][1:])
        assert err <= 1e-5, (mine, err)
    # psi arrays: the reference's FP32 arithmetic loses digits there (see
    # tests/helpers.compare_fields); bound against the FP32 restatement.
    o32 = O.Oracle(p.setup_ptr, fp32=True)
    o32.run(1, nmax)
    for name, w in PSI_NAMES.items():
        ref = st[name].astype(np.float64)
        mine = o.read_field(w)
        den = max(np.linalg.norm(ref), 1e-300)
        e64 = np.linalg.norm(mine - ref) / den
        e32 = np.linalg.norm(o32.read_field(w) - mine) / den
        assert e64 <= max(1e-5, 4 * e32 + 1e-7), (name, e64, e32)


def rc_rows_from_fields(p, o):
    """Dev_RCcalc restated per step on the oracle's fields (FP32 values)."""
    s = p.setup
    nmax, ny = p.n_steps, s.ny
    nl = s.n_rc
    scan = [s.rc_scan_i[l] for l in range(nl)]
    mx = [s.rc_max_i[l] for l in range(nl)]
    edge = np.full(nl, np.float32(s.rc_edge0), np.float32)
    level = np.float32(s.rc_level)
    rows = np.zeros((nmax, nl), np.int32)
    for n in range(1, nmax):
        o.run(n, n)
        ez = o.read_field(F.FIELD_EZ).astype(np.float32)
        for l in range(nl):
            temp = ez[0, mx[l]]
            col = ez[s.rc_j_cut:ny - 2, mx[l]]
            if col.size and col.max() > temp:
                temp = col.max()
            cand = np.float32(temp * level)
            if cand > edge[l]:
                edge[l] = cand
            hits = np.nonzero(~(np.abs(ez[1:ny - 2, scan[l]]) < edge[l]))[0]
            rows[n, l] = hits[-1] + 1 if hits.size else 0
    return rows


@pytest.mark.parametrize("case", ["sphere_fluc_chirp", "torus_wall_tof"])
def test_wavefront_tracker_rows_match_reference(case):
    p, _, st = load(case)
    o = O.Oracle(p.setup_ptr)
    rows = rc_rows_from_fields(p, o)
    ref = st["PspdLine"]
    assert np.mean(rows[1:] == ref[1:]) >= 0.999


@pytest.mark.parametrize("case", CASES)
def test_rc_files_from_reference_rows(case, tmp_path):
    p, _, st = load(case)
    p.write_rc_lines(st["PspdLine"], tmp_path)
    for f in ("RC_Line.txt", "TAU_Line.txt"):
        assert (tmp_path / f).read_text() == (GOLDEN / case / f).read_text(), f


@pytest.mark.parametrize("case", ["tof_line", "torus_wall_tof"])
def test_tof_files_match_reference(case, tmp_path):
    """TOF post-processing on the saved Ez line: the line restated from the
    oracle's fields (only the cells Dev_SaveLine copies; in torus_wall_tof
    PosJ is cell row 2, so the reference copies nothing and the input is 0)."""
    p, _, _ = load(case)
    s = p.setup
    ini = (GOLDEN / case / "Settings.ini").read_text()
    key = {ln.split("=")[0].strip(): ln.split("=")[1].split(";")[0].strip()
           for ln in ini.splitlines() if "=" in ln and not ln.startswith(";")}
    ds = float(key["ds"])
    size, pos_i = int(int(key["SizeI"]) / ds), int(int(key["PosI"]) / ds)
    first = int(key["BeginAfter"]) + 1
    times = min(int(int(key["FinishAt"]) * (1e-9 / s.dt)), p.n_steps) - first + 1
    field = np.zeros((times, size), np.float32)
    if s.line_n > 0:
        assert s.line_j == 1 and s.line_first == first
        o = O.Oracle(p.setup_ptr)
        if first > 1:
            o.run(1, first - 1)
        c0 = s.line_i0
        for t in range(times):
            o.run(first + t, first + t)
            field[t, c0 - pos_i:c0 - pos_i + s.line_n] = o.read_field(F.FIELD_EZ)[1, c0:c0 + s.line_n]
    p.write_tof(field, tmp_path)
    for f in ("SD.txt", "CF.txt", "ARC.txt", "det_SD.txt", "det_CF.txt", "det_ARC.txt"):
        mine = np.loadtxt(tmp_path / f)
        ref = np.loadtxt(GOLDEN / case / f)
        assert mine.shape == ref.shape, f
        # TOF step indices: equal for nearly all positions (a threshold crossing
        # may move by a step when the fields differ in the last bits)
        assert np.mean(np.abs(mine[:, 1] - ref[:, 1]) <= 1) >= 0.95, f
        assert np.array_equal(mine[:, 0], ref[:, 0]), f


NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def _table(path: Path) -> np.ndarray:
    return np.array([[float(x) for x in NUM.findall(ln)] for ln in path.read_text().splitlines() if ln.strip()])


def _rows(a: np.ndarray) -> np.ndarray:
    """Oracle trace rows (row r = step r+1) in the reference's file rows
    (row i = step i, row 0 zeros, the last step not printed)."""
    out = np.zeros_like(a)
    out[1:] = a[:-1]
    return out


def test_source_to_detect_files_match_reference():
    """SourceToDetect mode: the vacuum shot (no medium, no wall, full launch
    coverage: that pass launches one block more than the floor) against the
    reference's *_S2D.txt files, and main - vacuum against DifDetEx.txt.  Sum
    columns are held to 1e-5 of the summed element magnitudes (the Hy sum
    nearly cancels about the array centre)."""
    g = GOLDEN / "s2d_sphere"
    p = F.Problem.from_ini(g / "Settings.ini")
    v = F.Problem.from_ini(g / "Settings.ini", vacuum=True)
    n = p.n_steps
    sv = v.setup
    assert not np.ctypeslib.as_array(sv.id3, shape=(sv.nx * sv.ny,)).any()
    need = [sv.nx * sv.ny, sv.nx * sv.npml, sv.nx * sv.ny, sv.npml * sv.ny, sv.nx * sv.ny, sv.nx * sv.ny,
            sv.npml * sv.ny, sv.nx * sv.npml]   # cells per reference launch (kernel order of cover[])
    assert all(sv.cover[k] >= need[k] for k in range(8))
    om, ov = O.Oracle(p.setup_ptr), O.Oracle(v.setup_ptr)
    om.run(1, n)
    ov.run(1, n)
    tm, tv = om.traces(1, n), ov.traces(1, n)
    vez, vhx, vhy = (_rows(tv[k]) for k in ("comp_ez", "comp_hx", "comp_hy"))
    mez, mhx, mhy = (_rows(tm[k]) for k in ("comp_ez", "comp_hx", "comp_hy"))
    for f, a in (("detEz_S2D.txt", vez), ("detHx_S2D.txt", vhx), ("detHy_S2D.txt", vhy)):
        ref = np.array([float(x) for x in NUM.findall((g / f).read_text())]).reshape(n, -1) / 1000
        assert O.rel_l2(a, ref) <= 1e-5, f
    det = _table(g / "Detect_S2D.txt")
    vd = _rows(tv["det_ez"])
    assert np.abs(det[:, 0] - np.arange(n) * p.setup.dt * 1e6).max() <= 1e-6
    assert np.linalg.norm(det[:, 1] / 1000 - vd.sum(1)) <= 1e-5 * np.linalg.norm(np.abs(vd).sum(1))
    alls = _table(g / "detAll_S2D.txt")
    for c, a in ((3, vez), (4, vhx), (5, vhy)):
        assert np.linalg.norm(alls[:, c] / 1000 - a.sum(1)) <= 1e-5 * np.linalg.norm(np.abs(a).sum(1)), c
    dif = _table(g / "DifDetEx.txt")
    assert dif.shape == (n, 8) and not dif[:, [1, 2, 6]].any()
    sums = []
    for c, (m, w) in ((3, (mez, vez)), (4, (mhx, vhx)), (5, (mhy, vhy))):
        d = (m - w).sum(1)
        sums.append(d)
        assert np.linalg.norm(dif[:, c] / 1000 - d) <= 1e-5 * np.linalg.norm((np.abs(m) + np.abs(w)).sum(1)), c
    s3, s4, s5 = sums
    eh = np.hypot(s3 * s5, s3 * s4)
    assert O.rel_l2(dif[:, 7] / 1000, eh) <= 1e-5


def test_tof_window_after_the_run(tmp_path):
    """A TOF window that opens after the run's last step (BeginAfter past
    the shot's length, as the default Settings.ini's 6..18 ns window on a
    run shortened below 6 ns) leaves no saved samples: processing writes its
    files with the not-found taus instead of indexing an empty line."""
    p, _, _ = load("tof_line")
    ini = (GOLDEN / "tof_line" / "Settings.ini").read_text()
    key = {ln.split("=")[0].strip(): ln.split("=")[1].split(";")[0].strip()
           for ln in ini.splitlines() if "=" in ln and not ln.startswith(";")}
    size = int(int(key["SizeI"]) / float(key["ds"]))
    p.write_tof(np.zeros((0, size), np.float32), tmp_path)
    for f in ("SD.txt", "CF.txt", "ARC.txt"):
        rows = np.atleast_2d(np.loadtxt(tmp_path / f))
        assert rows.shape[0] > 0, f
        assert np.all(rows[:, 1] == int(key["BeginAfter"]) - 1), f


def test_tof_width_and_wrong_width_refused(tmp_path):
    """fdtd2d_tof_width reports the row length fdtd2d_write_tof reads (the
    Settings.ini SizeI in grid points, SizeI / ds); the Python call refuses
    a field of another width instead of letting the library read past it."""
    p, _, _ = load("tof_line")
    ini = (GOLDEN / "tof_line" / "Settings.ini").read_text()
    key = {ln.split("=")[0].strip(): ln.split("=")[1].split(";")[0].strip()
           for ln in ini.splitlines() if "=" in ln and not ln.startswith(";")}
    size = int(int(key["SizeI"]) / float(key["ds"]))
    assert p.tof_width == size > 0
    with pytest.raises(ValueError):
        p.write_tof(np.zeros((10, size - 1), np.float32), tmp_path)
    with pytest.raises(ValueError):
        p.write_tof(np.zeros(10 * size, np.float32), tmp_path)
    spec = F.Problem.from_spec(nx=64, ny=64, npml=6, n_steps=5)
    assert spec.tof_width == 0
