"""Snapshot and restore of a shot (fdtd2d_save_state / fdtd2d_load_state),
through the C ABI: a shot stopped after some steps, saved, destroyed, and
restored into a new context of the same setup continues with the bits it
would have had without the stop -- fields, CPML psi, traces, DFT, the
wave-front tracker's rows and the line probe -- on every path: the two-step
tensor path (FP32 and F16 storage), the persistent kernel, and a
Settings.ini shot on the material-ID kernel."""
from pathlib import Path

import numpy as np
import pytest

import fdtd_2d_gb300 as F
from helpers import FIELDS, PSI_FIELDS

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _outputs(shot, prob):
    out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
    s = prob.setup
    if s.record_traces:
        tr = shot.traces()
        out.update({k: v for k, v in tr.items()})
    if s.dft_freq > 0 and s.n_det > 0:
        out["dft"] = shot.dft()
    if s.n_rc > 0:
        out["rc"] = shot.rc(1, shot.step)
    if s.line_n > 0 and shot.step >= s.line_first:
        out["line"] = shot.line(s.line_first, min(shot.step, s.line_last))
    return out


def _check_resume(gpu, prob, stop, env=None, monkeypatch=None):
    for k, v in (env or {}).items():
        monkeypatch.setenv(k, v)
    n = prob.n_steps
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        shot.run(1, n)
        whole = _outputs(shot, prob)
    with F.Shot(prob, gpu) as shot:
        shot.run(1, stop)
        image = shot.save_state()
    with F.Shot(prob, gpu) as shot:
        shot.load_state(image)
        assert shot.step == stop
        shot.run(stop + 1, n)
        resumed = _outputs(shot, prob)
    for k in whole:
        assert np.array_equal(whole[k], resumed[k]), (name, k)
    return name


@pytest.mark.parametrize("storage", [F.STORE_F32, F.STORE_F16])
def test_resume_two_step_path(gpu, monkeypatch, storage):
    prob = F.Problem.from_spec(nx=1400, ny=260, npml=16, n_steps=90, profile=3, ne_peak=3e19, x_center=620,
                               width=40, grf_rms=0.05, grf_corr=10, seed=7, nu=2e9, n_elem=8, src_i=300, src_j=100,
                               src_dj=5, freq=50e9, steer_deg=15, pulse=1, pulse_width=0.1e-9, n_det=8, det_i=300,
                               det_j=100, det_dj=5, dft_freq=50e9, storage=storage)
    # stop after an odd step: the two-step path resumes with a single step
    name = _check_resume(gpu, prob, 37, {"FDTD2D_TB": "1"}, monkeypatch)
    assert name.startswith("step_tmat2_kernel"), name


def test_resume_persistent_kernel(gpu, monkeypatch):
    prob = F.Problem.from_spec(nx=256, ny=192, n_steps=80, x_lo=128, x_hi=246, src_i=30, src_j=96, det_i=34,
                               det_j=96, pulse_width=0.1e-9)
    name = _check_resume(gpu, prob, 50, {"FDTD2D_PERSIST": "1"}, monkeypatch)
    assert name.startswith("step_persist_kernel"), name


def test_resume_settings_ini_with_tracker_and_line(gpu, tmp_path):
    """A Settings.ini shot from the golden set with the wave-front tracker and
    the TOF line probe, stopped inside the probe's window."""
    prob = F.Problem.from_ini(GOLDEN / "tof_line" / "Settings.ini")
    s = prob.setup
    assert s.n_rc > 0 and s.line_n > 0
    stop = (s.line_first + s.line_last) // 2
    _check_resume(gpu, prob, stop)


def test_load_refuses_another_shot(gpu):
    a = F.Problem.from_spec(nx=256, ny=192, n_steps=40, src_i=30, src_j=96, det_i=34, det_j=96)
    b = F.Problem.from_spec(nx=260, ny=192, n_steps=40, src_i=30, src_j=96, det_i=34, det_j=96)
    with F.Shot(a, gpu) as sa:
        sa.run(1, 10)
        image = sa.save_state()
    with F.Shot(b, gpu) as sb:
        with pytest.raises(F.FdtdError) as e:
            sb.load_state(image)
        assert e.value.status == F.ERR_INVALID
        with pytest.raises(F.FdtdError) as e:
            sb.load_state(image[:64])
        assert e.value.status in (F.ERR_RANGE, F.ERR_INVALID)


def test_load_refuses_batch_members(gpu):
    """A batch steps its members itself (the batch kernel's members and the
    solo members alike): loading a state into one is FDTD2D_ERR_STATE."""
    small = F.Problem.from_spec(nx=256, ny=192, n_steps=40, src_i=30, src_j=96, det_i=34, det_j=96)
    big = F.Problem.from_spec(nx=1600, ny=1400, n_steps=40, src_i=40, src_j=700, det_i=42, det_j=700)
    images = []
    for p in (small, big):
        with F.Shot(p, gpu) as s:
            s.run(1, 10)
            images.append(s.save_state())
    with F.Batch(gpu) as b:
        ids = [b.add(small), b.add(big)]   # the large one (2.24 M cells) joins as a solo member
        for i, image in zip(ids, images):
            with pytest.raises(F.FdtdError) as e:
                b.shot(i).load_state(image)
            assert e.value.status == F.ERR_STATE
