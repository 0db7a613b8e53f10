"""The production shot itself against the FP64 oracle, through the C ABI.

8192 x 8192 cells, dx = 0.25 mm, 32-cell CPML, 16-element array on x = 64 at
50 GHz steered to 15 degrees (2 ns raised-cosine ramp), tanh x random-field
plasma, nu = 2e9 1/s, 16 co-located Ez detectors with the 50 GHz FP64
running DFT -- the shot the throughput is quoted on, on the path that runs
it: the two-step tensor kernel on the interior (two time steps per pass over
the fields), the one-row kernel on the CPML bands and rows, the frame
kernel between.  The oracle restates the reference step
(FDTD_2D_Full/kernel.cu:127-805, order :2073-2157) in FP64; the FP64 run of
all 20000 steps costs tens of minutes on the host, so the check covers a
bounded window of the same shot:

* 300 steps from rest: the ramp's first wave has crossed the x-CPML behind
  the array and spread ~200 cells; fields, CPML psi, traces and DFT.
* 20 steps from a random state: every cell of the grid carries field, so
  every interior unit, band strip, frame cell and CPML corner is exercised.

Tolerances are the parity bounds of the smaller cases: fields relative L2
<= 1e-5, traces <= 1e-5, DFT phase <= 1e-4 rad, CPML psi within 4x the
FP32 restatement's own error.
"""
import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O
from helpers import (FIELD_TOL, FIELDS, PHASE_TOL, PSI_FIELDS, compare_fields, dft_phase_error,
                     load_state, random_state, rel)

pytestmark = pytest.mark.gpu

N = 8192


@pytest.fixture
def two_step(monkeypatch):
    for k in ("FDTD2D_KERNEL", "FDTD2D_TMA", "FDTD2D_TMAT", "FDTD2D_PERSIST"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setenv("FDTD2D_TB", "1")   # the two-step form the timing keeps for this shot


def _production(steps):
    return F.Problem.from_spec(F.production_spec(n_steps=steps))


def test_production_shot_from_rest(gpu, two_step):
    steps = 300
    prob = _production(steps)
    assert prob.stability() < 1.0
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    ref.run(1, steps)
    ref32.run(1, steps)
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        assert name.startswith("step_tmat2_kernel<"), name
        shot.run(1, steps)
        errs = compare_fields(shot, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)
        terr = rel(shot.traces()["det_ez"], ref.traces()["det_ez"])
        perr = dft_phase_error(shot, ref)
        assert shot.check_finite()
    print(f"{name}: fields {errs}, traces {terr:.3e}, DFT phase {perr:.3e} rad")
    assert terr <= FIELD_TOL
    assert perr <= PHASE_TOL


def test_production_shot_random_state(gpu, two_step):
    steps = 20
    prob = _production(steps)
    rng = np.random.default_rng(8192)
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        assert name.startswith("step_tmat2_kernel<"), name
        st = random_state(shot, N, N, 32, rng)
        load_state([shot, ref, ref32], st)
        del st
        shot.run(1, steps)
        ref.run(1, steps)
        ref32.run(1, steps)
        errs = compare_fields(shot, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)
        terr = rel(shot.traces()["det_ez"], ref.traces()["det_ez"])
    print(f"{name}: fields {errs}, traces {terr:.3e}")
    assert terr <= FIELD_TOL
