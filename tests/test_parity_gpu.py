"""CUDA step vs the FP64 oracle, through the C ABI (fdtd2d_create/run/read_*).

Tolerances: fields relative L2 <= 1e-5 (normalised by the field's peak norm
over the run where the pulse has left the grid), detector traces relative L2
<= 1e-5, detector DFT phase <= 1e-4 rad.
"""
import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O
from helpers import (FIELD_TOL, FIELDS, PHASE_TOL, PSI_FIELDS, compare_fields, dft_phase_error,
                     load_state, random_state, rel)

pytestmark = pytest.mark.gpu

# Uniform-medium shots run on the shared-memory staged kernel by default;
# FDTD2D_KERNEL=stream selects the register-streaming kernel.  Both are checked.
KERNELS = ["tma", "stream", "persist"]


@pytest.fixture(params=KERNELS)
def kernel(request, monkeypatch):
    """tma: the staged kernels as timed at create; stream: the streaming
    kernel; persist: the streaming kernel's persistent form (many steps per
    cooperative launch)."""
    if request.param == "tma":
        monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
        monkeypatch.setenv("FDTD2D_PERSIST", "0")
    else:
        monkeypatch.setenv("FDTD2D_KERNEL", "stream")
        monkeypatch.setenv("FDTD2D_PERSIST", "1" if request.param == "persist" else "0")
    return request.param


def test_plain_512_shot_checkpoints(gpu, kernel):
    """512^2 plain shot (linear slab plasma, point source, 4000 steps).

    Physical fields: error / peak norm over the run <= 1e-5 at every
    checkpoint, and error / current norm <= 1e-5 while the field is above 10%
    of its peak.  CPML psi arrays: within 4x the error of the FP32 restatement
    of the same step (the reference's arithmetic), see helpers.compare_fields."""
    prob = F.Problem.from_spec()
    assert prob.stability() < 1.0
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    peaks = {w: 0.0 for w in FIELDS + PSI_FIELDS}
    snaps = []
    with F.Shot(prob, gpu) as shot:
        for n in (500, 1000, 1500, 2000, 3000, 4000):
            shot.run(shot.step + 1, n)
            ref.run(ref.step + 1, n)
            ref32.run(ref32.step + 1, n)
            snap = {}
            for w in FIELDS + PSI_FIELDS:
                c = ref.read_field(w)
                g = shot.read_field(w).astype(np.float64)
                f = ref32.read_field(w)
                peaks[w] = max(peaks[w], float(np.linalg.norm(c)))
                snap[w] = (float(np.linalg.norm(g - c)), float(np.linalg.norm(c)),
                           float(np.linalg.norm(f - c)))
            snaps.append((n, snap))
        for n, snap in snaps:
            for w, (d, c, d32) in snap.items():
                if w in FIELDS:
                    assert d / peaks[w] <= FIELD_TOL, (n, w, d / peaks[w])
                    if c >= 0.1 * peaks[w]:
                        assert d / c <= FIELD_TOL, (n, w, d / c)
                else:
                    assert d <= max(FIELD_TOL * peaks[w], 4.0 * d32), (n, w, d, d32, peaks[w])
        tg = shot.traces()["det_ez"]
        tc = ref.traces()["det_ez"]
        assert rel(tg, tc) <= FIELD_TOL
        assert dft_phase_error(shot, ref) <= PHASE_TOL
        assert shot.check_finite()


@pytest.mark.parametrize("nx,ny,P", [(203, 157, 7), (131, 96, 4), (64, 260, 12), (40, 40, 2),
                                    (1100, 90, 9)])
def test_random_state_uniform(gpu, kernel, nx, ny, P):
    """Random fields and psi on odd grids (nx not a multiple of 4, unit edges,
    tiny P), per-cell plasma, collisions; every code path of one step."""
    rng = np.random.default_rng(nx * 1000 + ny)
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=60, profile=1, x_lo=nx // 3,
                               x_hi=nx - 3, ne_peak=2e19, nu=3e9, src_i=P + 2, src_j=ny // 2,
                               det_i=P + 4, det_j=ny // 2 + 1, n_det=1)
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    with F.Shot(prob, gpu) as shot:
        st = random_state(shot, nx, ny, P, rng)
        load_state([shot, ref, ref32], st)
        shot.run(1, 1)
        ref.run(1, 1)
        ref32.run(1, 1)
        compare_fields(shot, ref, FIELDS, tol=1e-6)
        compare_fields(shot, ref, PSI_FIELDS, tol=1e-6, ref32=ref32)
        shot.run(2, 60)
        ref.run(2, 60)
        ref32.run(2, 60)
        compare_fields(shot, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)


def _random_state_case(gpu, nx, ny, P, steps=60):
    rng = np.random.default_rng(nx * 1000 + ny)
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=steps, profile=1, x_lo=nx // 3,
                               x_hi=nx - 3, ne_peak=2e19, nu=3e9, src_i=P + 2, src_j=ny // 2,
                               det_i=P + 4, det_j=ny // 2 + 1, n_det=1)
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        st = random_state(shot, nx, ny, P, rng)
        load_state([shot, ref, ref32], st)
        shot.run(1, steps)
        ref.run(1, steps)
        ref32.run(1, steps)
        compare_fields(shot, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)
    return name


# Launch shapes (warps per CTA, ring stages) compiled into the staged kernel.
TMA_SHAPES = ["4,3", "4,2", "4,4", "4,6", "8,2", "8,3", "8,4", "2,4", "2,6", "2,2", "2,3", "1,2", "1,3", "1,4"]


@pytest.mark.parametrize("shape", TMA_SHAPES)
def test_every_launch_shape(gpu, monkeypatch, shape):
    """Each compiled launch shape of the staged kernel, forced through
    FDTD2D_TMA, on grids whose width is not a multiple of any band and whose
    CPML strips fall inside the first and last bands."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.setenv("FDTD2D_TMA", shape)
    monkeypatch.setenv("FDTD2D_TMAT", "0")   # the one-row kernel on the whole grid
    for nx, ny, P in ((1100, 90, 9), (203, 157, 7)):
        assert _random_state_case(gpu, nx, ny, P) == f"step_tma_kernel<{shape}>"


# Multi-row tensor shapes (warps, rows per stage, stages) of step_tmat.cu.
TMAT_SHAPES = ["4,4,2", "4,2,3", "4,4,3", "2,8,2", "4,8,2", "8,2,2", "4,2,2"]


def _stepped_state(gpu, prob, st, steps):
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        load_state([shot], st)
        shot.run(1, steps)
        out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
        out["det"] = shot.traces()["det_ez"]
    return name, out


@pytest.mark.parametrize("shape", TMAT_SHAPES)
@pytest.mark.parametrize("storage", [F.STORE_F32, F.STORE_F16])
def test_tensor_interior_equals_staged(gpu, monkeypatch, shape, storage):
    """The multi-row tensor kernel on the interior (forced through
    FDTD2D_TMAT) gives every cell the same bits as the one-row staged kernel
    alone (FDTD2D_TMAT=0): same arithmetic, different staging.  Random state,
    a source and a detector inside the interior, width not a multiple of the
    band, rows not a multiple of the stage rows."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.delenv("FDTD2D_TMA", raising=False)
    nx, ny, P, steps = 2600, 301, 11, 25
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=steps, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                               ne_peak=2e19, nu=3e9, src_i=1300, src_j=150, det_i=1303, det_j=151, n_det=1,
                               storage=storage, field_max=100.0)
    rng = np.random.default_rng(11)
    st = {}
    for w in FIELDS:
        a = (rng.standard_normal(F.field_shape(w, nx, ny, P)) * 0.5).astype(np.float32)
        st[w] = a / np.float32(377.0) if w in (F.FIELD_HX, F.FIELD_HY) else a
    for w in PSI_FIELDS:
        st[w] = (rng.standard_normal(F.field_shape(w, nx, ny, P)) * 1e-3).astype(np.float32)
    monkeypatch.setenv("FDTD2D_TMAT", "0")
    name0, ref = _stepped_state(gpu, prob, st, steps)
    assert "tmat" not in name0
    monkeypatch.setenv("FDTD2D_TMAT", shape)
    monkeypatch.setenv("FDTD2D_TB", "0")
    name1, got = _stepped_state(gpu, prob, st, steps)
    assert name1.startswith(f"step_tmat_kernel<{shape}>+step_tma_kernel<"), name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), (shape, k)


def _random_fields(nx, ny, P, seed):
    rng = np.random.default_rng(seed)
    st = {}
    for w in FIELDS:
        a = (rng.standard_normal(F.field_shape(w, nx, ny, P)) * 0.5).astype(np.float32)
        st[w] = a / np.float32(377.0) if w in (F.FIELD_HX, F.FIELD_HY) else a
    for w in PSI_FIELDS:
        st[w] = (rng.standard_normal(F.field_shape(w, nx, ny, P)) * 1e-3).astype(np.float32)
    return st


def _stepped_all(gpu, prob, st, steps, chunks):
    """Fields, psi, traces, DFT and line probe after `steps` steps run as
    fdtd2d_run calls over the given chunk lengths."""
    with F.Shot(prob, gpu) as shot:
        name = shot.kernel_name()
        load_state([shot], st)
        n = 1
        for c in chunks:
            shot.run(n, n + c - 1)
            n += c
        assert n == steps + 1
        out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
        tr = shot.traces()
        out["det"] = tr["det_ez"]
        out["dft"] = shot.dft()
        s = prob.setup
        if s.line_n > 0:
            out["line"] = shot.line(s.line_first, s.line_last)
    return name, out


@pytest.mark.parametrize("shape", TMAT_SHAPES)
@pytest.mark.parametrize("storage", [F.STORE_F32, F.STORE_F16, F.STORE_BF16])
def test_two_step_equals_one_step(gpu, monkeypatch, shape, storage):
    """The two-step form (FDTD2D_TB=1: two time steps per pass over the
    interior, the CPML-band kernel stepping the rest once per step between)
    gives every cell, psi value, trace sample and DFT sum the bits of the
    one-row kernel alone.  80 sources and 80 detectors on a diagonal whose
    columns step by 31 and 29 (every residue mod 128: warp and band edges),
    down to the first interior row; random state; run calls of odd and even
    length (a single step after the pairs); a line probe over steps 9-10
    (single steps in the middle of a call)."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.delenv("FDTD2D_TMA", raising=False)
    nx, ny, P, steps = 2600, 301, 11, 25
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=steps, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                               ne_peak=2e19, nu=3e9, n_elem=80, src_i=P + 1, src_j=P + 1, src_di=31, src_dj=3,
                               n_det=80, det_i=P + 3, det_j=P + 2, det_di=29, det_dj=3, dft_freq=40e9,
                               storage=storage, field_max=100.0)
    s = prob.setup
    s.line_n, s.line_i0, s.line_j, s.line_first, s.line_last = 300, 200, 150, 9, 10
    st = _random_fields(nx, ny, P, 12)
    chunks = (7, 2, 9, 1, 6)
    monkeypatch.setenv("FDTD2D_TMAT", "0")
    name0, ref = _stepped_all(gpu, prob, st, steps, chunks)
    assert "tmat" not in name0
    monkeypatch.setenv("FDTD2D_TMAT", shape)
    monkeypatch.setenv("FDTD2D_TB", "1")
    name1, got = _stepped_all(gpu, prob, st, steps, chunks)
    assert name1.startswith(f"step_tmat2_kernel<{shape}>+step_tma_kernel<"), name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), (shape, k)


@pytest.mark.parametrize("tma,nx,storage", [("1,3", 2600, F.STORE_F32), ("2,2", 2600, F.STORE_F16),
                                             ("1,2", 2344, F.STORE_BF16), ("1,4", 2344, F.STORE_F32)])
def test_two_step_region_not_whole_units(gpu, monkeypatch, tma, nx, storage):
    """The two-step region R spans whole one-row bands, not whole tensor
    units: its first unit starts left of R and that unit's leading warps idle
    (one band kernel of 128 columns at nx = 2600: 1 idle warp of 4; 256
    columns: 2; 128 columns at nx = 2344: 3).  Every cell, psi value, trace
    sample and DFT sum keeps the one-row kernel's bits, with sources and
    detectors on R's first columns."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    ny, P, steps = 301, 11, 21
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=steps, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                               ne_peak=2e19, nu=3e9, n_elem=40, src_i=P + 1, src_j=P + 1, src_di=7, src_dj=7,
                               n_det=40, det_i=P + 3, det_j=P + 2, det_di=5, det_dj=7, dft_freq=40e9,
                               storage=storage, field_max=100.0)
    st = _random_fields(nx, ny, P, 31)
    chunks = (6, 1, 8, 6)
    monkeypatch.setenv("FDTD2D_TMA", tma)
    monkeypatch.setenv("FDTD2D_TMAT", "0")
    name0, ref = _stepped_all(gpu, prob, st, steps, chunks)
    assert "tmat" not in name0
    monkeypatch.setenv("FDTD2D_TMAT", "4,2,2")
    monkeypatch.setenv("FDTD2D_TB", "1")
    name1, got = _stepped_all(gpu, prob, st, steps, chunks)
    assert name1 == f"step_tmat2_kernel<4,2,2>+step_tma_kernel<{tma}>", name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), (tma, k)


@pytest.mark.parametrize("nx,ny,P", [(520, 300, 11), (1000, 613, 20)])
def test_persistent_equals_stream(gpu, monkeypatch, nx, ny, P):
    """The persistent kernel (FDTD2D_PERSIST=1: a run call's steps in one
    cooperative launch, a grid barrier between steps, the line probe on a
    service warp) gives every cell, psi value, trace sample, DFT sum and
    line-probe row the streaming kernel's bits: 40 sources and 40 detectors
    across warp edges and the CPML, random state, run calls of 1 to 9 steps,
    a probe window across a call boundary."""
    monkeypatch.setenv("FDTD2D_KERNEL", "stream")
    steps = 25
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=steps, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                               ne_peak=2e19, nu=3e9, n_elem=40, src_i=P - 3, src_j=P + 1, src_di=13, src_dj=7,
                               n_det=40, det_i=P - 2, det_j=P + 2, det_di=11, det_dj=7, dft_freq=40e9,
                               field_max=100.0)
    s = prob.setup
    s.line_n, s.line_i0, s.line_j, s.line_first, s.line_last = nx // 2, 3, ny // 3, 6, 12
    st = _random_fields(nx, ny, P, 41)
    chunks = (7, 2, 9, 1, 6)
    monkeypatch.setenv("FDTD2D_PERSIST", "0")
    name0, ref = _stepped_all(gpu, prob, st, steps, chunks)
    assert name0 == "step_stream_kernel<0>", name0
    monkeypatch.setenv("FDTD2D_PERSIST", "1")
    name1, got = _stepped_all(gpu, prob, st, steps, chunks)
    assert name1 == "step_persist_kernel<0>", name1
    for k in ref:
        assert np.array_equal(ref[k], got[k]), k


def test_persistent_shots_interleaved(gpu, monkeypatch):
    """Two shots on the persistent kernel, their run calls interleaved with
    no wait between them (a cooperative launch each, on their own streams):
    the launches run one after another, and each shot keeps the bits it
    has alone."""
    monkeypatch.setenv("FDTD2D_KERNEL", "stream")
    monkeypatch.setenv("FDTD2D_PERSIST", "1")
    probs = [F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=40, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                                 ne_peak=2e19, nu=3e9, src_i=P + 5, src_j=ny // 2, det_i=P + 9, det_j=ny // 2,
                                 n_det=1, dft_freq=40e9)
             for nx, ny, P in ((520, 300, 11), (700, 257, 16))]

    def result(shot):
        out = {w: shot.read_field(w) for w in FIELDS}
        out["dft"] = shot.dft()
        return out

    alone = []
    for p in probs:
        with F.Shot(p, gpu) as shot:
            assert shot.kernel_name() == "step_persist_kernel<0>", shot.kernel_name()
            shot.run(1, 40)
            alone.append(result(shot))
    shots = [F.Shot(p, gpu) for p in probs]
    try:
        for a, b in ((1, 10), (11, 25), (26, 40)):
            for shot in shots:
                shot.run(a, b)
        for shot, ref in zip(shots, alone):
            got = result(shot)
            for k in ref:
                assert np.array_equal(ref[k], got[k]), k
    finally:
        for shot in shots:
            shot.close()


def test_two_step_fields_written_between_runs(gpu, monkeypatch):
    """Fields and psi written between run calls reach every buffer the
    two-step path rotates through: runs of 9, then a write, then 6 and 2
    steps, give the one-row kernel's bits; a two-step shot's shortest runs
    (2 steps, then 1) too."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.delenv("FDTD2D_TMA", raising=False)
    nx, ny, P = 2600, 301, 11
    prob = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=17, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                               ne_peak=2e19, nu=3e9, src_i=1300, src_j=150, det_i=1303, det_j=151, n_det=1)
    st = _random_fields(nx, ny, P, 21)
    mid = _random_fields(nx, ny, P, 22)

    def stepped():
        with F.Shot(prob, gpu) as shot:
            name = shot.kernel_name()
            load_state([shot], st)
            shot.run(1, 9)
            shot.write_field(F.FIELD_EZ, mid[F.FIELD_EZ])
            shot.write_field(F.FIELD_HY, mid[F.FIELD_HY])
            shot.write_field(PSI_FIELDS[0], mid[PSI_FIELDS[0]])
            shot.run(10, 15)
            shot.run(16, 17)
            out = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
            out["det"] = shot.traces()["det_ez"]
        return name, out

    monkeypatch.setenv("FDTD2D_TMAT", "0")
    _, ref = stepped()
    monkeypatch.setenv("FDTD2D_TMAT", "4,2,2")
    monkeypatch.setenv("FDTD2D_TB", "1")
    name, got = stepped()
    assert name.startswith("step_tmat2_kernel<4,2,2>"), name
    for k in ref:
        assert np.array_equal(ref[k], got[k]), k

    short = F.Problem.from_spec(nx=nx, ny=ny, npml=P, n_steps=3, profile=1, x_lo=nx // 3, x_hi=nx - 3,
                                ne_peak=2e19, nu=3e9, src_i=1300, src_j=150, det_i=1303, det_j=151, n_det=1)
    outs = []
    for tmat in ("0", "4,2,2"):
        monkeypatch.setenv("FDTD2D_TMAT", tmat)
        with F.Shot(short, gpu) as shot:
            load_state([shot], st)
            shot.run(1, 2)
            shot.run(3, 3)
            outs.append({w: shot.read_field(w) for w in FIELDS})
    for w in FIELDS:
        assert np.array_equal(outs[0][w], outs[1][w]), w


def test_two_step_against_oracle(gpu, monkeypatch):
    """The two-step form against the FP64 oracle on a CPML-absorbed pulse
    from a steered array (fields, traces, DFT phase)."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.delenv("FDTD2D_TMA", raising=False)
    monkeypatch.delenv("FDTD2D_TMAT", raising=False)
    monkeypatch.setenv("FDTD2D_TB", "1")
    n_elem = 8
    prob = F.Problem.from_spec(nx=1400, ny=260, npml=16, n_steps=400, dx=0.25e-3, dy=0.25e-3, courant=0.99,
                               profile=3, ne_peak=3e19, x_center=900, width=60, grf_rms=0.05, grf_corr=10, seed=7,
                               nu=2e9, n_elem=n_elem, src_i=300, src_j=100, src_dj=5, src_di=0, freq=50e9,
                               steer_deg=15, pulse=1, pulse_width=0.2e-9, n_det=n_elem, det_i=300, det_j=100,
                               det_dj=5, det_di=0, dft_freq=50e9)
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    ref.run(1, prob.n_steps)
    ref32.run(1, prob.n_steps)
    with F.Shot(prob, gpu) as shot:
        assert shot.kernel_name().startswith("step_tmat2_kernel<"), shot.kernel_name()
        shot.run(1, prob.n_steps)
        compare_fields(shot, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)
        assert rel(shot.traces()["det_ez"], ref.traces()["det_ez"]) <= FIELD_TOL
        assert dft_phase_error(shot, ref) <= 1e-4


def test_autotuned_shape_and_deep_cpml(gpu, monkeypatch):
    """Without FDTD2D_TMA the create call times the shapes and keeps one; a
    CPML deeper than the staged kernel's x-strip slots streams instead."""
    monkeypatch.delenv("FDTD2D_KERNEL", raising=False)
    monkeypatch.delenv("FDTD2D_TMA", raising=False)
    assert _random_state_case(gpu, 700, 130, 16).startswith(("step_tma_kernel<", "step_tmat_kernel<",
                                                             "step_tmat2_kernel<", "step_persist_kernel<0>"))
    _random_state_case(gpu, 1600, 140, 12)   # interior bands: the tensor pair competes in the timing
    assert _random_state_case(gpu, 300, 260, 121, steps=20) in ("step_stream_kernel<0>", "step_persist_kernel<0>")


def test_phased_array_traces_and_dft(gpu, kernel):
    """Multi-element steered array with co-located detectors on a tanh x GRF
    plasma: per-step traces and the FP64 running DFT."""
    n_elem = 8
    prob = F.Problem.from_spec(nx=384, ny=320, npml=16, n_steps=1500, dx=0.25e-3, dy=0.25e-3,
                               courant=0.99, profile=3, ne_peak=3e19, x_center=250, width=40,
                               grf_rms=0.05, grf_corr=10, seed=7, nu=2e9, n_elem=n_elem, src_i=40,
                               src_j=140, src_dj=5, src_di=0, freq=50e9, steer_deg=15, pulse=1,
                               pulse_width=0.2e-9, n_det=n_elem, det_i=40, det_j=140, det_dj=5,
                               det_di=0, dft_freq=50e9)
    assert prob.stability() < 1.0
    ref = O.Oracle(prob.setup_ptr)
    with F.Shot(prob, gpu) as shot:
        shot.run(1, 1500)
        ref.run(1, 1500)
        tg, tc = shot.traces()["det_ez"], ref.traces()["det_ez"]
        assert rel(tg, tc) <= FIELD_TOL
        assert dft_phase_error(shot, ref) <= PHASE_TOL
        dg, dc = shot.dft(), ref.dft()
        assert np.max(np.abs(np.abs(dg) / np.abs(dc) - 1)) <= 1e-5


def test_material_id_medium(gpu, tmp_path):
    """Reference Settings.ini medium (sphere + fluctuation ID maps, 150-material
    table, PEC id 1 handling) with random fields."""
    ini = tmp_path / "Settings.ini"
    ini.write_text(SMALL_INI)
    prob = F.Problem.from_ini(ini)
    s = prob.setup
    assert s.medium == F.MEDIUM_MATERIAL_ID
    nx, ny, P = s.nx, s.ny, s.npml
    rng = np.random.default_rng(5)
    ref = O.Oracle(prob.setup_ptr)
    ref32 = O.Oracle(prob.setup_ptr, fp32=True)
    with F.Shot(prob, gpu) as shot:
        st = random_state(shot, nx, ny, P, rng, scale=10.0)
        load_state([shot, ref, ref32], st)
        shot.run(1, 40)
        ref.run(1, 40)
        ref32.run(1, 40)
        compare_fields(shot, ref, FIELDS + PSI_FIELDS, ref32=ref32)
        t = shot.traces()
        r = ref.traces()
        for k in ("det_ez", "comp_ez", "comp_hx", "comp_hy"):
            assert rel(t[k], r[k]) <= FIELD_TOL, k


def small(nx, ny, P, steps, **kw):
    """Spec for a small grid with the source and detector inside it."""
    base = dict(nx=nx, ny=ny, npml=P, n_steps=steps, src_i=P + 2, src_j=ny // 2, det_i=P + 3,
                det_j=ny // 2, x_lo=nx // 2, x_hi=nx - 2)
    base.update(kw)
    return F.Problem.from_spec(**base)


def test_write_read_roundtrip(gpu):
    prob = small(100, 77, 6, 5)
    rng = np.random.default_rng(1)
    with F.Shot(prob, gpu) as shot:
        for w in FIELDS + PSI_FIELDS:
            a = rng.standard_normal(F.field_shape(w, 100, 77, 6)).astype(np.float32)
            shot.write_field(w, a)
            assert np.array_equal(shot.read_field(w), a)


def test_nonfinite_detection(gpu):
    prob = small(64, 64, 4, 3)
    with F.Shot(prob, gpu) as shot:
        shot.run(1, 1)
        assert shot.check_finite()
        ez = shot.read_field("ez")
        ez[10, 10] = np.nan
        shot.write_field("ez", ez)
        assert not shot.check_finite()


def test_run_range_errors(gpu):
    prob = small(64, 64, 4, 10)
    with F.Shot(prob, gpu) as shot:
        with pytest.raises(F.FdtdError) as e:
            shot.run(2, 3)  # must start at step 1
        assert e.value.status == F.ERR_RANGE
        shot.run(1, 10)
        with pytest.raises(F.FdtdError):
            shot.run(11, 11)  # past n_steps
        with pytest.raises(F.FdtdError):
            shot.traces(5, 12)


def test_invalid_setups_rejected(gpu):
    # detector on the PEC ring
    prob = small(64, 64, 4, 3, det_i=0, det_j=5)
    with pytest.raises(F.FdtdError) as e:
        F.Shot(prob, gpu)
    assert e.value.status == F.ERR_RANGE
    # CPML strips overlapping
    prob = F.Problem.from_spec(nx=20, ny=64, npml=10, n_steps=3, src_i=5, det_i=6, src_j=30,
                               det_j=30, x_lo=8, x_hi=12)
    with pytest.raises(F.FdtdError):
        F.Shot(prob, gpu)


SMALL_INI = """;config for a small drop-in run
[hardware]
GPU_device=0
[regimes]
SourceToDetect = 0
[grid]
Use_Exp_time = 1
Imax = 60
Jmax = 110
Max_time = 400
Exp_time = 0.25
ds = 0.5
dt_coef = 0.5
Isource = 30
Jsource = 10
Idetect = 30
Jdetect = 14
[AESA]
SIsize = 10
SAutoDelta = 0
SIdelta = 2
SPAngle = 5
DIsize = 10
DAutoDelta = 0
DIdelta = 2
[PulseParam]
Chirp=1
FreqA=38
FreqB=30
Fronts_ns=0.05
Plato_ns=0.05
Pulse_amp = 1881
[2Dsave]
From=0
To=-25
TimeSieve=2000
GridSieve=1
[medium]
Build=1
Icen=30
Jcen=80
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
[mediumFluc]
FlucBuild=2
FlucIcen=25
FlucJcen=70
FlucRadius=8
FlucAlpha=2
FlucBeta=1
FlucNe0=1.028e+19
[RC_calc]
Iline = 30
LIsize = 10
LIdelta = 5
FilterWindow = 20
Rlevel = 0.07
"""
