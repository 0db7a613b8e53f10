"""Reduced field storage (F16 with per-array power-of-two scales, BF16): all
arithmetic FP32, storage rounded.  Results are held to stated error bounds
against the FP64 oracle (not the FP32 1e-5 bar), and the storage round trip,
the finiteness scan and the scale choice are checked directly."""
import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O
from helpers import FIELDS, dft_phase_error, rel

pytestmark = pytest.mark.gpu

# Bounds after 1500 steps of the steered-array shot below, a few times the
# errors measured on GB300 (F16: fields 0.4..1.6e-2 relative L2 over the four
# fields, traces 2.5e-3, DFT phase 2.7e-5 rad; BF16: fields 3..13e-2, traces
# 2.1e-2, phase 3.1e-4 rad).  Each store rounds a field to 11 (F16) or 8
# (BF16) significant bits and the leapfrog carries the rounding forward, so
# the error grows like 2^-12 sqrt(steps).  The F16 phase bound is the
# detector-phase bound of the FP32 path (1e-4 rad); BF16's 8 bits do not
# meet it.
BOUNDS = {F.STORE_F16: {"field": 4e-2, "trace": 1e-2, "phase": 1e-4},
          F.STORE_BF16: {"field": 3e-1, "trace": 6e-2, "phase": 1e-3}}


def array_shot(storage: int, **kw):
    n_elem = 8
    sp = dict(nx=384, ny=320, npml=16, n_steps=1500, dx=0.25e-3, dy=0.25e-3, courant=0.99, profile=3,
              ne_peak=3e19, x_center=250, width=40, grf_rms=0.05, grf_corr=10, seed=7, nu=2e9, n_elem=n_elem,
              src_i=40, src_j=140, src_dj=5, src_di=0, freq=50e9, steer_deg=15, pulse=1, pulse_width=0.2e-9,
              n_det=n_elem, det_i=40, det_j=140, det_dj=5, det_di=0, dft_freq=50e9, storage=storage)
    sp.update(kw)
    return F.Problem.from_spec(**sp)


@pytest.mark.parametrize("storage", [F.STORE_F16, F.STORE_BF16])
def test_reduced_storage_against_oracle(gpu, storage, monkeypatch):
    # the one-row kernel (the two-step case is below)
    monkeypatch.setenv("FDTD2D_TMAT", "0")
    prob = array_shot(storage)
    ref = O.Oracle(prob.setup_ptr)
    ref.run(1, prob.n_steps)
    with F.Shot(prob, gpu) as shot:
        assert shot.kernel_name().startswith("step_tma_kernel<")
        shot.run(1, prob.n_steps)
        assert shot.check_finite()
        errs = {w: rel(shot.read_field(w).astype(np.float64), ref.read_field(w)) for w in FIELDS}
        terr = rel(shot.traces()["det_ez"], ref.traces()["det_ez"])
        perr = dft_phase_error(shot, ref)
    print(f"storage {storage}: fields {errs} traces {terr:.3e} phase {perr:.3e} rad")
    b = BOUNDS[storage]
    assert max(errs.values()) <= b["field"], errs
    assert terr <= b["trace"]
    assert perr <= b["phase"]


# Bounds of the two-step case below (1400 x 260, 1000 steps): those of the
# one-row case above.  The pulse must reach the dense plasma: where the
# density is ~1e-5..1e-9 of its peak, a step's Jz increment is below half an
# F16 ulp at Jz's scale and rounds away, so F16 keeps no Jz there (BF16, with
# FP32's exponent range, does).  Such a Jz is that far below the peak's too
# and its effect on Ez is of the same order; measured on a 400-step window
# that ends before the dense plasma: F16 Ez/Hx/Hy within 3..7e-3 of FP64,
# Jz lost.
BOUNDS_TWO_STEP = BOUNDS


@pytest.mark.parametrize("storage", [F.STORE_F16, F.STORE_BF16])
def test_two_step_reduced_storage_against_oracle(gpu, monkeypatch, storage):
    """The 16-bit two-step path (stored-unit arithmetic, two time steps per
    pass) against the FP64 oracle directly: a steered array on a tanh x GRF
    plasma whose pulse crosses the interior region into the dense plasma
    and leaves through the CPML."""
    for k in ("FDTD2D_KERNEL", "FDTD2D_TMA", "FDTD2D_TMAT", "FDTD2D_PERSIST"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setenv("FDTD2D_TB", "1")
    n_elem = 8
    prob = F.Problem.from_spec(nx=1400, ny=260, npml=16, n_steps=1000, dx=0.25e-3, dy=0.25e-3, courant=0.99,
                               profile=3, ne_peak=3e19, x_center=620, width=40, grf_rms=0.05, grf_corr=10, seed=7,
                               nu=2e9, n_elem=n_elem, src_i=300, src_j=100, src_dj=5, src_di=0, freq=50e9,
                               steer_deg=15, pulse=1, pulse_width=0.2e-9, n_det=n_elem, det_i=300, det_j=100,
                               det_dj=5, det_di=0, dft_freq=50e9, storage=storage)
    assert prob.stability() < 1.0
    ref = O.Oracle(prob.setup_ptr)
    ref.run(1, prob.n_steps)
    with F.Shot(prob, gpu) as shot:
        assert shot.kernel_name().startswith("step_tmat2_kernel<"), shot.kernel_name()
        shot.run(1, prob.n_steps)
        assert shot.check_finite()
        errs = {w: rel(shot.read_field(w).astype(np.float64), ref.read_field(w)) for w in FIELDS}
        terr = rel(shot.traces()["det_ez"], ref.traces()["det_ez"])
        perr = dft_phase_error(shot, ref)
    print(f"two-step storage {storage}: fields {errs} traces {terr:.3e} phase {perr:.3e} rad")
    b = BOUNDS_TWO_STEP[storage]
    assert max(errs.values()) <= b["field"], errs
    assert terr <= b["trace"]
    assert perr <= b["phase"]


@pytest.mark.parametrize("storage", [F.STORE_F16, F.STORE_BF16])
def test_storage_roundtrip_and_nonfinite(gpu, storage):
    # field_max = 100 V/m: the F16 scales then hold |Ez| to ~800, |H| to ~8
    prob = array_shot(storage, n_steps=10, field_max=100.0)
    rng = np.random.default_rng(3)
    with F.Shot(prob, gpu) as shot:
        for w in FIELDS:
            shape = F.field_shape(w, prob.setup.nx, prob.setup.ny, prob.setup.npml)
            x = rng.standard_normal(shape).astype(np.float32) * 0.5
            shot.write_field(w, x)
            y = shot.read_field(w)
            # one rounding to 11 (F16) or 8 (BF16) significant bits (values
            # far below the array's scale fall into F16 subnormals: 1e-6 abs)
            tol = 2.0 ** -11 if storage == F.STORE_F16 else 2.0 ** -8
            assert np.all(np.abs(y - x) <= tol * np.abs(x) + 1e-6), w
        x = shot.read_field("ez")
        x[5, 7] = np.inf
        shot.write_field("ez", x)
        assert not shot.check_finite()


def test_reduced_storage_rejected_where_unsupported(gpu):
    """Reduced storage needs the staged kernel: a CPML deeper than its strip
    slots refuses it."""
    with pytest.raises(F.FdtdError):
        F.Shot(array_shot(F.STORE_F16, nx=300, ny=260, npml=121, src_i=130, det_i=130), gpu)


@pytest.mark.parametrize("storage", [F.STORE_F16, F.STORE_BF16])
def test_reduced_storage_in_batch_and_server(gpu, storage):
    """16-bit shots join a batch (and the serving loop) as solo members, next
    to FP32 shots on the batch kernel; every result is the same shot's run
    alone, bit for bit."""
    probs = [array_shot(storage, n_steps=300), array_shot(F.STORE_F32, n_steps=260, src_j=150),
             array_shot(storage, n_steps=200, nx=500, ny=300, src_j=120)]
    solo = []
    for p in probs:
        with F.Shot(p, gpu) as s:
            s.run(1, p.n_steps)
            solo.append((s.dft(), s.traces()["det_ez"]))
    with F.Batch(gpu) as b:
        ids = [b.add(p) for p in probs]
        assert all(i is not None for i in ids)
        while not all(b.finished(i) for i in ids):
            b.run(64)
        b.synchronize()
        for k, i in enumerate(ids):
            sh = b.shot(i)
            assert np.array_equal(sh.dft(), solo[k][0]) and np.array_equal(sh.traces()["det_ez"], solo[k][1])
    got = {}
    with F.Server(gpu, block_steps=32) as srv:
        for k, p in enumerate(probs):
            srv.submit(p, k)
        for _ in range(100000):
            srv.step()
            while (r := srv.pop()) is not None:
                got[r["tag"]] = r
            if len(got) == len(probs):
                break
    for k in range(len(probs)):
        assert np.array_equal(got[k]["dft"], solo[k][0]) and np.array_equal(got[k]["det_ez"], solo[k][1])
