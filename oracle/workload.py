"""Setup of the production reflectometry shot built with numpy alone -- TEST
INFRASTRUCTURE.

The CPU reference arm of the benchmark times the oracle's FP32 restatement of
the reference step on this shot.  It must not load the product library, so
the setup (an ``fdtd2d_setup`` as ``include/fdtd2d.h`` declares it) is built
here from the shot's parameters, restating the reference's precompute:

* CPML grading of ``initializeCPML`` (FDTD_2D_Full/FDTD_cuda.cu:1224-1460):
  sigma, kappa, alpha polynomial in depth (orders m, ma) at integer (E) and
  half-integer (H) depths, stored FP32, then b = exp(-(sigma/kappa + alpha)
  dt/eps0) and c = sigma (b - 1) / (sigma + kappa alpha) / kappa;
* update denominators 1/(kappa d) (FDTD_2D_Full/FDTD_cuda.cu:1466-1578);
* vacuum coefficients CA = 1, CB = dt/eps0, DA = 1, DB = dt/mu0
  (FDTD_2D_Full/FDTD_cuda.cu:1190-1200) with the reference's constants
  (FDTD_2D_Full/FDTD_cuda.cuh:20-21);
* the array's soft source of Dev_AESASourceCalc (FDTD_2D_Full/kernel.cu:
  621-659) with a per-element steering phase and a raised-cosine ramp.

The plasma map is 1.5e19 (1 + tanh((x - 5000)/600)) m^-3 times (1 + 0.05 g)
with g a unit-variance Gaussian random field of correlation length 40 cells,
drawn with numpy (seeded): the same profile and statistics as the product's
map, not the same draw.  The arithmetic of a step does not depend on the
draw, so the timing of the step does not either.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

C0 = 2.99792458e8
PI_REF = 3.14159265358979          # the reference's `pi` for mu0
PI = 3.14159265358979323846
MU0 = 4.0 * PI_REF * 1.0e-7
EPS0 = 1.0 / (C0 * C0 * MU0)
JZ_COEF = float(np.float32(2.81794e-8))   # D_CJ, e^2/m_e, stored as float (kernel.cu:119)


class Point(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32)]


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_pp = C.POINTER(Point)


class Setup(C.Structure):
    """fdtd2d_setup of include/fdtd2d.h, field for field."""
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("npml", C.c_int32), ("n_steps", C.c_int32),
        ("dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
        ("be_x_1", _fp), ("ce_x_1", _fp), ("be_x_2", _fp), ("ce_x_2", _fp),
        ("bh_x_1", _fp), ("ch_x_1", _fp), ("bh_x_2", _fp), ("ch_x_2", _fp),
        ("be_y_1", _fp), ("ce_y_1", _fp), ("be_y_2", _fp), ("ce_y_2", _fp),
        ("bh_y_1", _fp), ("ch_y_1", _fp), ("bh_y_2", _fp), ("ch_y_2", _fp),
        ("den_ex", _fp), ("den_hx", _fp), ("den_ey", _fp), ("den_hy", _fp),
        ("medium", C.c_int32), ("ca", C.c_float), ("cb", C.c_float), ("da", C.c_float),
        ("db", C.c_float),
        ("ne", _fp), ("id1", _ip), ("id2", _ip), ("id3", _ip), ("n_materials", C.c_int32),
        ("mat_ca", _fp), ("mat_cb", _fp), ("mat_da", _fp), ("mat_db", _fp), ("mat_ne", _fp),
        ("nu", C.c_double), ("jz_coef", C.c_double),
        ("n_src", C.c_int32), ("src", _pp), ("src_phase_deg", _dp), ("envelope", _fp),
        ("src_scale", C.c_double), ("f0", C.c_double), ("f1", C.c_double), ("t1", C.c_double),
        ("src_pi", C.c_double),
        ("n_det", C.c_int32), ("det", _pp), ("n_comp", C.c_int32), ("comp", _pp),
        ("record_traces", C.c_int32), ("dft_freq", C.c_double), ("storage", C.c_int32),
        ("n_rc", C.c_int32), ("rc_scan_i", _ip), ("rc_max_i", _ip), ("rc_j_cut", C.c_int32),
        ("rc_level", C.c_float), ("rc_edge0", C.c_float),
        ("line_n", C.c_int32), ("line_i0", C.c_int32), ("line_j", C.c_int32),
        ("line_first", C.c_int32), ("line_last", C.c_int32),
        ("cover", C.c_int64 * 8), ("field_max", C.c_double),
    ]


def grade(P: int, sig_max: float, kappa_max: float, alpha_max: float, m: float, ma: float, dt: float,
          half: bool) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(kappa, b, c) of one CPML side: E tables (P entries, integer depths)
    or H tables (P - 1 entries, half-integer depths); index 0 = outer edge."""
    L = P - 1 if half else P
    i = np.arange(L, dtype=np.float64)
    if half:
        depth = (P - 1 - i - 0.5) / (P - 1.0)
        adepth = (i + 1 - 0.5) / (P - 1.0)
    else:
        depth = (P - 1 - i) / (P - 1.0)
        adepth = i.astype(np.float32).astype(np.float64) / (P - 1.0)
    sig = (sig_max * depth ** m).astype(np.float32)
    alp = (alpha_max * adepth ** ma).astype(np.float32)
    kap = (1.0 + (kappa_max - 1.0) * depth ** m).astype(np.float32)
    rate = sig / kap + alp                                  # FP32, as the reference
    b = np.exp(-rate.astype(np.float64) * dt / EPS0).astype(np.float32)
    den = sig + kap * alp                                   # FP32
    c = np.zeros(L, np.float32)
    ok = den != 0
    if not half:
        ok &= ~((sig == 0) & (alp == 0) & (np.arange(L) == P - 1))
    c[ok] = (sig[ok].astype(np.float64) * (b[ok].astype(np.float64) - 1.0) / den[ok].astype(np.float64)
             / kap[ok].astype(np.float64)).astype(np.float32)
    return kap, b, c


def denominators(n: int, P: int, d: float, kap_e: np.ndarray, kap_h: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(den_e, den_h), n - 1 entries each: 1/(kappa d) inside the strips
    (mirrored on the far side), 1/d elsewhere."""
    den_h = np.full(n - 1, np.float32(1.0 / d), np.float32)
    den_e = np.full(n - 1, np.float32(1.0 / d), np.float32)
    for i in range(n - 1):
        if i < P - 1:
            den_h[i] = np.float32(1.0 / (float(kap_h[i]) * d))
        elif i >= n - P:
            den_h[i] = np.float32(1.0 / (float(kap_h[n - 2 - i]) * d))
        if i < P:
            den_e[i] = np.float32(1.0 / (float(kap_e[i]) * d))
        elif i >= n - P:
            den_e[i] = np.float32(1.0 / (float(kap_e[n - 1 - i]) * d))
    return den_e, den_h


def gaussian_random_field(nx: int, ny: int, corr: float, seed: int) -> np.ndarray:
    """Unit-variance field with correlation exp(-r^2/corr^2): white noise
    smoothed by a separable Gaussian of width corr/2 (FFT per axis)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((ny, nx), dtype=np.float32)
    s = corr / 2.0
    for axis, n in ((0, ny), (1, nx)):
        f = np.fft.rfftfreq(n)
        h = np.exp(-2.0 * (np.pi * s * f) ** 2).astype(np.float32)   # transform of the unit-area Gaussian
        shape = [1, 1]
        shape[axis] = h.size
        g = np.fft.irfft(np.fft.rfft(g, axis=axis) * h.reshape(shape), n=n, axis=axis).astype(np.float32)
    g -= g.mean()
    g /= g.std()
    return g


class Workload:
    """A built setup and the arrays it points to (kept alive with it)."""

    def __init__(self, setup: Setup, keep: list):
        self.setup = setup
        self._keep = keep
        self.setup_ptr = C.pointer(setup)


def production_setup(n_steps: int, size: int = 8192, seed: int = 1001) -> Workload:
    """The production reflectometry shot on a size x size grid (the 8192^2
    shot by default; other sizes keep the physics and scale the plasma
    front's position): dx = 0.25 mm, Courant 0.99, 32-cell CPML (m = 3,
    sigma_max = 0.8 (m + 1)/(eta0 dx), kappa_max = 5, alpha_max = 0.05),
    16 elements on x = 64 with a 5-cell pitch at 50 GHz steered 15 degrees
    after a 2 ns raised-cosine ramp, 16 co-located Ez detectors with the
    50 GHz running DFT, nu = 2e9 1/s."""
    nx = ny = size
    P, dx = 32, 0.25e-3
    dt = 0.99 / (C0 * np.sqrt(2.0 / (dx * dx)))
    eta = np.sqrt(MU0 / EPS0)
    sig_max = 0.8 * (3 + 1) / (dx * eta)
    kap_e, be, ce = grade(P, sig_max, 5.0, 0.05, 3.0, 1.0, dt, half=False)
    kap_h, bh, ch = grade(P, sig_max, 5.0, 0.05, 3.0, 1.0, dt, half=True)
    den_e, den_h = denominators(nx, P, dx, kap_e, kap_h)
    keep: list = [be, ce, bh, ch, den_e, den_h]

    xc = 5000.0 * size / 8192
    col = 0.5 * 3.0e19 * (1.0 + np.tanh((np.arange(nx) - xc) / 600.0))
    g = gaussian_random_field(nx, ny, 40.0, seed)
    ne = np.maximum(0.0, col[None, :].astype(np.float32) * (1.0 + np.float32(0.05) * g)).astype(np.float32)
    del g
    keep.append(ne)

    n_elem, pitch, freq = 16, 5, 50e9
    j0 = ny // 2 - (n_elem - 1) * pitch // 2
    pts = (Point * n_elem)(*[Point(64, j0 + e * pitch) for e in range(n_elem)])
    dphi = -360.0 * pitch * dx * np.sin(15.0 * PI / 180.0) / (C0 / freq)
    phase = np.array([90.0 + dphi * e for e in range(n_elem)], np.float64)
    t = np.arange(n_steps + 1) * dt
    env = np.where(t < 2e-9, 0.5 * (1.0 - np.cos(PI * t / 2e-9)), 1.0).astype(np.float32)
    keep += [pts, phase, env]

    s = Setup()
    s.nx, s.ny, s.npml, s.n_steps = nx, ny, P, n_steps
    s.dt, s.dx, s.dy = dt, dx, dx
    fp = lambda a: a.ctypes.data_as(_fp)
    for side in ("1", "2"):
        for ax in ("x", "y"):
            setattr(s, f"be_{ax}_{side}", fp(be))
            setattr(s, f"ce_{ax}_{side}", fp(ce))
            setattr(s, f"bh_{ax}_{side}", fp(bh))
            setattr(s, f"ch_{ax}_{side}", fp(ch))
    s.den_ex, s.den_hx, s.den_ey, s.den_hy = fp(den_e), fp(den_h), fp(den_e), fp(den_h)
    s.medium = 0
    s.ca, s.cb, s.da, s.db = 1.0, float(np.float32(dt / EPS0)), 1.0, float(np.float32(dt / MU0))
    s.ne = fp(ne)
    s.nu, s.jz_coef = 2e9, JZ_COEF
    s.n_src, s.src, s.src_phase_deg, s.envelope = n_elem, C.cast(pts, _pp), phase.ctypes.data_as(_dp), fp(env)
    s.src_scale, s.f0, s.f1, s.t1, s.src_pi = 1.0, freq, freq, 1.0, PI
    s.n_det, s.det = n_elem, C.cast(pts, _pp)
    s.record_traces, s.dft_freq = 1, freq
    return Workload(s, keep)
