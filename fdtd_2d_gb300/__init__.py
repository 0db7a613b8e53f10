"""GB300-native TMz FDTD time-step engine.

Python mirror of the C ABI in ``include/fdtd2d.h`` (ctypes over the in-tree
``libfdtd2d.so``).  The compute path is the CUDA library; there is no CPU
fallback: importing this package without the built library raises, and
creating a shot without a CUDA device raises.

The objects mirror the reference's device-driver boundary
(FDTD_2D_Full/Kernel.cuh:100-108):

* :class:`Problem` -- the host-side setup the reference builds in
  FDTD_2D_Full/FDTD_cuda.cu (from a parameter spec or from Settings.ini).
* :class:`Shot` -- ``DevMemoryAllocation`` (constructor), the
  ``DevFieldCalculation`` loop (:meth:`Shot.run`), detector/field read-back,
  ``DevMemoryFree`` (:meth:`Shot.close`).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libfdtd2d.so"

# ---- status codes and enums (fdtd2d.h) ------------------------------------
OK = 0
ERR_INVALID, ERR_NOMEM, ERR_CUDA, ERR_NONFINITE, ERR_RANGE = -1, -2, -3, -4, -5
ERR_IO, ERR_CONFIG, ERR_STATE, ERR_BUDGET, ERR_NODEVICE = -6, -7, -8, -9, -10
ERR_TIMEOUT = -11

MEDIUM_UNIFORM, MEDIUM_MATERIAL_ID = 0, 1
STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2

FIELD_EZ, FIELD_HX, FIELD_HY, FIELD_JZ = 0, 1, 2, 3
FIELD_PSI_EZX_1, FIELD_PSI_EZX_2, FIELD_PSI_EZY_1, FIELD_PSI_EZY_2 = 4, 5, 6, 7
FIELD_PSI_HYX_1, FIELD_PSI_HYX_2, FIELD_PSI_HXY_1, FIELD_PSI_HXY_2 = 8, 9, 10, 11
FIELD_NAMES = {"ez": FIELD_EZ, "hx": FIELD_HX, "hy": FIELD_HY, "jz": FIELD_JZ,
               "psi_ezx_1": FIELD_PSI_EZX_1, "psi_ezx_2": FIELD_PSI_EZX_2,
               "psi_ezy_1": FIELD_PSI_EZY_1, "psi_ezy_2": FIELD_PSI_EZY_2,
               "psi_hyx_1": FIELD_PSI_HYX_1, "psi_hyx_2": FIELD_PSI_HYX_2,
               "psi_hxy_1": FIELD_PSI_HXY_1, "psi_hxy_2": FIELD_PSI_HXY_2}


class FdtdError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _lib().fdtd2d_strerror(status).decode() if LIB_PATH.exists() else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


# ---- C structs --------------------------------------------------------------
class Point(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32)]


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_pp = C.POINTER(Point)


class Setup(C.Structure):
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


class Spec(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("npml", C.c_int32), ("n_steps", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("courant", C.c_double), ("dt", C.c_double),
        ("cpml_m", C.c_double), ("cpml_ma", C.c_double), ("sigma_factor", C.c_double),
        ("kappa_max", C.c_double), ("alpha_max", C.c_double),
        ("profile", C.c_int32), ("ne_peak", C.c_double), ("x_lo", C.c_double),
        ("x_hi", C.c_double), ("x_center", C.c_double), ("width", C.c_double),
        ("grf_rms", C.c_double), ("grf_corr", C.c_double), ("seed", C.c_uint64),
        ("nu", C.c_double),
        ("n_elem", C.c_int32), ("src_i", C.c_int32), ("src_j", C.c_int32),
        ("src_di", C.c_int32), ("src_dj", C.c_int32),
        ("freq", C.c_double), ("steer_deg", C.c_double), ("amp", C.c_double),
        ("pulse", C.c_int32), ("pulse_width", C.c_double), ("pulse_t0", C.c_double),
        ("n_det", C.c_int32), ("det_i", C.c_int32), ("det_j", C.c_int32),
        ("det_di", C.c_int32), ("det_dj", C.c_int32),
        ("record_traces", C.c_int32), ("dft_freq", C.c_double), ("storage", C.c_int32),
        ("field_max", C.c_double),
    ]


_LIB = None


def _lib():
    """Load libfdtd2d.so (fails loudly when it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -m fdtd_2d_gb300.build, or __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    sig = {
        "fdtd2d_abi_version": (C.c_int, []),
        "fdtd2d_strerror": (C.c_char_p, [C.c_int]),
        "fdtd2d_create": (C.c_int, [C.POINTER(Setup), C.c_int, C.POINTER(vp)]),
        "fdtd2d_run": (C.c_int, [vp, C.c_int32, C.c_int32]),
        "fdtd2d_synchronize": (C.c_int, [vp]),
        "fdtd2d_current_step": (C.c_int, [vp, _ip]),
        "fdtd2d_read_traces": (C.c_int, [vp, C.c_int32, C.c_int32, _fp, _fp, _fp, _fp]),
        "fdtd2d_read_dft": (C.c_int, [vp, _dp, _dp]),
        "fdtd2d_read_rc": (C.c_int, [vp, C.c_int32, C.c_int32, _ip]),
        "fdtd2d_read_line": (C.c_int, [vp, C.c_int32, C.c_int32, _fp]),
        "fdtd2d_read_field": (C.c_int, [vp, C.c_int, _fp]),
        "fdtd2d_write_field": (C.c_int, [vp, C.c_int, _fp]),
        "fdtd2d_check_finite": (C.c_int, [vp]),
        "fdtd2d_destroy": (C.c_int, [vp]),
        "fdtd2d_device_bytes": (C.c_int64, [C.POINTER(Setup)]),
        "fdtd2d_launch_count": (C.c_int64, [vp]),
        "fdtd2d_kernel_name": (C.c_char_p, [vp]),
        "fdtd2d_batch_create": (C.c_int, [C.c_int, C.c_int64, C.POINTER(vp)]),
        "fdtd2d_batch_add": (C.c_int, [vp, C.POINTER(Setup), C.POINTER(C.c_int32)]),
        "fdtd2d_batch_run": (C.c_int, [vp, C.c_int32]),
        "fdtd2d_batch_synchronize": (C.c_int, [vp]),
        "fdtd2d_batch_shot_step": (C.c_int32, [vp, C.c_int32]),
        "fdtd2d_batch_shot": (vp, [vp, C.c_int32]),
        "fdtd2d_batch_remove": (C.c_int, [vp, C.c_int32]),
        "fdtd2d_batch_free_bytes": (C.c_int64, [vp]),
        "fdtd2d_batch_launch_count": (C.c_int64, [vp]),
        "fdtd2d_batch_kernel_name": (C.c_char_p, [vp]),
        "fdtd2d_batch_destroy": (C.c_int, [vp]),
        "fdtd2d_server_create": (C.c_int, [C.c_int, C.c_int64, C.c_int32, C.POINTER(vp)]),
        "fdtd2d_server_submit": (C.c_int, [vp, C.POINTER(Setup), C.c_int64]),
        "fdtd2d_server_step": (C.c_int, [vp]),
        "fdtd2d_server_pop": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_float), C.c_int64]),
        "fdtd2d_server_counts": (C.c_int, [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "fdtd2d_server_batch": (vp, [vp]),
        "fdtd2d_server_destroy": (C.c_int, [vp]),
        "fdtd2d_last_cuda_error": (C.c_int, [vp]),
        "fdtd2d_spec_defaults": (None, [C.POINTER(Spec)]),
        "fdtd2d_problem_from_spec": (C.c_int, [C.POINTER(Spec), C.POINTER(vp)]),
        "fdtd2d_problem_from_ini": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "fdtd2d_problem_from_ini_vacuum": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "fdtd2d_problem_setup": (C.POINTER(Setup), [vp]),
        "fdtd2d_problem_free": (None, [vp]),
        "fdtd2d_run_settings": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int]),
        "fdtd2d_device_count": (C.c_int, []),
        "fdtd2d_write_rc_lines": (C.c_int, [vp, _ip, C.c_int32, C.c_char_p]),
        "fdtd2d_write_tof": (C.c_int, [vp, _fp, C.c_int32, C.c_char_p]),
        "fdtd2d_tof_width": (C.c_int32, [vp]),
        "fdtd2d_run_timed": (C.c_int, [vp, C.c_int32, C.c_int32, _fp]),
        "fdtd2d_time_step_kernel": (C.c_int, [vp, C.c_int]),
        "fdtd2d_clear_kernel_choices": (None, []),
        "fdtd2d_kernel_choice_source": (C.c_int, [vp]),
        "fdtd2d_server_cancel": (C.c_int, [vp, C.c_int64]),
        "fdtd2d_state_bytes": (C.c_int64, [vp]),
        "fdtd2d_save_state": (C.c_int, [vp, vp, C.c_int64]),
        "fdtd2d_load_state": (C.c_int, [vp, vp, C.c_int64]),
        "fdtd2d_step_kernel_time": (C.c_int, [vp, _dp, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int32)]),
        "fdtd2d_stability": (C.c_double, [C.POINTER(Setup)]),
        "fdtd2d_check_finite_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)  # every declared entry point must be exported
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def lib():
    return _lib()


def _check(rc: int, what: str) -> None:
    if rc != OK:
        raise FdtdError(rc, what)


def default_spec(**overrides) -> Spec:
    """The plain 512^2 workload (see fdtd2d_spec_defaults) with overrides."""
    sp = Spec()
    _lib().fdtd2d_spec_defaults(C.byref(sp))
    for k, v in overrides.items():
        if not hasattr(sp, k):
            raise AttributeError(f"fdtd2d_spec has no field {k!r}")
        setattr(sp, k, v)
    return sp


def production_spec(**overrides) -> Spec:
    """8192^2 production shot: dx = 0.25 mm, 32-cell CPML, 20000 steps,
    16-element array on x = 64 (pitch 5 cells, centred), CW 50 GHz steered to
    15 degrees with a 2 ns raised-cosine ramp, tanh plasma
    1.5e19 (1 + tanh((x - 5000)/600)) times (1 + 0.05 g) with g a seeded
    Gaussian random field (correlation length 40 cells, seed 1001),
    nu = 2e9 1/s, 16 co-located Ez detectors with a 50 GHz running DFT."""
    n = 8192
    n_elem, pitch = 16, 5
    base = dict(nx=n, ny=n, npml=32, n_steps=20000, dx=0.25e-3, dy=0.25e-3, courant=0.99,
                profile=3, ne_peak=3.0e19, x_center=5000.0, width=600.0, grf_rms=0.05,
                grf_corr=40.0, seed=1001, nu=2e9,
                n_elem=n_elem, src_i=64, src_j=n // 2 - (n_elem - 1) * pitch // 2, src_di=0,
                src_dj=pitch, freq=50e9, steer_deg=15.0, amp=1.0, pulse=1, pulse_width=2e-9,
                n_det=n_elem, det_i=64, det_j=n // 2 - (n_elem - 1) * pitch // 2, det_di=0,
                det_dj=pitch, record_traces=1, dft_freq=50e9)
    base.update(overrides)
    return default_spec(**base)


def field_shape(which: int, nx: int, ny: int, npml: int) -> tuple[int, int]:
    P = npml
    return {FIELD_EZ: (ny, nx), FIELD_JZ: (ny, nx), FIELD_HX: (ny - 1, nx), FIELD_HY: (ny, nx - 1),
            FIELD_PSI_EZX_1: (ny, P), FIELD_PSI_EZX_2: (ny, P),
            FIELD_PSI_HYX_1: (ny, P - 1), FIELD_PSI_HYX_2: (ny, P - 1),
            FIELD_PSI_EZY_1: (P, nx), FIELD_PSI_EZY_2: (P, nx),
            FIELD_PSI_HXY_1: (P - 1, nx), FIELD_PSI_HXY_2: (P - 1, nx)}[which]


class Problem:
    """Host-side precomputed setup; owns the arrays its fdtd2d_setup points to."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        self.setup_ptr = _lib().fdtd2d_problem_setup(self._h)
        self.setup = self.setup_ptr.contents

    @classmethod
    def from_spec(cls, spec: Spec | None = None, **overrides) -> "Problem":
        sp = spec if spec is not None else default_spec(**overrides)
        h = C.c_void_p()
        _check(_lib().fdtd2d_problem_from_spec(C.byref(sp), C.byref(h)), "problem_from_spec")
        return cls(h.value)

    @classmethod
    def from_ini(cls, path: str | os.PathLike, vacuum: bool = False) -> "Problem":
        """Setup of a Settings.ini; vacuum=True gives its SourceToDetect vacuum
        shot (no medium, fluctuation or wall)."""
        h = C.c_void_p()
        fn = _lib().fdtd2d_problem_from_ini_vacuum if vacuum else _lib().fdtd2d_problem_from_ini
        _check(fn(str(path).encode(), C.byref(h)), "problem_from_ini")
        return cls(h.value)

    def close(self) -> None:
        if self._h:
            _lib().fdtd2d_problem_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # convenience views (copies) of the setup arrays
    def array(self, name: str, n: int, dtype=np.float32) -> np.ndarray:
        p = getattr(self.setup, name)
        if not p:
            return np.zeros(0, dtype)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dtype, copy=True)

    @property
    def nx(self) -> int:
        return self.setup.nx

    @property
    def ny(self) -> int:
        return self.setup.ny

    @property
    def n_steps(self) -> int:
        return self.setup.n_steps

    def device_bytes(self) -> int:
        return int(_lib().fdtd2d_device_bytes(self.setup_ptr))

    def write_rc_lines(self, spd, out_dir) -> None:
        """RC_Line.txt / TAU_Line.txt from wave-front rows spd[n][l] (row 0 = before step 1)."""
        a = np.ascontiguousarray(spd, dtype=np.int32)
        _check(_lib().fdtd2d_write_rc_lines(self._h, a.ctypes.data_as(_ip), a.shape[0], str(out_dir).encode()),
               "write_rc_lines")

    @property
    def tof_width(self) -> int:
        """Row length of the saved line write_tof takes (SizeI in grid points)."""
        return int(_lib().fdtd2d_tof_width(self._h))

    def write_tof(self, field, out_dir) -> None:
        """Time-of-flight files from a saved Ez line field[t][i], i < tof_width."""
        a = np.ascontiguousarray(field, dtype=np.float32)
        if a.ndim != 2 or a.shape[1] != self.tof_width:
            raise ValueError(f"write_tof wants a [times][{self.tof_width}] array, got shape {a.shape}")
        _check(_lib().fdtd2d_write_tof(self._h, a.ctypes.data_as(_fp), a.shape[0], str(out_dir).encode()),
               "write_tof")

    def stability(self) -> float:
        return float(_lib().fdtd2d_stability(self.setup_ptr))


class Shot:
    """One shot's device state on one GPU (one CUDA stream)."""

    def __init__(self, problem: Problem, device: int = 0, _handle=None):
        self.problem = problem
        s = problem.setup
        self.nx, self.ny, self.npml, self.n_steps = s.nx, s.ny, s.npml, s.n_steps
        self.n_det, self.n_comp = s.n_det, s.n_comp
        self._owned = _handle is None
        if _handle is not None:   # a batch member's context (owned by the batch)
            self._h = C.c_void_p(_handle)
            return
        h = C.c_void_p()
        _check(_lib().fdtd2d_create(problem.setup_ptr, device, C.byref(h)), "fdtd2d_create")
        self._h = h

    @property
    def step(self) -> int:
        n = C.c_int32()
        _check(_lib().fdtd2d_current_step(self._h, C.byref(n)), "current_step")
        return n.value

    def run(self, n_first: int, n_last: int) -> None:
        _check(_lib().fdtd2d_run(self._h, n_first, n_last), "fdtd2d_run")

    def advance(self, k: int) -> None:
        n0 = self.step + 1
        self.run(n0, n0 + k - 1)

    def run_timed(self, n_first: int, n_last: int) -> float:
        """Run steps and return their device time (ms, CUDA events on the shot's stream)."""
        ms = C.c_float()
        _check(_lib().fdtd2d_run_timed(self._h, n_first, n_last, C.byref(ms)), "run_timed")
        return float(ms.value)

    def time_step_kernel(self, on: bool = True) -> None:
        """Start (or stop and clear) event timing of the interior step kernel."""
        _check(_lib().fdtd2d_time_step_kernel(self._h, int(on)), "time_step_kernel")

    def step_kernel_time(self) -> dict:
        """Device time of the interior step kernel's timed launches: total ms,
        launches, cells one launch updates and the time steps it advances."""
        ms, n, cells, steps = C.c_double(), C.c_int64(), C.c_int64(), C.c_int32()
        _check(_lib().fdtd2d_step_kernel_time(self._h, C.byref(ms), C.byref(n), C.byref(cells), C.byref(steps)),
               "step_kernel_time")
        return {"ms": ms.value, "launches": n.value, "cells": cells.value, "steps": steps.value}

    def synchronize(self) -> None:
        _check(_lib().fdtd2d_synchronize(self._h), "synchronize")

    def launches(self) -> int:
        return int(_lib().fdtd2d_launch_count(self._h))

    def kernel_name(self) -> str:
        """The step kernel this shot launches, with its launch shape."""
        return _lib().fdtd2d_kernel_name(self._h).decode()

    def save_state(self) -> np.ndarray:
        """Host image of the shot's state after its last step (fdtd2d_save_state)."""
        n = int(_lib().fdtd2d_state_bytes(self._h))
        if n < 0:
            raise FdtdError(n, "fdtd2d_state_bytes")
        buf = np.empty(n, np.uint8)
        _check(_lib().fdtd2d_save_state(self._h, buf.ctypes.data, n), "fdtd2d_save_state")
        return buf

    def load_state(self, image: np.ndarray) -> None:
        """Continue from a saved image (fdtd2d_load_state): the next run call
        starts at the saved step + 1."""
        img = np.ascontiguousarray(image, np.uint8)
        _check(_lib().fdtd2d_load_state(self._h, img.ctypes.data, img.size), "fdtd2d_load_state")

    def choice_source(self) -> int:
        """How its kernel choices were made: 0 timed at create (or forced), 1
        kept by this process from an earlier shot of the class, 2 read from
        the persisted choices file (fdtd2d_kernel_choice_source)."""
        return int(_lib().fdtd2d_kernel_choice_source(self._h))

    def read_field(self, which) -> np.ndarray:
        w = FIELD_NAMES[which] if isinstance(which, str) else which
        out = np.empty(field_shape(w, self.nx, self.ny, self.npml), np.float32)
        _check(_lib().fdtd2d_read_field(self._h, w, out.ctypes.data_as(_fp)), "read_field")
        return out

    def write_field(self, which, arr) -> None:
        w = FIELD_NAMES[which] if isinstance(which, str) else which
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.shape != field_shape(w, self.nx, self.ny, self.npml):
            raise ValueError(f"field {which}: shape {a.shape} != {field_shape(w, self.nx, self.ny, self.npml)}")
        _check(_lib().fdtd2d_write_field(self._h, w, a.ctypes.data_as(_fp)), "write_field")

    def traces(self, n0: int = 1, n1: int | None = None) -> dict[str, np.ndarray]:
        n1 = self.step if n1 is None else n1
        rows = n1 - n0 + 1
        det = np.zeros((rows, max(self.n_det, 0)), np.float32)
        cez = np.zeros((rows, max(self.n_comp, 0)), np.float32)
        chx = np.zeros_like(cez)
        chy = np.zeros_like(cez)
        _check(_lib().fdtd2d_read_traces(self._h, n0, n1, det.ctypes.data_as(_fp),
                                         cez.ctypes.data_as(_fp), chx.ctypes.data_as(_fp),
                                         chy.ctypes.data_as(_fp)), "read_traces")
        return {"det_ez": det, "comp_ez": cez, "comp_hx": chx, "comp_hy": chy}

    def dft(self) -> np.ndarray:
        re = np.zeros(self.n_det, np.float64)
        im = np.zeros(self.n_det, np.float64)
        _check(_lib().fdtd2d_read_dft(self._h, re.ctypes.data_as(_dp), im.ctypes.data_as(_dp)), "read_dft")
        return re + 1j * im

    def rc(self, n0: int = 1, n1: int | None = None) -> np.ndarray:
        n1 = self.step if n1 is None else n1
        out = np.zeros((n1 - n0 + 1, self.problem.setup.n_rc), np.int32)
        _check(_lib().fdtd2d_read_rc(self._h, n0, n1, out.ctypes.data_as(_ip)), "read_rc")
        return out

    def line(self, n0: int, n1: int) -> np.ndarray:
        out = np.zeros((n1 - n0 + 1, self.problem.setup.line_n), np.float32)
        _check(_lib().fdtd2d_read_line(self._h, n0, n1, out.ctypes.data_as(_fp)), "read_line")
        return out

    def check_finite(self) -> bool:
        rc = _lib().fdtd2d_check_finite(self._h)
        if rc == ERR_NONFINITE:
            return False
        _check(rc, "check_finite")
        return True

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value and getattr(self, "_owned", True):
            _lib().fdtd2d_destroy(self._h)
        self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def clear_kernel_choices() -> None:
    """Forget the kernel choices shot creation keeps per shot class."""
    _lib().fdtd2d_clear_kernel_choices()


class Batch:
    """Many uniform-medium shots advanced together on one GPU (fdtd2d_batch_*):
    one persistent launch per time step in CUDA-graph blocks, each shot at its
    own step, admission by a device-memory budget."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        h = C.c_void_p()
        _check(_lib().fdtd2d_batch_create(device, budget_bytes, C.byref(h)), "fdtd2d_batch_create")
        self._h = h
        self._problems: dict[int, Problem] = {}

    def add(self, problem: Problem) -> int | None:
        """Admit a shot; None when it does not fit the remaining budget."""
        sid = C.c_int32()
        rc = _lib().fdtd2d_batch_add(self._h, problem.setup_ptr, C.byref(sid))
        if rc == ERR_BUDGET:
            return None
        _check(rc, "fdtd2d_batch_add")
        self._problems[sid.value] = problem
        return sid.value

    def run(self, n_steps: int) -> None:
        _check(_lib().fdtd2d_batch_run(self._h, n_steps), "fdtd2d_batch_run")

    def synchronize(self) -> None:
        _check(_lib().fdtd2d_batch_synchronize(self._h), "fdtd2d_batch_synchronize")

    def step(self, shot: int) -> int:
        return int(_lib().fdtd2d_batch_shot_step(self._h, shot))

    def finished(self, shot: int) -> bool:
        return self.step(shot) >= self._problems[shot].n_steps

    def shot(self, shot: int) -> Shot:
        """The member as a Shot (traces, dft, read_field); owned by the batch."""
        h = _lib().fdtd2d_batch_shot(self._h, shot)
        if not h:
            raise FdtdError(ERR_INVALID, "fdtd2d_batch_shot")
        return Shot(self._problems[shot], _handle=h)

    def remove(self, shot: int) -> None:
        _check(_lib().fdtd2d_batch_remove(self._h, shot), "fdtd2d_batch_remove")
        self._problems.pop(shot, None)

    def free_bytes(self) -> int:
        return int(_lib().fdtd2d_batch_free_bytes(self._h))

    def launches(self) -> int:
        return int(_lib().fdtd2d_batch_launch_count(self._h))

    def kernel_name(self) -> str:
        return _lib().fdtd2d_batch_kernel_name(self._h).decode()

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib().fdtd2d_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop (fdtd2d_server_*): shots queued as they arrive, admitted in
    arrival order by device-memory budget, stepped together in blocks of
    `block_steps`, retired as soon as the GPU has finished them."""

    def __init__(self, device: int = 0, budget_bytes: int = 0, block_steps: int = 64):
        h = C.c_void_p()
        _check(_lib().fdtd2d_server_create(device, budget_bytes, block_steps, C.byref(h)), "fdtd2d_server_create")
        self._h = h
        self._held: dict[int, Problem] = {}   # setups must outlive admission

    def submit(self, problem: Problem, tag: int) -> None:
        _check(_lib().fdtd2d_server_submit(self._h, problem.setup_ptr, tag), "fdtd2d_server_submit")
        self._held[tag] = problem

    def step(self) -> int:
        rc = _lib().fdtd2d_server_step(self._h)
        if rc < 0:
            raise FdtdError(rc, "fdtd2d_server_step")
        return rc

    def cancel(self, tag: int) -> int:
        """Cancel the shots submitted under `tag` (fdtd2d_server_cancel);
        returns how many were cancelled."""
        n = _lib().fdtd2d_server_cancel(self._h, tag)
        if n < 0:
            raise FdtdError(n, "fdtd2d_server_cancel")
        self._held.pop(tag, None)
        return int(n)

    def counts(self) -> tuple[int, int, int]:
        q, r, f = C.c_int32(), C.c_int32(), C.c_int32()
        _check(_lib().fdtd2d_server_counts(self._h, C.byref(q), C.byref(r), C.byref(f)), "fdtd2d_server_counts")
        return q.value, r.value, f.value

    def pop(self) -> dict | None:
        """Oldest finished shot: {"tag", "dft" (complex per detector), "det_ez"
        ([n_steps][n_det])}, or None."""
        tag, nd, ns = C.c_int64(), C.c_int32(), C.c_int32()
        if not self.counts()[2]:
            return None
        # sizes first: peek via the held problem of the oldest finished shot is
        # not possible, so allocate for the largest held setup
        md = max((p.setup.n_det for p in self._held.values()), default=0)
        mt = max((p.setup.n_det * p.setup.n_steps for p in self._held.values()), default=0)
        dft = np.zeros(2 * max(md, 1), np.float64)
        tr = np.zeros(max(mt, 1), np.float32)
        rc = _lib().fdtd2d_server_pop(self._h, C.byref(tag), C.byref(nd), C.byref(ns),
                                      dft.ctypes.data_as(C.POINTER(C.c_double)), md,
                                      tr.ctypes.data_as(C.POINTER(C.c_float)), mt)
        if rc < 0:
            raise FdtdError(rc, "fdtd2d_server_pop")
        if rc == 0:
            return None
        self._held.pop(tag.value, None)
        n_det, n_steps = nd.value, ns.value
        return {"tag": tag.value, "dft": dft[: 2 * n_det:2] + 1j * dft[1: 2 * n_det:2],
                "det_ez": tr[: n_steps * n_det].reshape(n_steps, n_det).copy()}

    def batch_kernel_name(self) -> str:
        return _lib().fdtd2d_batch_kernel_name(_lib().fdtd2d_server_batch(self._h)).decode()

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib().fdtd2d_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_finite_noalloc(device_ptr: int, n: int, stream: int = 0) -> tuple[int, int]:
    """Count NaN/Inf in a caller-owned device float array without allocating
    (fdtd2d_check_finite_noalloc).  Returns (status, count): status is OK or
    ERR_NONFINITE; other statuses raise."""
    cnt = C.c_int64()
    rc = _lib().fdtd2d_check_finite_noalloc(C.c_void_p(device_ptr), n, C.byref(cnt), C.c_void_p(stream))
    if rc not in (OK, ERR_NONFINITE):
        raise FdtdError(rc, "check_finite_noalloc")
    return rc, int(cnt.value)


def device_count() -> int:
    return int(_lib().fdtd2d_device_count())


def run_settings(ini_path, out_dir, device: int = 0) -> None:
    """Whole reference program on the GPU: Settings.ini in, reference output files out."""
    _check(_lib().fdtd2d_run_settings(str(ini_path).encode(), str(out_dir).encode(), device),
           "run_settings")
