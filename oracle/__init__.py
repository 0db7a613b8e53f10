"""ctypes binding of the CPU oracle (``oracle/liboracle.so``).

TEST INFRASTRUCTURE: the FP64 restatement of the reference step that the CUDA
path is checked against, and (in FP32) the CPU baseline bench.py times.
Only ``tests/``, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_LIB = None


def build() -> Path:
    """Compile liboracle.so from oracle.c (gcc, OpenMP)."""
    src = HERE / "oracle.c"
    subprocess.run(["gcc", "-std=c11", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
                    str(src), "-o", str(LIB_PATH), "-lm"], check=True)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        sig = {
            "oracle_create": (vp, [C.c_void_p, C.c_int]),
            "oracle_destroy": (None, [vp]),
            "oracle_run": (C.c_int, [vp, C.c_int, C.c_int]),
            "oracle_current_step": (C.c_int, [vp]),
            "oracle_read_field": (C.c_int, [vp, C.c_int, _dp]),
            "oracle_write_field": (C.c_int, [vp, C.c_int, _dp]),
            "oracle_read_traces": (C.c_int, [vp, C.c_int, C.c_int, _fp, _fp, _fp, _fp]),
            "oracle_read_dft": (C.c_int, [vp, _dp, _dp]),
            "oracle_threads": (C.c_int, []),
            "oracle_set_threads": (None, [C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _shape(which: int, nx: int, ny: int, P: int) -> tuple[int, int]:
    return {0: (ny, nx), 3: (ny, nx), 1: (ny - 1, nx), 2: (ny, nx - 1),
            4: (ny, P), 5: (ny, P), 8: (ny, P - 1), 9: (ny, P - 1),
            6: (P, nx), 7: (P, nx), 10: (P - 1, nx), 11: (P - 1, nx)}[which]


class Oracle:
    """CPU restatement of one shot (FP64 by default; fp32=True for the baseline)."""

    def __init__(self, setup_ptr, fp32: bool = False):
        s = setup_ptr.contents
        self.nx, self.ny, self.npml, self.n_steps = s.nx, s.ny, s.npml, s.n_steps
        self.n_det, self.n_comp = s.n_det, s.n_comp
        h = lib().oracle_create(C.cast(setup_ptr, C.c_void_p), 1 if fp32 else 0)
        if not h:
            raise RuntimeError("oracle_create failed")
        self._h = C.c_void_p(h)

    @property
    def step(self) -> int:
        return lib().oracle_current_step(self._h)

    def run(self, n_first: int, n_last: int) -> None:
        rc = lib().oracle_run(self._h, n_first, n_last)
        if rc:
            raise RuntimeError(f"oracle_run({n_first},{n_last}) -> {rc}")

    def advance(self, k: int) -> None:
        n0 = self.step + 1
        self.run(n0, n0 + k - 1)

    def read_field(self, which: int) -> np.ndarray:
        out = np.empty(_shape(which, self.nx, self.ny, self.npml), np.float64)
        if lib().oracle_read_field(self._h, which, out.ctypes.data_as(_dp)):
            raise RuntimeError("oracle_read_field")
        return out

    def write_field(self, which: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.shape != _shape(which, self.nx, self.ny, self.npml):
            raise ValueError("shape")
        if lib().oracle_write_field(self._h, which, a.ctypes.data_as(_dp)):
            raise RuntimeError("oracle_write_field")

    def traces(self, n0: int = 1, n1: int | None = None) -> dict[str, np.ndarray]:
        n1 = self.step if n1 is None else n1
        rows = n1 - n0 + 1
        det = np.zeros((rows, self.n_det), np.float32)
        cez = np.zeros((rows, self.n_comp), np.float32)
        chx, chy = np.zeros_like(cez), np.zeros_like(cez)
        rc = lib().oracle_read_traces(self._h, n0, n1, det.ctypes.data_as(_fp), cez.ctypes.data_as(_fp),
                                      chx.ctypes.data_as(_fp), chy.ctypes.data_as(_fp))
        if rc:
            raise RuntimeError(f"oracle_read_traces -> {rc}")
        return {"det_ez": det, "comp_ez": cez, "comp_hx": chx, "comp_hy": chy}

    def dft(self) -> np.ndarray:
        re = np.zeros(self.n_det)
        im = np.zeros(self.n_det)
        lib().oracle_read_dft(self._h, re.ctypes.data_as(_dp), im.ctypes.data_as(_dp))
        return re + 1j * im

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().oracle_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def threads() -> int:
    return lib().oracle_threads()


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))
