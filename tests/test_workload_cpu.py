"""The numpy-built production setup the CPU reference arm times
(oracle/workload.py) against the product's spec builder on the same shot:
every table, coefficient, source and detector bitwise, the plasma map by its
profile and statistics (its random field is another draw).  CPU only."""
import numpy as np

import fdtd_2d_gb300 as F
from oracle import workload as W

N = 1024


def _pair():
    w = W.production_setup(40, size=N)
    p = F.Problem.from_spec(F.production_spec(n_steps=40, nx=N, ny=N, x_center=N * 5000 / 8192,
                                              src_j=N // 2 - 37, det_j=N // 2 - 37))
    return w, p


def test_workload_tables_equal_product():
    w, p = _pair()
    a, b = w.setup, p.setup
    for k in ("nx", "ny", "npml", "n_steps", "dt", "dx", "dy", "medium", "ca", "cb", "da", "db", "nu",
              "jz_coef", "n_src", "src_scale", "f0", "f1", "src_pi", "n_det", "record_traces", "dft_freq"):
        assert getattr(a, k) == getattr(b, k), k
    for ax in ("x", "y"):
        for side in ("1", "2"):
            for t, L in (("be", 32), ("ce", 32), ("bh", 31), ("ch", 31)):
                n = f"{t}_{ax}_{side}"
                assert np.array_equal(np.ctypeslib.as_array(getattr(a, n), (L,)),
                                      np.ctypeslib.as_array(getattr(b, n), (L,))), n
    for n in ("den_ex", "den_hx", "den_ey", "den_hy"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(a, n), (N - 1,)),
                              np.ctypeslib.as_array(getattr(b, n), (N - 1,))), n
    assert np.array_equal(np.ctypeslib.as_array(a.envelope, (41,)), np.ctypeslib.as_array(b.envelope, (41,)))
    assert np.array_equal(np.ctypeslib.as_array(a.src_phase_deg, (16,)),
                          np.ctypeslib.as_array(b.src_phase_deg, (16,)))
    for e in range(16):
        assert (a.src[e].i, a.src[e].j) == (b.src[e].i, b.src[e].j)
        assert (a.det[e].i, a.det[e].j) == (b.det[e].i, b.det[e].j)


def test_workload_plasma_statistics():
    w, p = _pair()
    x = np.ctypeslib.as_array(w.setup.ne, (N, N)).astype(np.float64)
    y = np.ctypeslib.as_array(p.setup.ne, (N, N)).astype(np.float64)
    col = 0.5 * 3.0e19 * (1.0 + np.tanh((np.arange(N) - N * 5000 / 8192) / 600.0))
    rx, ry = x / col, y / col       # 1 + 0.05 g
    assert abs(rx.mean() - 1) < 0.02 and abs(ry.mean() - 1) < 0.02
    assert abs(rx.std() - 0.05) < 0.005 and abs(ry.std() - 0.05) < 0.005
    # correlation length: lag-40 autocorrelation exp(-1) of the field along x
    gx = (rx - 1) / 0.05
    c40 = float(np.mean(gx[:, :-40] * gx[:, 40:]))
    assert abs(c40 - np.exp(-1)) < 0.08, c40
