"""Failure detection on the GPU without a GPU fault, through the C ABI.

* A bounded device wait that runs out: the persistent kernel's grid barrier
  is given a target one higher than the CTAs that arrive (a test parameter
  read at create) and a 1 ms bound, so every CTA gives up, records the
  timeout in the shot's error word and returns.  fdtd2d_synchronize reports
  FDTD2D_ERR_TIMEOUT; the shot can still be destroyed and the device keeps
  working for the next shot.  The reference ignores every return code
  (FDTD_2D_Full/FDTD_cuda.cu:406,418,439).
* The serving loop's admission: a shot whose admission fails stays at the
  head of the queue while the shots admitted before it run exactly once.
"""
import ctypes as C

import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O
from helpers import FIELD_TOL, FIELDS, compare_fields

pytestmark = pytest.mark.gpu


def _small(**kw):
    args = dict(nx=256, ny=192, n_steps=60, x_lo=128, x_hi=246, src_i=30, src_j=96, det_i=34, det_j=96,
                pulse_width=0.1e-9)
    args.update(kw)
    return F.Problem.from_spec(**args)


def test_barrier_wait_runs_out(gpu, monkeypatch):
    monkeypatch.setenv("FDTD2D_PERSIST", "1")
    monkeypatch.setenv("FDTD2D_WAIT_NS", "1000000")          # 1 ms
    monkeypatch.setenv("FDTD2D_TEST_BARRIER_EXTRA", "1")     # no barrier completes
    prob = _small()
    shot = F.Shot(prob, gpu)
    assert shot.kernel_name().startswith("step_persist_kernel")
    shot.run(1, 40)
    with pytest.raises(F.FdtdError) as e:
        shot.synchronize()
    assert e.value.status == F.ERR_TIMEOUT
    shot.close()   # fdtd2d_destroy after the timeout

    # the device is usable: the same shot, barrier as normal, matches the oracle
    monkeypatch.delenv("FDTD2D_WAIT_NS")
    monkeypatch.delenv("FDTD2D_TEST_BARRIER_EXTRA")
    ref = O.Oracle(prob.setup_ptr)
    with F.Shot(prob, gpu) as ok:
        assert ok.kernel_name().startswith("step_persist_kernel")
        ok.run(1, 40)
        ok.synchronize()
        ref.run(1, 40)
        compare_fields(ok, ref, FIELDS, tol=FIELD_TOL)
        assert ok.check_finite()


def test_server_admission_error_keeps_queue(gpu):
    """Three shots queued; the second is made invalid after it was accepted
    (its setup must stay valid until admission, and here it does not).  The
    scheduling round that meets it returns its error with the first shot
    admitted once and the second still queued; once the setup is valid again
    every shot finishes exactly once, each equal to its solo run."""
    probs = [_small(n_steps=48 + 8 * k, src_j=90 + k) for k in range(3)]
    solo = []
    for p in probs:
        with F.Shot(p, gpu) as s:
            s.run(1, p.n_steps)
            solo.append(s.dft())
    with F.Server(gpu, block_steps=16) as srv:
        for k, p in enumerate(probs):
            srv.submit(p, 100 + k)
        nx = probs[1].setup.nx
        probs[1].setup.nx = 4            # fdtd2d_create refuses a grid below 8 cells
        with pytest.raises(F.FdtdError) as e:
            srv.step()
        assert e.value.status == F.ERR_INVALID
        queued, running, finished = srv.counts()
        assert (queued, running) == (2, 1)
        probs[1].setup.nx = nx
        got = {}
        for _ in range(10000):
            srv.step()
            while (r := srv.pop()) is not None:
                assert r["tag"] not in got
                got[r["tag"]] = r["dft"]
            if len(got) == 3 and srv.counts() == (0, 0, 0):
                break
        assert sorted(got) == [100, 101, 102]
        for k in range(3):
            assert np.array_equal(got[100 + k], solo[k])


def test_server_submit_refuses_invalid(gpu):
    prob = _small()
    prob.setup.det[0].i = prob.setup.nx + 5   # detector off the grid
    with F.Server(gpu, block_steps=16) as srv:
        with pytest.raises(F.FdtdError) as e:
            srv.submit(prob, 1)
        assert e.value.status == F.ERR_RANGE
        assert srv.counts() == (0, 0, 0)


def test_server_pop_negative_sizes(gpu):
    """Negative buffer sizes copy nothing into the caller's buffers."""
    prob = _small(n_steps=20)
    with F.Server(gpu, block_steps=16) as srv:
        srv.submit(prob, 7)
        for _ in range(10000):
            srv.step()
            if srv.counts()[2]:
                break
        L = F.lib()
        dft = np.full(8, 123.0)
        tr = np.full(8, 5.0, np.float32)
        tag, nd, ns = C.c_int64(), C.c_int32(), C.c_int32()
        rc = L.fdtd2d_server_pop(srv._h, C.byref(tag), C.byref(nd), C.byref(ns),
                                 dft.ctypes.data_as(C.POINTER(C.c_double)), -1,
                                 tr.ctypes.data_as(C.POINTER(C.c_float)), -1)
        assert rc == 1 and tag.value == 7
        assert np.all(dft == 123.0) and np.all(tr == 5.0)


def test_create_on_recycled_memory(gpu):
    """Shots created on device memory the pool hands back from freed shots
    start clean.  Each shot leaves its fields full of large nonzero values
    before it is freed; the next shot of the same class (kernel choice
    remembered, so no timing trial synchronises its stream) gets that memory
    back.  Its error word is zeroed on its own stream and read in that
    stream's order, so no spurious FDTD2D_ERR_TIMEOUT, and every shot gives
    the first one's results."""
    prob = _small(n_steps=20)
    s = prob.setup
    first = None
    for k in range(12):
        with F.Shot(prob, gpu) as shot:
            shot.run(1, 20)
            shot.synchronize()
            out = (shot.dft(), shot.read_field(F.FIELD_EZ))
            if first is None:
                first = out
            assert np.array_equal(out[0], first[0]) and np.array_equal(out[1], first[1]), k
            for w in FIELDS:
                shot.write_field(w, np.full(F.field_shape(w, s.nx, s.ny, s.npml), 3e33, np.float32))


def _pool_used_bytes(device):
    """Bytes in use in the device's default memory pool (cudaMemPoolAttrUsedMemCurrent),
    through the CUDA runtime library, or None where it cannot be loaded."""
    import ctypes.util

    for name in ("libcudart.so.13", "libcudart.so", ctypes.util.find_library("cudart") or ""):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    else:
        return None
    pool = C.c_void_p()
    if rt.cudaDeviceGetDefaultMemPool(C.byref(pool), device) != 0:
        return None
    used = C.c_uint64()
    if rt.cudaMemPoolGetAttribute(pool, 7, C.byref(used)) != 0:   # cudaMemPoolAttrUsedMemCurrent
        return None
    return used.value


def test_allocation_failures_in_create(gpu, monkeypatch):
    """Each device allocation fdtd2d_create makes fails in turn (a test
    parameter read at create makes the k-th report cudaErrorMemoryAllocation
    without allocating).  Every failure returns FDTD2D_ERR_NOMEM and gives
    back what the shot had allocated (the pool's bytes in use return to where
    they were), except where the library has a smaller form to fall back to:
    the two-step path's extra buffers, whose failure leaves a shot on the
    one-step path with the same results.  Past the last allocation the shot
    is created as usual."""
    prob = F.Problem.from_spec(nx=1400, ny=260, npml=16, n_steps=24, src_i=300, src_j=100, det_i=302,
                               det_j=100, x_lo=700, x_hi=1380)
    with F.Shot(prob, gpu) as s:
        s.run(1, 24)
        ref = s.dft()
    base = _pool_used_bytes(gpu)
    nomem = in_a_row = 0
    for k in range(1, 300):
        monkeypatch.setenv("FDTD2D_TEST_FAIL_ALLOC", str(k))
        try:
            shot = F.Shot(prob, gpu)
        except F.FdtdError as e:
            assert e.status == F.ERR_NOMEM, (k, e)
            nomem += 1
            in_a_row = 0
            if base is not None:
                assert _pool_used_bytes(gpu) == base, k
            continue
        with shot:
            shot.run(1, 24)
            assert np.array_equal(shot.dft(), ref), k
        in_a_row += 1
        if in_a_row == 3:   # past the last allocation of create
            break
    assert in_a_row == 3 and nomem >= 8, (nomem, k)
