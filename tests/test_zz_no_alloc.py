"""The allocation-free non-finite scan (fdtd2d_check_finite_noalloc) against
the context-based one (fdtd2d_check_finite), through the C ABI.

The entry point exists for callers that cannot allocate GPU memory; its
scratch is a fixed array inside the library shared by every call.  This file
sorts last so that a run stopping at the first failure has run every other
test first; it passes alone in a fresh process and after the other tests.
"""
import numpy as np
import pytest

import fdtd_2d_gb300 as F

pytestmark = pytest.mark.gpu

FIELDS = (F.FIELD_EZ, F.FIELD_HX, F.FIELD_HY, F.FIELD_JZ)


def test_noalloc_scan_matches_context_scan(gpu):
    torch = pytest.importorskip("torch")
    prob = F.Problem.from_spec(nx=96, ny=80, npml=6, n_steps=40, src_i=10, src_j=40, det_i=12,
                               det_j=40, x_lo=48, x_hi=90)
    rng = np.random.default_rng(3)
    with F.Shot(prob, gpu) as shot:
        shot.run(1, 20)
        # Two calls in a row: all finite, then with NaN/Inf planted in Ez and Hy.
        for call in range(2):
            if call == 1:
                ez = shot.read_field(F.FIELD_EZ)
                hy = shot.read_field(F.FIELD_HY)
                ez[rng.integers(1, 79, 3), rng.integers(1, 95, 3)] = np.nan
                hy[5, 7] = np.inf
                shot.write_field(F.FIELD_EZ, ez)
                shot.write_field(F.FIELD_HY, hy)
            host = [shot.read_field(w) for w in FIELDS]
            expected = int(sum((~np.isfinite(a)).sum() for a in host))
            context_ok = shot.check_finite()
            total = 0
            statuses = []
            for a in host:
                dev = torch.from_numpy(a).to(f"cuda:{gpu}")
                torch.cuda.synchronize()
                status, count = F.check_finite_noalloc(dev.data_ptr(), dev.numel())
                statuses.append(status)
                total += count
            assert total == expected
            assert (total == 0) == context_ok
            assert all(s == (F.OK if c == 0 else F.ERR_NONFINITE)
                       for s, c in zip(statuses, [int((~np.isfinite(a)).sum()) for a in host]))
            assert (call == 0) == context_ok


def test_noalloc_rejects_oversize(gpu):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, device=f"cuda:{gpu}")
    with pytest.raises(F.FdtdError) as e:
        F.check_finite_noalloc(buf.data_ptr(), (1 << 31) + 1)
    assert e.value.status == F.ERR_RANGE


def _planted(n, idx, values, torch, device):
    """A device array of n zeros with `values` at `idx`, and its non-finite count."""
    a = torch.zeros(n, dtype=torch.float32, device=device)
    if idx:
        a[torch.tensor(idx, device=device)] = torch.tensor(values, dtype=torch.float32, device=device)
    host = np.zeros(len(idx), np.float32)
    host[:] = values
    return a, int((~np.isfinite(host)).sum())


def test_noalloc_many_blocks_on_a_stream(gpu):
    """Three full 2^20-value blocks and a ragged tail of 5 values, scanned on a
    side stream: values planted in the first block, the third and the last
    element.  Two calls in a row with different counts, so a block slot left
    from the first call would show up in the second's total."""
    torch = pytest.importorskip("torch")
    dev = f"cuda:{gpu}"
    chunk = 1 << 20
    n = 3 * chunk + 5
    side = torch.cuda.Stream(device=dev)
    cases = [
        ([7, 2 * chunk + 11, n - 1], [np.nan, np.inf, -np.inf]),
        ([chunk + 3, chunk + 4, 3 * chunk], [np.nan, 1.0, np.nan]),   # one finite plant
    ]
    for idx, vals in cases:
        a, expected = _planted(n, idx, vals, torch, dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        status, count = F.check_finite_noalloc(a.data_ptr(), n, side.cuda_stream)
        assert count == expected, (idx, count, expected)
        assert status == (F.ERR_NONFINITE if expected else F.OK)
    # all finite after a call that counted some
    a = torch.ones(n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    assert F.check_finite_noalloc(a.data_ptr(), n, side.cuda_stream) == (F.OK, 0)


def test_noalloc_largest_call(gpu):
    """n = 2^31 exactly, the most one call covers (every scratch slot used):
    NaN/Inf at the first value, the middle and the last."""
    torch = pytest.importorskip("torch")
    dev = f"cuda:{gpu}"
    n = 1 << 31
    free, _ = torch.cuda.mem_get_info(dev)
    if free < 12 * (1 << 30):
        pytest.skip("needs 8 GiB of free device memory")
    a, expected = _planted(n, [0, (1 << 30) + 1, n - 1], [np.nan, np.inf, np.nan], torch, dev)
    try:
        torch.cuda.synchronize(dev)
        assert F.check_finite_noalloc(a.data_ptr(), n) == (F.ERR_NONFINITE, expected)
        a[0] = 0.0
        torch.cuda.synchronize(dev)
        assert F.check_finite_noalloc(a.data_ptr(), n) == (F.ERR_NONFINITE, expected - 1)
    finally:
        del a
        torch.cuda.empty_cache()
