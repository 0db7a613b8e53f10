"""Batched / continuous stepping (fdtd2d_batch_*) on the GPU.

A shot stepped in a batch goes through the same update code as a shot
stepped alone (one launch per step, every unit's halo recomputed bit-exactly
from the previous step's buffers), so its fields, traces and DFT must be
bitwise identical to the same shot run alone, whatever else is in the batch
and whenever it was admitted.  One member is also checked against the FP64
oracle.
"""
import numpy as np
import pytest

import fdtd_2d_gb300 as F
import oracle as O
from helpers import FIELD_TOL, FIELDS, PSI_FIELDS, compare_fields, dft_phase_error, rel

pytestmark = pytest.mark.gpu


def shot_spec(k: int) -> dict:
    """Uneven shots: sizes, CPML depths, frequencies, plasma and arrays differ."""
    rng = np.random.default_rng(100 + k)
    nx = int(rng.integers(150, 700))
    ny = int(rng.integers(120, 500))
    P = int(rng.integers(6, 24))
    n_elem = int(rng.integers(2, 6))
    return dict(nx=nx, ny=ny, npml=P, n_steps=int(rng.integers(150, 400)), dx=0.5e-3, dy=0.5e-3,
                courant=0.9, profile=3, ne_peak=float(rng.uniform(5e18, 3e19)), x_center=nx * 0.6,
                width=nx * 0.1, grf_rms=0.05, grf_corr=8, seed=k + 1, nu=2e9, n_elem=n_elem,
                src_i=P + 6, src_j=ny // 2 - 2 * n_elem, src_di=0, src_dj=4,
                freq=float(rng.uniform(20e9, 60e9)), steer_deg=10, pulse=1, pulse_width=0.1e-9,
                n_det=n_elem, det_i=P + 6, det_j=ny // 2 - 2 * n_elem, det_di=0, det_dj=4,
                dft_freq=0.0)


def problems(n: int):
    out = []
    for k in range(n):
        sp = shot_spec(k)
        sp["dft_freq"] = sp["freq"]
        out.append(F.Problem.from_spec(**sp))
    return out


def alone(prob, gpu):
    with F.Shot(prob, gpu) as s:
        s.run(1, prob.n_steps)
        return snapshot(s)


def snapshot(shot):
    d = {w: shot.read_field(w) for w in FIELDS + PSI_FIELDS}
    d["traces"] = shot.traces()
    d["dft"] = shot.dft()
    return d


def assert_same(a, b, what):
    for k in a:
        if k == "traces":
            for t in a[k]:
                assert np.array_equal(a[k][t], b[k][t]), (what, k, t)
        else:
            assert np.array_equal(a[k], b[k]), (what, k)


def test_batch_members_equal_alone(gpu):
    """Five uneven shots admitted together, stepped to completion in blocks
    that do not divide their lengths: each equals its solo run bitwise."""
    probs = problems(5)
    ref = [alone(p, gpu) for p in probs]
    with F.Batch(gpu) as b:
        ids = [b.add(p) for p in probs]
        assert all(i is not None for i in ids)
        assert b.kernel_name().startswith("step_tma_batch_kernel<")
        while not all(b.finished(i) for i in ids):
            b.run(37)
        b.synchronize()
        for i, r, p in zip(ids, ref, probs):
            assert b.step(i) == p.n_steps
            assert_same(snapshot(b.shot(i)), r, f"shot {i}")


def test_continuous_admission_equal_alone(gpu):
    """Shots admitted while others are part-way through (continuous batching),
    and a finished shot removed to make room: results are unchanged."""
    probs = problems(4)
    ref = [alone(p, gpu) for p in probs]
    with F.Batch(gpu) as b:
        a = b.add(probs[0])
        b.run(60)
        c = b.add(probs[1])
        b.run(45)
        d = b.add(probs[2])
        while not b.finished(a):
            b.run(16)
        b.synchronize()
        assert_same(snapshot(b.shot(a)), ref[0], "first")
        b.remove(a)
        e = b.add(probs[3])
        while not all(b.finished(i) for i in (c, d, e)):
            b.run(50)
        b.synchronize()
        for i, r in ((c, ref[1]), (d, ref[2]), (e, ref[3])):
            assert_same(snapshot(b.shot(i)), r, f"shot {i}")


def test_member_against_oracle(gpu):
    """A batch member against the FP64 oracle: fields (1e-5 of the peak norm),
    traces and DFT phase, with another shot in the batch."""
    p0, p1 = problems(2)
    ref = O.Oracle(p0.setup_ptr)
    ref32 = O.Oracle(p0.setup_ptr, fp32=True)
    ref.run(1, p0.n_steps)
    ref32.run(1, p0.n_steps)
    with F.Batch(gpu) as b:
        i = b.add(p0)
        b.add(p1)
        b.run(max(p0.n_steps, p1.n_steps))
        b.synchronize()
        s = b.shot(i)
        compare_fields(s, ref, FIELDS + PSI_FIELDS, tol=FIELD_TOL, ref32=ref32)
        assert rel(s.traces()["det_ez"], ref.traces()["det_ez"]) <= FIELD_TOL
        assert dft_phase_error(s, ref) <= 1e-4


def test_budget_admission_and_state(gpu):
    """Admission by device-memory budget; a member cannot be run on its own."""
    p0, p1 = problems(2)
    budget = p0.device_bytes() + p1.device_bytes() // 2
    with F.Batch(gpu, budget_bytes=budget) as b:
        i = b.add(p0)
        assert i is not None
        assert b.add(p1) is None                    # does not fit yet
        assert b.free_bytes() == budget - p0.device_bytes()
        with pytest.raises(F.FdtdError) as ei:
            b.shot(i).run(1, 1)
        assert ei.value.status == F.ERR_STATE
        b.run(p0.n_steps)
        b.synchronize()
        b.remove(i)
        assert b.add(p1) is not None                # room after the removal


def test_serving_results_equal_alone(gpu):
    """Serving loop: requests arrive while others are on the GPU (submitted
    between scheduling rounds), a budget that holds only part of them forces
    queueing; every shot's DFT and Ez traces equal its solo run bitwise."""
    probs = problems(6)
    solo = []
    for p in probs:
        with F.Shot(p, gpu) as s:
            s.run(1, p.n_steps)
            solo.append((s.dft(), s.traces()["det_ez"]))
    budget = sum(sorted(p.device_bytes() for p in probs)[-3:])   # about three at a time
    got = {}
    with F.Server(gpu, budget_bytes=budget, block_steps=24) as srv:
        arrivals = {0: [0, 1], 2: [2], 5: [3, 4], 9: [5]}   # round -> shots arriving
        rnd = 0
        while len(got) < len(probs):
            for k in arrivals.get(rnd, []):
                srv.submit(probs[k], k)
            srv.step()
            while (r := srv.pop()) is not None:
                got[r["tag"]] = r
            rnd += 1
            assert rnd < 10000
    for k, (dft, tr) in enumerate(solo):
        assert np.array_equal(got[k]["dft"], dft), k
        assert np.array_equal(got[k]["det_ez"], tr), k


def big_problem(k: int):
    """A wide shot whose interior takes the tensor path when run alone."""
    sp = shot_spec(k)
    sp.update(nx=1400 + 64 * k, ny=260 + 16 * k, x_center=900.0, width=120.0)
    sp["dft_freq"] = sp["freq"]
    return F.Problem.from_spec(**sp)


def test_solo_members_equal_alone(gpu, monkeypatch):
    """Members of at least FDTD2D_BATCH_SOLO_CELLS cells are solo members:
    full shots on their own streams (the tensor path, two steps per pass
    where it wins) stepped from the batch's run calls beside the batch
    kernel's members.  Every result equals its solo run bitwise."""
    monkeypatch.setenv("FDTD2D_BATCH_SOLO_CELLS", "300000")
    probs = problems(4) + [big_problem(0), big_problem(1)]
    ref = [alone(p, gpu) for p in probs]
    with F.Batch(gpu) as b:
        ids = [b.add(p) for p in probs]
        assert all(i is not None for i in ids)
        names = [b.shot(i).kernel_name() for i in ids]
        assert any(n.startswith("step_tmat") for n in names), names
        while not all(b.finished(i) for i in ids):
            b.run(37)
        b.synchronize()
        for i, r, p in zip(ids, ref, probs):
            assert b.step(i) == p.n_steps
            assert_same(snapshot(b.shot(i)), r, f"shot {i}")


def test_serving_with_solo_members(gpu, monkeypatch):
    """The serving loop with solo members among the shots (retired on their
    own events): DFT and Ez traces equal each solo run bitwise."""
    monkeypatch.setenv("FDTD2D_BATCH_SOLO_CELLS", "300000")
    probs = problems(3) + [big_problem(0), big_problem(2)]
    solo = []
    for p in probs:
        with F.Shot(p, gpu) as s:
            s.run(1, p.n_steps)
            solo.append((s.dft(), s.traces()["det_ez"]))
    got = {}
    with F.Server(gpu, block_steps=24) as srv:
        arrivals = {0: [0, 3], 2: [1], 4: [4, 2]}
        rnd = 0
        while len(got) < len(probs):
            for k in arrivals.get(rnd, []):
                srv.submit(probs[k], k)
            srv.step()
            while (r := srv.pop()) is not None:
                got[r["tag"]] = r
            rnd += 1
            assert rnd < 10000
    for k, (dft, tr) in enumerate(solo):
        assert np.array_equal(got[k]["dft"], dft), k
        assert np.array_equal(got[k]["det_ez"], tr), k


def test_batch_kernel_members_of_mixed_sample_size(gpu):
    """Members of the mixed-shot sample's size range that stay on the batch
    kernel (sides 1024..2040, below the 2^21-cell solo threshold, aspect up
    to 1:2, CPML 16..32, dx = lambda/20): each equals its solo run bitwise,
    with a small shot beside them."""
    specs = []
    for k, (nx, ny, P, f) in enumerate(((1024, 1536, 16, 30e9), (2040, 1024, 32, 55e9), (1100, 1100, 24, 75e9))):
        assert nx * ny < 1 << 21
        dx = 299792458.0 / f / 20
        specs.append(dict(nx=nx, ny=ny, npml=P, n_steps=120 + 17 * k, dx=dx, dy=dx, courant=0.95, profile=2,
                          ne_peak=2e19, x_center=0.6 * nx, width=0.1 * nx, nu=2e9, n_elem=8, src_i=P + 32,
                          src_j=ny // 2 - 20, src_di=0, src_dj=5, freq=f, steer_deg=15, pulse=1,
                          pulse_width=0.1e-9, n_det=8, det_i=P + 32, det_j=ny // 2 - 20, det_di=0, det_dj=5,
                          dft_freq=f))
    probs = [F.Problem.from_spec(**sp) for sp in specs] + problems(1)
    ref = [alone(p, gpu) for p in probs]
    with F.Batch(gpu) as b:
        ids = [b.add(p) for p in probs]
        assert all(i is not None for i in ids)
        while not all(b.finished(i) for i in ids):
            b.run(40)
        b.synchronize()
        for k, i in enumerate(ids):
            sh = b.shot(i)
            assert not sh.kernel_name().startswith("step_tmat"), "a batch-kernel member"
            assert_same(ref[k], snapshot(sh), f"member {k}")


def test_server_cancel(gpu):
    """fdtd2d_server_cancel: a running batch-kernel member and a running solo
    member cancelled mid-flight stop and never pop; a queued shot cancelled
    before admission never runs; the others finish equal to their solo runs."""
    probs = problems(4)
    big = F.Problem.from_spec(nx=1600, ny=1400, n_steps=200, src_i=40, src_j=700, det_i=42, det_j=700,
                              dft_freq=30e9)
    ref = {k: alone(probs[k], gpu)["dft"] for k in (0, 2, 3)}
    with F.Server(gpu, block_steps=16) as srv:
        for k, p in enumerate(probs):
            srv.submit(p, k)
        srv.submit(big, 10)
        srv.step()
        srv.step()
        assert srv.counts()[1] == 5            # all admitted and running
        assert srv.cancel(1) == 1              # a batch-kernel member
        assert srv.cancel(10) == 1             # the solo member
        assert srv.cancel(99) == 0
        got = {}
        for _ in range(100000):
            srv.step()
            while (r := srv.pop()) is not None:
                got[r["tag"]] = r["dft"]
            if srv.counts() == (0, 0, 0):
                break
        assert sorted(got) == [0, 2, 3]
        for k in got:
            assert np.array_equal(got[k], ref[k]), k
    # a queued shot: the budget holds one shot at a time
    with F.Server(gpu, budget_bytes=probs[0].device_bytes() + 1024, block_steps=16) as srv:
        srv.submit(probs[0], 0)
        srv.submit(probs[0], 5)
        srv.step()
        assert srv.counts()[:2] == (1, 1)
        assert srv.cancel(5) == 1
        got = []
        for _ in range(100000):
            srv.step()
            while (r := srv.pop()) is not None:
                got.append(r["tag"])
            if srv.counts() == (0, 0, 0):
                break
        assert got == [0]
