"""GPU: failure paths, made on the host (no GPU fault, hang or trap).

* Neighbour-slot overflow: a tiny per-atom capacity forced through the API
  (yg_nlist_set_capacity) makes the next build overflow; the host build
  regrows and reruns (the reference's resumable buffer, yaff/pes/nlist.py:
  170-182) and gives the same list and energies; in the device-resident MD
  the overflowing rebuild rolls the batch back to its snapshot, grows the
  slots and reruns it, and the trajectory equals one without overflow.
* Bounded waits: the mbarrier wait the bulk-copy kernels use, run on a
  barrier nothing arrives at with a short poll limit, gives up and reports
  the timeout status; the context keeps working.
* Serving: a request larger than the whole memory budget is rejected while
  the others are served; a request cancelled before admission is never
  started; one cancelled in service stops at its next batch of steps and
  its memory goes back to the pool.
"""
import ctypes
import hashlib
import threading
import time

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _digest(rows):
    keys, _ = gc.pair_keys_from_rows(rows)
    return hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()


def test_host_build_regrows_after_forced_overflow():
    import yaff_gb300
    spec, data = gc.load('tric600')
    ff = yaff_gb300.build_forcefield(spec, precision='fp64')
    n = len(spec['pos'])
    g1, v1 = np.zeros((n, 3)), np.zeros((3, 3))
    e1 = ff.compute(g1, v1)
    sha1, nn1 = _digest(ff.nlist.neighs), ff.nlist.nneigh
    ff.nlist.set_capacity(1)            # 32 slots per atom: the next build overflows
    ff.update_pos(spec['pos'])          # the next compute updates the list
    g2, v2 = np.zeros((n, 3)), np.zeros((3, 3))
    e2 = ff.compute(g2, v2)
    assert ff.nlist.nneigh == nn1 and _digest(ff.nlist.neighs) == sha1
    assert abs(e2 - e1) <= 1e-12 * abs(e1)
    assert np.abs(g2 - g1).max() <= 1e-12 * np.abs(g1).max()
    assert abs(e1 - float(data['step0_energy'])) <= 1e-10 * np.abs(data['step0_part_energy']).max()


def test_device_md_rolls_back_and_reruns_after_overflow():
    import yaff_gb300
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import DeviceVerlet
    spec = yaff_gb300.configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64roll')
    vel0 = np.random.default_rng(3).normal(0, 1, spec['pos'].shape) * \
        np.sqrt(300 * 3.166811563e-6 / spec['masses'])[:, None]
    runs = []
    for force_overflow in (False, True):
        ff = yaff_gb300.build_forcefield(spec, precision='fp64')
        dv = DeviceVerlet(ff, 0.5 * femtosecond, vel0=vel0, max_steps=64, use_graph=True)
        if force_overflow:
            # the next device step rebuilds into 32 slots per atom (about 70
            # needed here): the batch rolls back, the slots grow, it reruns
            ff.nlist.set_capacity(1)
        dv.run(40)
        pos, vel, log = dv.fetch()
        runs.append((pos, vel, log, dv.nrebuild))
    (p0, v0, l0, r0), (p1, v1, l1, r1) = runs
    assert r1 >= 1
    assert np.isfinite(l1).all() and l1.shape == l0.shape
    # same trajectory up to the summation order of a list built at another step
    assert np.abs(p1 - p0).max() <= 1e-9 * np.abs(p0).max()
    assert np.abs(l1 - l0).max() <= 1e-9 * np.abs(l0).max()


def test_bounded_wait_reports_timeout_and_context_survives():
    import yaff_gb300
    from yaff_gb300 import _lib
    spec, data = gc.load('lat216')
    ff = yaff_gb300.build_forcefield(spec, precision='mixed')
    e0 = ff.compute()
    dev = yaff_gb300.device_of(ff.system)
    flag = ctypes.c_int(-1)
    t0 = time.perf_counter()
    assert dev.lib.yg_check_wait_timeout(dev.ctx, 1000, ctypes.byref(flag)) == _lib.YG_OK
    assert flag.value == 1
    assert time.perf_counter() - t0 < 30.0
    assert dev.lib.yg_check_wait_timeout(dev.ctx, 0, ctypes.byref(flag)) == _lib.YG_ERR_ARG
    ff.nlist.rebuild_next = True
    assert ff.compute() == pytest.approx(e0, rel=1e-12)


def _workload(n, nmax=700, nsteps=20, seed=8):
    from yaff_gb300.serve import make_workload
    return make_workload(nreq=n, rate=0.0, seed=seed, nmin=64, nmax=nmax, nsteps=nsteps)


def test_serving_rejects_over_budget_request_and_serves_the_rest():
    from yaff_gb300.serve import ServingEngine, estimate_bytes
    reqs = _workload(12)
    est = [estimate_bytes(r.spec) for r in reqs]
    big = int(np.argmax(est))
    budget = int(max(e for i, e in enumerate(est) if i != big) * 1.05)
    assert est[big] > budget
    eng = ServingEngine(nslots=3, budget_bytes=budget, precision='mixed')
    eng.run(reqs, realtime=False)
    assert reqs[big].error is not None and reqs[big].error.startswith('rejected')
    assert reqs[big].log is None
    for i, r in enumerate(reqs):
        if i != big:
            assert r.error is None, r.error
            assert r.log.shape == (r.nsteps + 1, 2) and np.isfinite(r.log).all()
    assert eng.peak_inflight_bytes <= budget


def test_serving_cancel_pending_and_running_requests():
    import yaff_gb300
    from yaff_gb300 import _lib
    from yaff_gb300.serve import ServingEngine
    lib = _lib.load()

    def pool_used():
        used, high, reserved = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        assert lib.yg_pool_usage(ctypes.byref(used), ctypes.byref(high), ctypes.byref(reserved)) == 0
        return used.value

    reqs = _workload(3, nmax=500, nsteps=20)
    long_req = _workload(1, nmax=600, nsteps=4000, seed=11)[0]
    long_req.rid = 99
    pending = reqs[1]
    pending.cancel()                       # withdrawn before the run starts
    order = [long_req, pending, reqs[0], reqs[2]]
    eng = ServingEngine(nslots=1, budget_bytes=1 << 32, precision='mixed', batch_steps=20)
    eng.run(_workload(1, nmax=100, nsteps=5, seed=3), realtime=False)   # one-time set-up of the pool
    used0 = pool_used()

    def canceller():
        deadline = time.perf_counter() + 60.0
        while long_req.t_start is None and time.perf_counter() < deadline:
            time.sleep(0.001)
        long_req.cancel()
    th = threading.Thread(target=canceller)
    th.start()
    eng.run(order, realtime=False)
    th.join()
    assert long_req.error == 'cancelled' and long_req.log is None
    assert pending.error == 'cancelled' and pending.t_start is None
    for r in (reqs[0], reqs[2]):
        assert r.error is None, r.error
        assert np.isfinite(r.log).all()
    assert pool_used() <= used0           # every context's memory went back to the pool
    assert eng._inflight == 0
