"""GPU: the serving loop (many small NVE requests sharing one GPU).

Checks that a request's answer is the same whether it runs alone or in the
mix (bitwise: the serving systems have no floating-point atomics), that the
device-memory admission budget is respected (the estimate bounds every
context's measured high-water mark, and the in-flight estimates never exceed
the budget), that every request completes, and that the device integrator
agrees with the host-driven reference integrator on a served system.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(n, nmax=900, nsteps=20, seed=5):
    from yaff_gb300.serve import make_workload
    return make_workload(nreq=n, rate=0.0, seed=seed, nmin=64, nmax=nmax, nsteps=nsteps)


def test_serving_mix_equals_alone_and_budget():
    from yaff_gb300.serve import ServingEngine, estimate_bytes, summarize
    reqs = _workload(40)
    big = max(estimate_bytes(r.spec) for r in reqs)
    budget = int(2.5 * big)
    eng = ServingEngine(nslots=4, budget_bytes=budget, precision='mixed')
    wall = eng.run(reqs, realtime=False)
    s = summarize(reqs, wall)
    assert s['errors'] == 0, [r.error for r in reqs if r.error]
    assert eng.peak_inflight_bytes <= budget
    assert eng.peak_inflight >= 2  # requests did overlap
    for r in reqs:
        assert r.log.shape == (r.nsteps + 1, 2) and np.isfinite(r.log).all()
        assert 0 < r.bytes_high <= r.estimate, (r.natom, r.bytes_high, r.estimate)
    # the same requests alone (one slot, nothing else in flight)
    picks = [0, 7, 23]
    alone = _workload(40)
    solo = ServingEngine(nslots=1, budget_bytes=budget, precision='mixed')
    solo.run([alone[i] for i in picks], realtime=False)
    for i in picks:
        a, b = reqs[i], alone[i]
        assert b.error is None, b.error
        np.testing.assert_array_equal(a.log, b.log)
        np.testing.assert_array_equal(a.pos, b.pos)
        np.testing.assert_array_equal(a.vel, b.vel)


def test_served_request_matches_host_integrator():
    """One served system, FP64: the device-resident run against the host
    VerletIntegrator driving ForceField.compute (same initial velocities)."""
    import yaff_gb300
    from yaff_gb300.serve import ServingEngine
    from yaff_gb300.verlet import VerletIntegrator
    req = _workload(1, nmax=300, nsteps=10, seed=9)[0]
    eng = ServingEngine(nslots=1, budget_bytes=1 << 32, precision='fp64')
    eng.run([req], realtime=False)
    assert req.error is None, req.error
    ff = yaff_gb300.build_forcefield(req.spec, precision='fp64')
    vi = VerletIntegrator(ff, eng.dt, temp0=300.0, rng=np.random.default_rng(req.seed))
    epots = [vi.epot]
    for _ in range(req.nsteps):
        vi.propagate()
        epots.append(vi.epot)
    np.testing.assert_allclose(req.pos, vi.pos, rtol=0, atol=1e-9 * np.abs(vi.pos).max())
    np.testing.assert_allclose(req.log[:, 0], epots, rtol=1e-9, atol=1e-12)
