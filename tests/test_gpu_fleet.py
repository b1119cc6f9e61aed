"""GPU: many small systems stepped together (yaff_gb300.fleet, yg_fleet_*).

* Step-0 energy of each system against the oracle (the reference's
  algorithm in FP64): within 1e-6 of the largest part's magnitude (FP32 pair
  terms, phases and structure factors with compensated sums).
* The same request through the fleet and through the per-system context
  path (serve.serve_request: neighbour list, pair and tensor-core Ewald
  kernels of a yg_ctx): energies within 1e-6 of the largest part and
  positions within 1e-6 relative after 20 steps.
* A system's log, positions and velocities are bitwise the same alone and in
  a mix (placed at other atom and k ranges, with other systems stepping).
* Launches per step: eight, with one system or with twenty.
* A system whose neighbour rows overflow fails alone; the others finish.
* FleetEngine serves a workload with continuous admission, rejects a request
  larger than the whole fleet and withdraws a cancelled one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reqs(n, nmax=900, nsteps=20, seed=5):
    from yaff_gb300.serve import make_workload
    return make_workload(nreq=n, rate=0.0, seed=seed, nmin=64, nmax=nmax, nsteps=nsteps)


def _vel(req, temp0=300.0):
    from yaff_gb300.verlet import get_random_vel
    return get_random_vel(temp0, True, np.asarray(req.spec['masses'], float), rng=np.random.default_rng(req.seed))


def _fleet(**kw):
    from yaff_gb300.fleet import Fleet
    args = dict(max_atoms=1 << 15, max_systems=32, max_k=1 << 17, max_steps=64)
    args.update(kw)
    return Fleet(**args)


def _run(fleet, slots, nsteps):
    fleet.step(nsteps + 1)
    state, steps = fleet.poll()
    out = {}
    for s in slots:
        assert state[s] == 2, (s, state[s])
        out[s] = fleet.get(s)
    return out


def test_fleet_step0_energy_matches_oracle():
    from oracle import OracleForceField
    from yaff_gb300.units import femtosecond
    reqs = _reqs(6, nmax=1200)
    fl = _fleet()
    slots = [fl.add(r.spec, _vel(r), 1, 0.5 * femtosecond) for r in reqs]
    res = _run(fl, slots, 1)
    for r, s in zip(reqs, slots):
        orc = OracleForceField(r.spec)
        e_ref = orc.compute()
        scale = max(abs(v) for v in orc.part_energies.values())
        e = res[s][2][0, 0]
        assert abs(e - e_ref) <= 1e-6 * scale, (r.natom, e, e_ref, scale)


def test_fleet_matches_per_context_path():
    import torch
    from yaff_gb300.serve import serve_request
    from yaff_gb300.units import femtosecond
    req = _reqs(1, nmax=700, nsteps=20, seed=13)[0]
    dt = 0.5 * femtosecond
    stream = torch.cuda.Stream()
    serve_request(req, stream.cuda_stream, 'mixed', dt, 300.0, True)
    fl = _fleet()
    s = fl.add(req.spec, _vel(req), req.nsteps, dt)
    pos, vel, log, failed = _run(fl, [s], req.nsteps)[s]
    assert not failed
    from oracle import OracleForceField
    orc = OracleForceField(req.spec)
    orc.compute()
    scale = max(abs(v) for v in orc.part_energies.values())
    assert log.shape == req.log.shape
    assert np.abs(log - req.log).max() <= 1e-6 * scale
    assert np.abs(pos - req.pos).max() <= 1e-6 * np.abs(req.pos).max()


def test_fleet_alone_equals_mix_bitwise():
    from yaff_gb300.units import femtosecond
    dt = 0.5 * femtosecond
    reqs = _reqs(10, nmax=900, nsteps=20, seed=7)
    target = reqs[3]
    alone = _fleet()
    s0 = alone.add(target.spec, _vel(target), target.nsteps, dt)
    a = _run(alone, [s0], target.nsteps)[s0]
    mix = _fleet()
    slots = []
    for r in reqs[5:]:
        slots.append(mix.add(r.spec, _vel(r), r.nsteps, dt))   # others first: the target lands elsewhere
    st = mix.add(target.spec, _vel(target), target.nsteps, dt)
    for r in reqs[:3]:
        slots.append(mix.add(r.spec, _vel(r), r.nsteps, dt))
    b = _run(mix, slots + [st], target.nsteps)[st]
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)


def test_fleet_launches_per_step_do_not_grow():
    from yaff_gb300.units import femtosecond
    dt = 0.5 * femtosecond
    counts = []
    for n in (1, 20):
        fl = _fleet()
        for r in _reqs(n, nmax=400, nsteps=30, seed=3):
            assert fl.add(r.spec, _vel(r), r.nsteps, dt) is not None
        c0 = fl.launch_count()
        fl.step(10)
        fl.poll()
        counts.append(fl.launch_count() - c0)
    assert counts[0] == counts[1] == 80


def test_fleet_overflow_fails_alone():
    from yaff_gb300 import configs
    from yaff_gb300.units import femtosecond
    dt = 0.5 * femtosecond
    from yaff_gb300.units import angstrom
    sparse = configs.serving_request(64, 1, density=0.004)   # about 22 neighbours within 11 A
    sparse['skin'] = 1.0 * angstrom
    dense = _reqs(1, nmax=500, nsteps=5, seed=2)[0]
    fl = _fleet(max_neighbors=32)
    sd = fl.add(dense.spec, _vel(dense), 5, dt)
    ss = fl.add(sparse, np.zeros((64, 3)), 5, dt)
    fl.step(6)
    state, _ = fl.poll()
    assert state[sd] == 3 and state[ss] == 2
    assert fl.get(sd)[3] and not fl.get(ss)[3]


def test_fleet_engine_serves_rejects_and_cancels():
    from yaff_gb300.fleet import FleetEngine
    from yaff_gb300.serve import summarize
    reqs = _reqs(40, nmax=900, nsteps=20, seed=21)
    big = _reqs(1, nmax=4000, nsteps=20, seed=99)[0]
    big.natom = 1 << 20                # larger than the whole fleet
    cancelled = reqs[10]
    cancelled.cancel()
    eng = FleetEngine(max_atoms=1 << 15, max_systems=16, max_k=1 << 17, chunk=5)
    wall = eng.run(reqs + [big], realtime=False)
    s = summarize(reqs, wall)
    assert big.error.startswith('rejected')
    assert cancelled.error == 'cancelled'
    ok = [r for r in reqs if r is not cancelled]
    assert all(r.error is None for r in ok), [r.error for r in ok if r.error]
    assert s['errors'] == 1
    assert eng.peak_inflight >= 2
    for r in ok:
        assert r.log.shape == (r.nsteps + 1, 2) and np.isfinite(r.log).all()
    # one request again, alone in a fresh engine: bitwise the same
    again = _reqs(40, nmax=900, nsteps=20, seed=21)[7]
    solo = FleetEngine(max_atoms=1 << 15, max_systems=16, max_k=1 << 17, chunk=5)
    solo.run([again], realtime=False)
    np.testing.assert_array_equal(again.log, reqs[7].log)
    np.testing.assert_array_equal(again.pos, reqs[7].pos)


def test_fleet_rejects_systems_it_cannot_hold():
    """A cell smaller than (rcut + skin) / 2.5 needs more than two periodic
    images per axis, and a large cell with a fine reciprocal grid needs more
    than 64 phase-table entries per atom: both are refused with
    YG_ERR_ARG (a ValueError) before anything is copied, and the fleet keeps
    stepping its other systems."""
    from yaff_gb300 import configs
    from yaff_gb300.units import femtosecond
    dt = 0.5 * femtosecond
    fl = _fleet()
    ok = _reqs(1, nmax=300, nsteps=5, seed=4)[0]
    s_ok = fl.add(ok.spec, _vel(ok), 5, dt)
    tiny = configs.serving_request(2, 1)              # a 3.1 A cube, rcut 10 A: three images per axis
    with pytest.raises(ValueError):
        fl.add(tiny, np.zeros((2, 3)), 5, dt)
    fine = configs.serving_request(400, 2)
    fine['ewald'] = dict(fine['ewald'], gcut=fine['ewald']['gcut'] * 6.0)   # about 6x the k-vectors per axis
    with pytest.raises(ValueError):
        fl.add(fine, np.zeros((400, 3)), 5, dt)
    res = _run(fl, [s_ok], 5)
    assert not res[s_ok][3] and np.isfinite(res[s_ok][2]).all()
