"""GPU: NVE velocity Verlet driven by the device force field, against the
same integrator driven by the oracle (the reference's algorithm on the CPU).

System: 64 flexible waters (192 atoms, 12.42 A box), LJ + EI + Ewald + bonds
and bends with 1-2/1-3 exclusions, rcut 5 A, skin 0.5 A; 1000 steps of 0.5 fs
from seeded 300 K velocities.  Checks: the first 20 steps follow the oracle
trajectory (FP64 form: 1e-8 relative on positions); the conserved-energy
drift (linear fit, per atom and ps) and the reference's conserved-energy
fluctuation ratio sqrt(var Econs / var Ekin) are no worse than the oracle's
(a 25 % margin, no absolute floor: the oracle's drift on this system is
4.6e-5 Ha/atom/ps, its fluctuation ratio 0.022).
"""
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NSTEP = 1000


def _spec():
    from yaff_gb300 import configs
    return configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64nve')


def _run(ff, spec, nstep, record):
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import VerletIntegrator
    rng = np.random.default_rng(11)
    times, econs, traj = [], [], []

    def hook(it):
        times.append(it.time)
        econs.append(it.econs)
        if it.counter <= record:
            traj.append(it.pos.copy())
    vi = VerletIntegrator(ff, 0.5 * femtosecond, temp0=300.0, rng=rng, hooks=[hook])
    vi.run(nstep)
    return np.array(times), np.array(econs), traj, vi.cons_err.get()


@pytest.fixture(scope='module')
def oracle_run():
    from oracle import OracleForceField
    spec = _spec()
    orc = OracleForceField(spec)
    orc.system = types.SimpleNamespace(pos=orc.pos, masses=spec['masses'])
    return _run(orc, spec, NSTEP, 20)


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_nve_drift_no_worse_than_reference(oracle_run, precision):
    import yaff_gb300
    from yaff_gb300.verlet import drift_per_ps
    spec = _spec()
    natom = len(spec['pos'])
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    t, e, traj, ratio = _run(ff, spec, NSTEP, 20)
    t_ref, e_ref, traj_ref, ratio_ref = oracle_run
    if precision == 'fp64':
        for a, b in zip(traj, traj_ref):
            assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max()
    d = abs(drift_per_ps(t, e, natom))
    d_ref = abs(drift_per_ps(t_ref, e_ref, natom))
    assert d <= 1.25 * d_ref, (d, d_ref)
    assert ratio <= 1.25 * ratio_ref, (ratio, ratio_ref)
    assert ff.nlist.nrebuild >= 1 and ff.nlist.nrecompute >= 1


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_device_verlet_follows_reference_and_drift(oracle_run, precision):
    """The device-resident integrator (graph replay, on-device skin test):
    the first 20 steps follow the oracle trajectory (FP64: 1e-8 relative),
    and over 1000 steps its drift and fluctuation ratio are no worse than the
    oracle's, with the same margins as the host-driven integrator."""
    import yaff_gb300
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import DeviceVerlet, ConsErrTracker, drift_per_ps
    spec = _spec()
    natom = len(spec['pos'])
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    dt = 0.5 * femtosecond
    dv = DeviceVerlet(ff, dt, temp0=300.0, rng=np.random.default_rng(11), max_steps=NSTEP, use_graph=True)
    dv.run(20)
    p20, _, _ = dv.fetch(vel=False)
    t_ref, e_ref, traj_ref, ratio_ref = oracle_run
    tol = 1e-8 if precision == 'fp64' else 1e-5
    assert np.abs(p20 - traj_ref[19]).max() <= tol * np.abs(traj_ref[19]).max()
    dv.run(NSTEP - 20)
    _, _, log = dv.fetch(pos=False, vel=False)
    assert log.shape == (NSTEP + 1, 2) and np.isfinite(log).all()
    econs = log[:, 0] + log[:, 1]
    # same conserved quantity as the oracle-driven run while the trajectories
    # still coincide (later they decorrelate; only the statistics compare)
    etol = 1e-9 if precision == 'fp64' else 1e-6
    assert abs(econs[1:21] - e_ref[:20]).max() <= etol * np.abs(e_ref).max()
    tr = ConsErrTracker()
    for ep, ek in log:
        tr.update(ek, ep + ek)
    times = dt * np.arange(1, NSTEP + 1)
    d = abs(drift_per_ps(times, econs[1:], natom))
    d_ref = abs(drift_per_ps(t_ref, e_ref, natom))
    assert d <= 1.25 * d_ref, (d, d_ref)
    assert tr.get() <= 1.25 * ratio_ref, (tr.get(), ratio_ref)
    assert dv.nrebuild >= 1
