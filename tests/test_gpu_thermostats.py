"""GPU: thermostats inside the device-resident Verlet step.

Deterministic (Berendsen, Nose-Hoover chain): DeviceVerlet on the FP64
device force field follows the reference's own thermostatted trajectories
(tests/golden/md_thermostats.npz, 64 flexible waters, 12 steps of 0.5 fs):
positions within 1e-8 relative, per-step potential and kinetic energies and
the final conserved energy (with the thermostat's correction read from the
device) within 1e-8 relative.
Stochastic (Langevin, CSVR; device counter-based noise, so not the
reference's random stream): the time-averaged temperature of 1.5 ps after
0.5 ps of equilibration is within 3 % of the target, and the same seed
replays the same trajectory.
"""
import os

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

DATA = dict(np.load(os.path.join(gc.GOLDEN, 'md_thermostats.npz')))


def _spec():
    from yaff_gb300 import configs
    return configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')


def _thermostat(name, temp, timecon):
    from yaff_gb300 import verlet
    if name == 'berendsen':
        return verlet.BerendsenThermostat(temp, timecon=timecon)
    if name == 'langevin':
        return verlet.LangevinThermostat(temp, timecon=timecon)
    if name == 'csvr':
        return verlet.CSVRThermostat(temp, timecon=timecon)
    return verlet.NHCThermostat(temp, timecon=timecon, chainlength=3, chain_vel0=DATA['chain_vel0'].copy())


@pytest.mark.parametrize('name', ['berendsen', 'nhc'])
def test_device_thermostat_follows_reference(name):
    import yaff_gb300
    from yaff_gb300.verlet import DeviceVerlet
    spec = _spec()
    ff = yaff_gb300.build_forcefield(spec, precision='fp64')
    th = _thermostat(name, float(DATA['temp']), float(DATA['timecon']))
    nstep = int(DATA['nstep'])
    md = DeviceVerlet(ff, float(DATA['timestep']), vel0=DATA['vel0'].copy(), thermostat=th, max_steps=nstep)
    assert md.ndof == int(DATA['%s_ndof' % name])
    md.run(nstep)
    pos, vel, log = md.fetch()
    ref_pos = DATA['%s_pos' % name]
    assert np.allclose(pos, ref_pos[-1], rtol=0, atol=1e-8 * abs(ref_pos[-1]).max())
    assert np.allclose(log[:, 0], DATA['%s_epot' % name], rtol=1e-8, atol=0)
    assert np.allclose(log[:, 1], DATA['%s_ekin' % name], rtol=1e-8, atol=0)
    corr, _, _ = md.thermo_state()
    econs = log[-1, 0] + log[-1, 1] + corr
    ref = float(DATA['%s_econs' % name][-1])
    assert abs(econs - ref) <= 1e-8 * abs(ref)


@pytest.mark.parametrize('name', ['langevin', 'csvr'])
def test_device_stochastic_thermostat_temperature(name):
    import yaff_gb300
    from yaff_gb300.units import femtosecond, boltzmann
    from yaff_gb300.verlet import DeviceVerlet
    spec = _spec()
    temp = 300.0
    ff = yaff_gb300.build_forcefield(spec, precision='mixed')
    n_eq, n_run = 1000, 3000
    runs = []
    for rep in range(2):
        th = _thermostat(name, temp, 25 * femtosecond)
        md = DeviceVerlet(ff, 0.5 * femtosecond, vel0=DATA['vel0'].copy(), thermostat=th, seed=1234,
                          max_steps=n_eq + n_run)
        md.run(n_eq + n_run)
        pos, vel, log = md.fetch()
        runs.append((pos, log))
        if rep == 0:
            t_mean = (2.0 * log[n_eq + 1:, 1] / (md.ndof * boltzmann)).mean()
            assert abs(t_mean - temp) <= 0.03 * temp, (name, t_mean)
    # a replay with the same seed gives the same trajectory
    assert np.allclose(runs[0][1][:200], runs[1][1][:200], rtol=1e-9, atol=0)


BARO = dict(np.load(os.path.join(gc.GOLDEN, 'md_barostats.npz')))


@pytest.mark.parametrize('name', ['iso', 'aniso'])
def test_barostat_on_device_force_field(name):
    """The host Berendsen barostat (with the Berendsen thermostat) driving
    the FP64 device force field through cell changes (ForceField.update_rvecs:
    new cell, k-space set-up and list) follows the reference trajectory."""
    import yaff_gb300
    from yaff_gb300 import verlet
    spec = _spec()
    ff = yaff_gb300.build_forcefield(spec, precision='fp64')
    T, tc = float(BARO['temp']), float(BARO['timecon'])
    th = verlet.BerendsenThermostat(T, timecon=tc)
    baro = verlet.BerendsenBarostat(ff, T, float(BARO['press']), timecon=float(BARO['baro_timecon']),
                                    anisotropic=(name == 'aniso'))
    vi = verlet.VerletIntegrator(ff, float(BARO['timestep']), vel0=BARO['vel0'].copy(), hooks=[th, baro])
    vi.run(int(BARO['nstep']))
    ref = BARO['%s_pos' % name][-1]
    assert np.allclose(vi.pos, ref, rtol=0, atol=1e-8 * abs(ref).max())
    assert np.allclose(ff.system.cell.rvecs, BARO['%s_rvecs' % name][-1], rtol=0, atol=1e-9 * 30)
    assert abs(vi.econs - BARO['%s_econs' % name][-1]) <= 1e-8 * abs(BARO['%s_econs' % name][-1])
