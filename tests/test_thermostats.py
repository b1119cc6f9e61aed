"""CPU: the host VerletIntegrator with each thermostat hook (Berendsen,
Langevin, CSVR, Nose-Hoover chain), driving the oracle force field, follows
the reference's own VerletIntegrator trajectories stored in
tests/golden/md_thermostats.npz (made by make_md_golden.py): positions,
velocities, kinetic and conserved energies over 12 steps.  The stochastic
thermostats draw from NumPy's global generator in the reference's call
order, seeded as the reference run was."""
import os
import types

import numpy as np
import pytest

import golden_cases as gc
from oracle import OracleForceField
from yaff_gb300 import configs, verlet

DATA = dict(np.load(os.path.join(gc.GOLDEN, 'md_thermostats.npz')))


def _oracle_ff(spec):
    orc = OracleForceField(spec)
    orc.system = types.SimpleNamespace(pos=orc.pos, masses=spec['masses'], cell=orc.cell)
    return orc


def _hook(name):
    T, tc = float(DATA['temp']), float(DATA['timecon'])
    if name == 'berendsen':
        return verlet.BerendsenThermostat(T, timecon=tc)
    if name == 'langevin':
        return verlet.LangevinThermostat(T, timecon=tc)
    if name == 'csvr':
        return verlet.CSVRThermostat(T, timecon=tc)
    return verlet.NHCThermostat(T, timecon=tc, chainlength=3, chain_vel0=DATA['chain_vel0'].copy())


@pytest.mark.parametrize('name', ['berendsen', 'langevin', 'csvr', 'nhc'])
def test_host_thermostat_matches_reference(name):
    spec = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
    assert np.array_equal(spec['pos'], DATA['pos0'])
    ff = _oracle_ff(spec)
    np.random.seed(int(DATA['%s_seed' % name]))
    vi = verlet.VerletIntegrator(ff, float(DATA['timestep']), vel0=DATA['vel0'].copy(), hooks=[_hook(name)])
    assert vi.ndof == int(DATA['%s_ndof' % name])
    pos, vel = DATA['%s_pos' % name], DATA['%s_vel' % name]
    econs, ekin = DATA['%s_econs' % name], DATA['%s_ekin' % name]
    for s in range(int(DATA['nstep']) + 1):
        if s:
            vi.propagate()
        assert np.allclose(vi.pos, pos[s], rtol=0, atol=1e-11 * abs(pos[s]).max()), (name, s)
        assert np.allclose(vi.vel, vel[s], rtol=0, atol=1e-9 * abs(vel[s]).max()), (name, s)
        assert abs(vi.ekin - ekin[s]) <= 1e-10 * abs(ekin[s]), (name, s)
        assert abs(vi.econs - econs[s]) <= 1e-10 * abs(econs[s]), (name, s)


def test_ndof_and_momenta():
    assert verlet.get_ndof_internal_md(10, 3) == 27
    assert verlet.get_ndof_internal_md(2, 0) == 1
    assert verlet.get_ndof_internal_md(10, 0) == 24
    rng = np.random.default_rng(1)
    pos, vel, m = rng.normal(size=(20, 3)), rng.normal(size=(20, 3)), rng.uniform(1, 2, 20)
    verlet.clean_momenta(pos, vel, m, types.SimpleNamespace(nvec=0))
    assert np.allclose(m @ vel, 0, atol=1e-12)
    com = m @ pos / m.sum()
    assert np.allclose((np.cross(pos - com, vel) * m[:, None]).sum(0), 0, atol=1e-10)
