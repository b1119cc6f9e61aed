"""CPU: the host VerletIntegrator with each thermostat hook (Berendsen,
Langevin, CSVR, Nose-Hoover chain), driving the oracle force field, follows
the reference's own VerletIntegrator trajectories stored in
tests/golden/md_thermostats.npz (made by make_md_golden.py): positions,
velocities, kinetic and conserved energies over 12 steps; with the Berendsen
barostat added (isotropic and anisotropic), positions, cells, potential and
conserved energies follow tests/golden/md_barostats.npz.  The stochastic
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


BARO = dict(np.load(os.path.join(gc.GOLDEN, 'md_barostats.npz')))


class _OracleAdapter(object):
    """The oracle as a force field whose system follows its cell."""

    def __init__(self, spec):
        self.orc = OracleForceField(spec)
        self.system = types.SimpleNamespace(pos=self.orc.pos, masses=spec['masses'], cell=self.orc.cell)

    def __getattr__(self, name):
        return getattr(self.orc, name)

    def update_rvecs(self, rvecs):
        self.orc.update_rvecs(rvecs)
        self.system.cell = self.orc.cell


@pytest.mark.parametrize('name', ['iso', 'aniso'])
def test_host_barostat_matches_reference(name):
    spec = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
    ff = _OracleAdapter(spec)
    T, tc = float(BARO['temp']), float(BARO['timecon'])
    th = verlet.BerendsenThermostat(T, timecon=tc)
    baro = verlet.BerendsenBarostat(ff, T, float(BARO['press']), timecon=float(BARO['baro_timecon']),
                                    anisotropic=(name == 'aniso'))
    vi = verlet.VerletIntegrator(ff, float(BARO['timestep']), vel0=BARO['vel0'].copy(), hooks=[th, baro])
    for s in range(int(BARO['nstep']) + 1):
        if s:
            vi.propagate()
        ref = BARO['%s_pos' % name][s]
        assert np.allclose(vi.pos, ref, rtol=0, atol=1e-11 * abs(ref).max()), (name, s)
        assert np.allclose(ff.orc.cell.rvecs, BARO['%s_rvecs' % name][s], rtol=0, atol=1e-12 * 30), (name, s)
        assert abs(vi.epot - BARO['%s_epot' % name][s]) <= 1e-10 * abs(BARO['%s_epot' % name][s])
        assert abs(vi.econs - BARO['%s_econs' % name][s]) <= 1e-10 * abs(BARO['%s_econs' % name][s])


NPT = dict(np.load(os.path.join(gc.GOLDEN, 'md_npt.npz')))


def _npt_hooks(name, ff):
    T, tc = float(NPT['temp']), float(NPT['timecon'])
    press, btc = float(NPT['press']), float(NPT['baro_timecon'])
    cv0 = NPT['chain_vel0']
    if name == 'mtk_nhc_aniso':
        return [verlet.NHCThermostat(T, timecon=tc, chainlength=3, chain_vel0=cv0.copy()),
                verlet.MTKBarostat(ff, T, press, timecon=btc, anisotropic=True)]
    if name == 'mtk_nhc_iso':
        return [verlet.NHCThermostat(T, timecon=tc, chainlength=3, chain_vel0=cv0.copy()),
                verlet.MTKBarostat(ff, T, press, timecon=btc, anisotropic=False)]
    if name == 'mtk_cellchain':
        return [verlet.NHCThermostat(T, timecon=tc, chainlength=3, chain_vel0=cv0.copy()),
                verlet.MTKBarostat(ff, T, press, timecon=btc, anisotropic=True,
                                   baro_thermo=verlet.NHCThermostat(T, timecon=tc, chainlength=3))]
    if name == 'langevin_berendsen_aniso':
        return [verlet.BerendsenThermostat(T, timecon=tc),
                verlet.LangevinBarostat(ff, T, press, timecon=btc, anisotropic=True)]
    return [verlet.LangevinThermostat(T, timecon=tc),
            verlet.LangevinBarostat(ff, T, press, timecon=btc, anisotropic=False)]


@pytest.mark.parametrize('name', ['mtk_nhc_aniso', 'mtk_nhc_iso', 'mtk_cellchain', 'langevin_berendsen_aniso',
                                  'langevin_langevin_iso'])
def test_host_npt_matches_reference(name):
    """MTK barostat (with a particle Nose-Hoover chain, isotropic and
    anisotropic, and with a chain of its own on the cell) and Langevin
    barostat (with Berendsen and Langevin thermostats), combined as the
    reference combines them, follow the reference's trajectories
    (tests/golden/md_npt.npz): positions, velocities, cells, potential,
    kinetic and conserved energies over 12 steps; random draws from NumPy's
    global generator seeded as the reference run was."""
    spec = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
    ff = _OracleAdapter(spec)
    np.random.seed(int(NPT['%s_seed' % name]))
    hooks = _npt_hooks(name, ff)
    vi = verlet.VerletIntegrator(ff, float(NPT['timestep']), vel0=NPT['vel0'].copy(), hooks=hooks)
    assert vi.ndof == int(NPT['%s_ndof' % name])
    for s in range(int(NPT['nstep']) + 1):
        if s:
            vi.propagate()
        ref = NPT['%s_pos' % name][s]
        assert np.allclose(vi.pos, ref, rtol=0, atol=1e-10 * abs(ref).max()), (name, s)
        vref = NPT['%s_vel' % name][s]
        assert np.allclose(vi.vel, vref, rtol=0, atol=1e-8 * abs(vref).max()), (name, s)
        assert np.allclose(ff.orc.cell.rvecs, NPT['%s_rvecs' % name][s], rtol=0, atol=1e-10 * 30), (name, s)
        for key in ('epot', 'ekin', 'econs'):
            r = NPT['%s_%s' % (name, key)][s]
            assert abs(getattr(vi, key) - r) <= 1e-9 * max(abs(r), 1.0), (name, key, s)
