"""CPU: the XYZ trajectory hook writes one frame per selected step (atom
count, title with counter, potential energy and cell in angstrom, symbols
and positions in angstrom) while the host integrator runs on the oracle."""
import types

import numpy as np

from oracle import OracleForceField
from yaff_gb300 import configs, verlet
from yaff_gb300.io import XYZWriter
from yaff_gb300.units import angstrom, femtosecond


def test_xyz_trajectory(tmp_path):
    spec = configs.flexible_water(nside=2, box=6.21, rcut=3.0, skin=0.3, name='water8')
    orc = OracleForceField(spec)
    n = len(spec['pos'])
    numbers = np.where(np.arange(n) % 3 == 0, 8, 1)
    orc.system = types.SimpleNamespace(pos=orc.pos, masses=spec['masses'], cell=orc.cell, numbers=numbers)
    fn = str(tmp_path / 'traj.xyz')
    w = XYZWriter(fn, start=1, step=2, select=np.arange(6))
    vi = verlet.VerletIntegrator(orc, 0.5 * femtosecond, temp0=300.0, rng=np.random.default_rng(0), hooks=[w])
    frames = []
    for _ in range(5):
        vi.propagate()
        if vi.counter % 2 == 1:
            frames.append((vi.counter, vi.epot, vi.pos[:6].copy()))
    lines = open(fn).read().splitlines()
    assert len(lines) == len(frames) * 8
    for f, (counter, epot, pos) in enumerate(frames):
        blk = lines[8 * f:8 * f + 8]
        assert int(blk[0]) == 6
        title = blk[1].split()
        assert int(title[0]) == counter and abs(float(title[3]) - epot) <= 1e-9 * abs(epot)
        assert np.allclose([float(x) for x in title[4:]], spec['rvecs'].ravel() / angstrom)
        syms = [l.split()[0] for l in blk[2:]]
        assert syms == ['O', 'H', 'H', 'O', 'H', 'H']
        xyz = np.array([[float(x) for x in l.split()[1:]] for l in blk[2:]])
        assert np.allclose(xyz, pos / angstrom, atol=1e-9)


import pytest  # noqa: E402


@pytest.mark.parametrize('thermo', [None, 'nhc', 'berendsen'])
def test_restart_continues_the_run(tmp_path, thermo):
    """A run continued from a RestartWriter record (written at step 10)
    repeats the last 5 steps of the uninterrupted run: positions,
    velocities, conserved energy and counter."""
    from yaff_gb300.io import RestartWriter, read_restart
    spec = configs.flexible_water(nside=2, box=6.21, rcut=3.0, skin=0.3, name='water8')
    dt = 0.5 * femtosecond

    def make_ff():
        orc = OracleForceField(spec)
        orc.system = types.SimpleNamespace(pos=orc.pos, masses=spec['masses'], cell=orc.cell,
                                           numbers=np.where(np.arange(len(spec['pos'])) % 3 == 0, 8, 1))
        return orc

    def make_thermo():
        if thermo == 'nhc':
            return [verlet.NHCThermostat(300.0, timecon=20 * femtosecond, chainlength=3)]
        if thermo == 'berendsen':
            return [verlet.BerendsenThermostat(300.0, timecon=20 * femtosecond)]
        return []

    fn = str(tmp_path / 'restart.npz')
    vi = verlet.VerletIntegrator(make_ff(), dt, temp0=300.0, rng=np.random.default_rng(0),
                                 hooks=make_thermo() + [RestartWriter(fn, start=5, step=5)])
    vi.run(10)
    state = read_restart(fn)
    assert int(state['counter']) == 10
    assert np.array_equal(state['pos'], vi.pos) and np.array_equal(state['vel'], vi.vel)
    vi.run(5)
    vi2 = verlet.VerletIntegrator(make_ff(), hooks=make_thermo(), restart=state)   # the step-10 record
    assert vi2.counter == 10 and vi2.timestep == dt
    assert vi2.econs == pytest.approx(float(state['econs']), rel=1e-12, abs=1e-14)
    vi2.run(5)
    assert vi2.counter == 15
    assert np.abs(vi2.pos - vi.pos).max() <= 1e-12 * np.abs(vi.pos).max()
    assert np.abs(vi2.vel - vi.vel).max() <= 1e-10 * np.abs(vi.vel).max()
    assert vi2.econs == pytest.approx(vi.econs, rel=1e-10)
