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
