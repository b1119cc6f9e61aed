"""GPU: NVE of the 24,000-atom flexible water workload against the reference.

tests/golden/md_water24000.npz holds the reference's own VerletIntegrator
(yaff/sampling/verlet.py:320-367) driving the reference ForceField on this
system: 10 steps of 0.5 fs from stored initial velocities, with the
potential, kinetic and conserved energies of every step and the positions and
velocities after the last one.  Both integrators of this package -- the
host-driven VerletIntegrator on ForceField.compute (the reference's call
sequence) and the device-resident DeviceVerlet replayed from a CUDA graph --
start from the same velocities and must follow that trajectory:

* FP64 form: energies within 1e-9 of the largest conserved-energy magnitude,
  positions within 1e-8 relative, velocities within 1e-7 relative RMS;
* mixed forms: energies within 1e-6, positions within 1e-6 relative,
  velocities within 1e-4 relative RMS.
"""
import os

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = {'fp64': (1e-9, 1e-8, 1e-7), 'mixed': (1e-6, 1e-6, 1e-4)}


@pytest.fixture(scope='module')
def ref():
    path = os.path.join(gc.GOLDEN, 'md_water24000.npz')
    return dict(np.load(path))


def _check(ep, ek, pos, vel, ref, precision):
    etol, ptol, vtol = TOL[precision]
    scale = np.abs(ref['econs']).max()
    assert np.abs(ep - ref['epot']).max() <= etol * scale, np.abs(ep - ref['epot']).max() / scale
    assert np.abs(ek - ref['ekin']).max() <= etol * scale, np.abs(ek - ref['ekin']).max() / scale
    assert np.abs(pos - ref['pos_last']).max() <= ptol * np.abs(ref['pos_last']).max()
    assert gc.rel_rms(vel, ref['vel_last']) <= vtol


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_device_verlet_follows_reference(ref, precision):
    import yaff_gb300
    from yaff_gb300 import configs
    from yaff_gb300.verlet import DeviceVerlet
    spec = configs.water_24000()
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    dv = DeviceVerlet(ff, float(ref['timestep']), vel0=ref['vel0'], max_steps=64, use_graph=True)
    n = int(ref['nstep'])
    dv.run(n)
    pos, vel, log = dv.fetch()
    assert log.shape == (n + 1, 2)
    _check(log[:, 0], log[:, 1], pos, vel, ref, precision)


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_host_verlet_follows_reference(ref, precision):
    import yaff_gb300
    from yaff_gb300 import configs
    from yaff_gb300.verlet import VerletIntegrator
    spec = configs.water_24000()
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    ep, ek = [], []

    def hook(it):
        ep.append(it.epot)
        ek.append(it.ekin)
    vi = VerletIntegrator(ff, float(ref['timestep']), vel0=ref['vel0'].copy(), hooks=[hook])
    ep.append(vi.epot)   # step 0 (plain hooks run after each step only)
    ek.append(vi.ekin)
    vi.run(int(ref['nstep']))
    _check(np.array(ep), np.array(ek), vi.pos, vi.vel, ref, precision)
