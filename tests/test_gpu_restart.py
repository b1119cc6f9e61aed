"""GPU: snapshot and resume of the device-resident integrator.

DeviceVerlet.save_restart writes the run's state in the layout of
io.RestartWriter (the reference's restart record, yaff/sampling/io.py:
159-287, as .npz); DeviceVerlet(restart=...) continues from it.  A run
stopped after 20 steps, saved and resumed must repeat the last 10 steps of
the uninterrupted run (FP64; the resumed run builds its neighbour list at
step 20, so only the summation order of the pair terms can differ: 1e-9),
for NVE and with the Nose-Hoover chain, whose chain state is part of the
record; the counter continues.  The host integrator resumes from the same
record."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec():
    from yaff_gb300 import configs
    return configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64restart')


@pytest.mark.parametrize('thermo', [None, 'nhc'])
def test_device_verlet_resumes_from_snapshot(tmp_path, thermo):
    import yaff_gb300
    from yaff_gb300.io import read_restart
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import DeviceVerlet, NHCThermostat, VerletIntegrator
    spec = _spec()
    dt = 0.5 * femtosecond
    vel0 = np.random.default_rng(2).normal(0, 1, spec['pos'].shape) * \
        np.sqrt(300 * 3.166811563e-6 / spec['masses'])[:, None]

    def thermostat():
        return None if thermo is None else NHCThermostat(300.0, timecon=20 * femtosecond, chainlength=3,
                                                          chain_vel0=np.array([1e-4, -2e-4, 5e-5]))

    ff = yaff_gb300.build_forcefield(spec, precision='fp64')
    dv = DeviceVerlet(ff, dt, vel0=vel0, max_steps=64, thermostat=thermostat())
    dv.run(20)
    fn = str(tmp_path / 'snap.npz')
    dv.save_restart(fn)
    dv.run(10)
    p_ref, v_ref, log_ref = dv.fetch()
    st = read_restart(fn)
    assert int(st['counter']) == 20

    ff2 = yaff_gb300.build_forcefield(spec, precision='fp64')
    dv2 = DeviceVerlet(ff2, max_steps=64, thermostat=thermostat(), restart=fn)
    assert dv2.counter0 == 20 and dv2.timestep == dt
    dv2.run(10)
    p2, v2, log2 = dv2.fetch()
    assert np.abs(p2 - p_ref).max() <= 1e-9 * np.abs(p_ref).max()
    assert np.abs(v2 - v_ref).max() <= 1e-7 * np.abs(v_ref).max()
    assert np.abs(log2[-1] - log_ref[-1]).max() <= 1e-9 * np.abs(log_ref[-1]).max()
    if thermo == 'nhc':
        c1, cp1, cv1 = dv.thermo_state()
        c2, cp2, cv2 = dv2.thermo_state()
        assert np.allclose(cp2, cp1, rtol=1e-8, atol=1e-12) and np.allclose(cv2, cv1, rtol=1e-7, atol=1e-12)
    # the host integrator continues from the same record
    if thermo is None:
        ff3 = yaff_gb300.build_forcefield(spec, precision='fp64')
        vi = VerletIntegrator(ff3, restart=fn)
        assert vi.counter == 20
        vi.run(10)
        assert np.abs(vi.pos - p_ref).max() <= 1e-9 * np.abs(p_ref).max()
