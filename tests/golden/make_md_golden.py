"""Generate tests/golden/md_thermostats.npz by running the reference.

Run in a container that holds the reference checkout ($YAFF_REFERENCE) after
``sh oracle/build_ref.sh``:

    python tests/golden/make_md_golden.py            # thermostats, barostats
    python tests/golden/make_md_golden.py water24000 # md_water24000.npz only
    python tests/golden/make_md_golden.py npt        # md_npt.npz only (Langevin, MTK barostats)

For each thermostat of the reference (Berendsen, Langevin, CSVR, Nose-Hoover
chain) the script runs the reference's own VerletIntegrator with that hook on
the 64-molecule flexible water box (reference force field), 12 steps of
0.5 fs from fixed initial velocities (md_thermostats.npz), and the Berendsen
barostat with the Berendsen thermostat, isotropic and anisotropic
(md_barostats.npz), and stores positions, velocities,
kinetic, potential and conserved energies and the degrees of freedom per
step.  The stochastic thermostats draw from NumPy's global generator, seeded
per run (stored), in the reference's call order.
"""
import os
import sys
import warnings

import numpy as np

warnings.filterwarnings('ignore')
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, 'oracle'))

from yaff_gb300 import configs  # noqa: E402
from yaff_gb300.units import femtosecond, kelvin  # noqa: E402
import ref_shim  # noqa: E402
from ref_ff import build_reference_ff  # noqa: E402

NSTEP = 12
TIMESTEP = 0.5 * femtosecond
TEMP = 300.0 * kelvin
TIMECON = 20.0 * femtosecond


def main():
    if not ref_shim.reference_available():
        raise SystemExit('reference not available: run oracle/build_ref.sh first')
    ref_shim.import_reference()
    from yaff.sampling.verlet import VerletIntegrator
    from yaff.sampling.nvt import BerendsenThermostat, LangevinThermostat, CSVRThermostat, NHCThermostat
    spec = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
    rng = np.random.default_rng(99)
    natom = len(spec['pos'])
    vel0 = rng.normal(0, 1, (natom, 3)) * np.sqrt(1.2 * 300.0 * 3.166811563e-6 / spec['masses'])[:, None]
    chain_vel0 = np.array([1e-3, -2e-3, 5e-4]) / femtosecond * 1e-2
    data = {'pos0': spec['pos'], 'vel0': vel0, 'timestep': np.array(TIMESTEP), 'temp': np.array(TEMP),
            'timecon': np.array(TIMECON), 'chain_vel0': chain_vel0, 'nstep': np.array(NSTEP)}
    makers = {
        'berendsen': lambda: BerendsenThermostat(TEMP, timecon=TIMECON),
        'langevin': lambda: LangevinThermostat(TEMP, timecon=TIMECON),
        'csvr': lambda: CSVRThermostat(TEMP, timecon=TIMECON),
        'nhc': lambda: NHCThermostat(TEMP, timecon=TIMECON, chainlength=3, chain_vel0=chain_vel0.copy()),
    }
    for k, (name, make) in enumerate(makers.items()):
        ff = build_reference_ff(spec)
        seed = 1000 + k
        np.random.seed(seed)
        hook = make()
        vi = VerletIntegrator(ff, TIMESTEP, hooks=[hook], vel0=vel0.copy())
        rows = {'pos': [vi.pos.copy()], 'vel': [vi.vel.copy()], 'ekin': [vi.ekin], 'epot': [vi.epot],
                'econs': [vi.econs]}
        for _ in range(NSTEP):
            vi.propagate()
            rows['pos'].append(vi.pos.copy())
            rows['vel'].append(vi.vel.copy())
            rows['ekin'].append(vi.ekin)
            rows['epot'].append(vi.epot)
            rows['econs'].append(vi.econs)
        for key, v in rows.items():
            data['%s_%s' % (name, key)] = np.array(v)
        data['%s_seed' % name] = np.array(seed)
        data['%s_ndof' % name] = np.array(vi.ndof)
        print('%-10s ndof %d  T %.2f K  econs drift %.3e' % (name, vi.ndof, vi.temp / kelvin,
                                                              rows['econs'][-1] - rows['econs'][0]))
    np.savez_compressed(os.path.join(HERE, 'md_thermostats.npz'), **data)
    barostat_runs(spec, vel0)


def barostat_runs(spec, vel0):
    """Berendsen thermostat + Berendsen barostat (isotropic, and anisotropic
    with the cell symmetrized first) at 1 GPa -> md_barostats.npz: positions,
    cells, energies and the conserved energy per step."""
    from yaff.sampling.verlet import VerletIntegrator
    from yaff.sampling.nvt import BerendsenThermostat
    from yaff.sampling.npt import BerendsenBarostat
    from yaff_gb300.units import pascal
    press = 1e9 * pascal
    data = {'pos0': spec['pos'], 'vel0': vel0, 'timestep': np.array(TIMESTEP), 'temp': np.array(TEMP),
            'timecon': np.array(TIMECON), 'press': np.array(press), 'baro_timecon': np.array(200 * femtosecond),
            'nstep': np.array(NSTEP)}
    for name, aniso in (('iso', False), ('aniso', True)):
        ff = build_reference_ff(spec)
        th = BerendsenThermostat(TEMP, timecon=TIMECON)
        baro = BerendsenBarostat(ff, TEMP, press, timecon=200 * femtosecond, anisotropic=aniso)
        vi = VerletIntegrator(ff, TIMESTEP, hooks=[th, baro], vel0=vel0.copy())
        rows = {'pos': [vi.pos.copy()], 'rvecs': [ff.system.cell.rvecs.copy()], 'epot': [vi.epot],
                'econs': [vi.econs]}
        for _ in range(NSTEP):
            vi.propagate()
            rows['pos'].append(vi.pos.copy())
            rows['rvecs'].append(ff.system.cell.rvecs.copy())
            rows['epot'].append(vi.epot)
            rows['econs'].append(vi.econs)
        for key, v in rows.items():
            data['%s_%s' % (name, key)] = np.array(v)
        print('%-6s volume %.6f -> %.6f' % (name, np.linalg.det(rows['rvecs'][0]), np.linalg.det(rows['rvecs'][-1])))
    np.savez_compressed(os.path.join(HERE, 'md_barostats.npz'), **data)


def npt_runs(spec, vel0):
    """The reference's Langevin and MTK barostats with their thermostats
    (combined by the reference's VerletIntegrator into a TBCombination) at
    1 GPa -> md_npt.npz: positions, cells, energies and the conserved energy
    per step.  The random draws (barostat and chain velocities, Langevin
    forces) come from NumPy's global generator, seeded per run (stored)."""
    from yaff.sampling.verlet import VerletIntegrator
    from yaff.sampling.nvt import BerendsenThermostat, LangevinThermostat, NHCThermostat
    from yaff.sampling.npt import LangevinBarostat, MTKBarostat
    from yaff_gb300.units import pascal
    press = 1e9 * pascal
    btc = 200 * femtosecond
    chain_vel0 = np.array([1e-3, -2e-3, 5e-4]) / femtosecond * 1e-2
    data = {'pos0': spec['pos'], 'vel0': vel0, 'timestep': np.array(TIMESTEP), 'temp': np.array(TEMP),
            'timecon': np.array(TIMECON), 'press': np.array(press), 'baro_timecon': np.array(btc),
            'nstep': np.array(NSTEP), 'chain_vel0': chain_vel0}
    runs = {
        'mtk_nhc_aniso': lambda ff: [NHCThermostat(TEMP, timecon=TIMECON, chainlength=3, chain_vel0=chain_vel0.copy()),
                                     MTKBarostat(ff, TEMP, press, timecon=btc, anisotropic=True)],
        'mtk_nhc_iso': lambda ff: [NHCThermostat(TEMP, timecon=TIMECON, chainlength=3, chain_vel0=chain_vel0.copy()),
                                   MTKBarostat(ff, TEMP, press, timecon=btc, anisotropic=False)],
        'mtk_cellchain': lambda ff: [NHCThermostat(TEMP, timecon=TIMECON, chainlength=3, chain_vel0=chain_vel0.copy()),
                                     MTKBarostat(ff, TEMP, press, timecon=btc, anisotropic=True,
                                                 baro_thermo=NHCThermostat(TEMP, timecon=TIMECON, chainlength=3))],
        'langevin_berendsen_aniso': lambda ff: [BerendsenThermostat(TEMP, timecon=TIMECON),
                                                LangevinBarostat(ff, TEMP, press, timecon=btc, anisotropic=True)],
        'langevin_langevin_iso': lambda ff: [LangevinThermostat(TEMP, timecon=TIMECON),
                                             LangevinBarostat(ff, TEMP, press, timecon=btc, anisotropic=False)],
    }
    for k, (name, make) in enumerate(runs.items()):
        ff = build_reference_ff(spec)
        seed = 2000 + k
        np.random.seed(seed)
        hooks = make(ff)
        vi = VerletIntegrator(ff, TIMESTEP, hooks=hooks, vel0=vel0.copy())
        rows = {'pos': [vi.pos.copy()], 'vel': [vi.vel.copy()], 'rvecs': [ff.system.cell.rvecs.copy()],
                'epot': [vi.epot], 'ekin': [vi.ekin], 'econs': [vi.econs]}
        for _ in range(NSTEP):
            vi.propagate()
            rows['pos'].append(vi.pos.copy())
            rows['vel'].append(vi.vel.copy())
            rows['rvecs'].append(ff.system.cell.rvecs.copy())
            rows['epot'].append(vi.epot)
            rows['ekin'].append(vi.ekin)
            rows['econs'].append(vi.econs)
        for key, v in rows.items():
            data['%s_%s' % (name, key)] = np.array(v)
        data['%s_seed' % name] = np.array(seed)
        data['%s_ndof' % name] = np.array(vi.ndof)
        print('%-26s volume %.6f -> %.6f  econs %+.3e' % (name, np.linalg.det(rows['rvecs'][0]),
                                                          np.linalg.det(rows['rvecs'][-1]),
                                                          rows['econs'][-1] - rows['econs'][0]))
    np.savez_compressed(os.path.join(HERE, 'md_npt.npz'), **data)


def nve_water24000(nstep=10):
    """NVE of the 8,000-molecule (24,000-atom) flexible water workload with the
    reference's own VerletIntegrator and force field: nstep steps of 0.5 fs
    from seeded 300 K Maxwell velocities (stored) -> md_water24000.npz with the
    potential, kinetic and conserved energies of every step and the positions
    and velocities after the last step."""
    ref_shim.import_reference()
    from yaff.sampling.verlet import VerletIntegrator
    spec = configs.water_24000()
    natom = len(spec['pos'])
    rng = np.random.default_rng(24000)
    vel0 = rng.normal(0, 1, (natom, 3)) * np.sqrt(300.0 * 3.166811563e-6 / spec['masses'])[:, None]
    vel0 -= (spec['masses'][:, None] * vel0).sum(0) / spec['masses'].sum()
    ff = build_reference_ff(spec)
    vi = VerletIntegrator(ff, TIMESTEP, vel0=vel0.copy())
    rows = {'ekin': [vi.ekin], 'epot': [vi.epot], 'econs': [vi.econs]}
    for s in range(nstep):
        vi.propagate()
        for key in rows:
            rows[key].append(getattr(vi, key))
        print('  step %d  epot %.12e  ekin %.12e  econs %.12e' % (s + 1, vi.epot, vi.ekin, vi.econs), flush=True)
    data = {'vel0': vel0, 'timestep': np.array(TIMESTEP), 'nstep': np.array(nstep),
            'pos_last': vi.pos.copy(), 'vel_last': vi.vel.copy(), 'nrebuild': np.array(-1)}
    for key, v in rows.items():
        data[key] = np.array(v)
    np.savez_compressed(os.path.join(HERE, 'md_water24000.npz'), **data)


if __name__ == '__main__':
    if sys.argv[1:] == ['water24000']:
        if not ref_shim.reference_available():
            raise SystemExit('reference not available: run oracle/build_ref.sh first')
        nve_water24000()
    elif sys.argv[1:] == ['npt']:
        if not ref_shim.reference_available():
            raise SystemExit('reference not available: run oracle/build_ref.sh first')
        ref_shim.import_reference()
        spec = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
        rng = np.random.default_rng(99)
        vel0 = rng.normal(0, 1, (len(spec['pos']), 3)) * np.sqrt(1.2 * 300.0 * 3.166811563e-6 / spec['masses'])[:, None]
        npt_runs(spec, vel0)
    else:
        main()
