"""Trajectory and restart output for the integrators.

XYZWriter is the reference's XYZ trajectory hook (yaff/sampling/io.py:
113-156): one frame per call (every `step` steps from `start`), the atom
count, a title line with the step counter, the potential energy and the cell
vectors in angstrom, then one line per atom with its element symbol and
Cartesian position in angstrom.  It works as a plain hook of
VerletIntegrator; ``write_frame`` writes a frame from arrays (for example
positions fetched from a DeviceVerlet run).

RestartWriter is the reference's restart hook (yaff/sampling/io.py:159-287)
with a plain NumPy .npz file instead of HDF5 (h5py is not part of this
build): every `step` steps from `start` it replaces the file, atomically,
with the state an integrator needs to continue -- counter, time, time step,
positions, velocities, cell vectors, the conserved energy and the running
sums of its fluctuation tracker, and per Verlet hook (thermostat) its
conserved-energy correction and, for a Nose-Hoover chain, the chain's
positions and velocities.  ``read_restart`` returns it as a dict;
VerletIntegrator(restart=...) and DeviceVerlet(restart=...) continue from it.
"""
import os

import numpy as np

from .units import angstrom

__all__ = ['XYZWriter', 'RestartWriter', 'read_restart', 'restart_state', 'SYMBOLS']

# element symbols by atomic number (index 0 unused)
SYMBOLS = ('X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se '
           'Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er '
           'Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No '
           'Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og').split()


class XYZWriter(object):
    """Trajectory hook: appends a frame to `fn_xyz` every `step` steps from
    `start`; `select` restricts the frame to those atom indices."""

    def __init__(self, fn_xyz, select=None, start=0, step=1):
        self.fn_xyz = fn_xyz
        self.select = None if select is None else np.asarray(select, dtype=np.int64)
        self.start = start
        self.step = step
        self._symbols = None
        open(fn_xyz, 'w').close()

    def expects_call(self, counter):
        return counter >= self.start and (counter - self.start) % self.step == 0

    def __call__(self, iterative):
        if not self.expects_call(iterative.counter):
            return
        system = iterative.ff.system
        self.write_frame(system.numbers, iterative.pos, getattr(system.cell, 'rvecs', np.zeros((0, 3))),
                         iterative.counter, iterative.epot)

    def write_frame(self, numbers, pos, rvecs, counter, epot):
        if self._symbols is None:
            numbers = np.asarray(numbers)
            if self.select is not None:
                numbers = numbers[self.select]
            self._symbols = [SYMBOLS[int(n)] if 0 < int(n) < len(SYMBOLS) else 'X' for n in numbers]
        pos = np.asarray(pos)
        if self.select is not None:
            pos = pos[self.select]
        cell = ' '.join(str(x / angstrom) for x in np.asarray(rvecs, float).ravel())
        lines = ['%d' % len(pos), '%7i E_pot = %.10f    %s' % (counter, epot, cell)]
        for sym, p in zip(self._symbols, pos / angstrom):
            lines.append('%-2s % 15.10f % 15.10f % 15.10f' % (sym, p[0], p[1], p[2]))
        with open(self.fn_xyz, 'a') as fh:
            fh.write('\n'.join(lines) + '\n')


def restart_state(counter, time, timestep, pos, vel, rvecs, econs=np.nan, cons_err=None, hooks=()):
    """The restart record (a dict of arrays) of an integrator state."""
    st = {'counter': np.array(int(counter)), 'time': np.array(float(time)), 'timestep': np.array(float(timestep)),
          'pos': np.array(pos, dtype=np.float64), 'vel': np.array(vel, dtype=np.float64),
          'rvecs': np.array(rvecs, dtype=np.float64).reshape(-1, 3), 'econs': np.array(float(econs))}
    if cons_err is not None:
        st['cons_err'] = np.array([cons_err.counter, cons_err.ekin_m, cons_err.ekin_s, cons_err.econs_m,
                                   cons_err.econs_s], dtype=np.float64)
    corr, names = [], []
    for k, hook in enumerate(hooks):
        names.append(type(hook).__name__)
        corr.append(float(getattr(hook, 'econs_correction', 0.0)))
        chain = getattr(hook, 'chain', None)
        if chain is not None:
            st['hook%d_chain_pos' % k] = np.array(chain.pos, dtype=np.float64)
            st['hook%d_chain_vel' % k] = np.array(chain.vel, dtype=np.float64)
    st['hook_names'] = np.array(names if names else [''])
    st['hook_econs_correction'] = np.array(corr, dtype=np.float64)
    return st


def _write_npz(fn, state):
    tmp = '%s.%d.tmp.npz' % (fn, os.getpid())
    np.savez(tmp, **state)
    os.replace(tmp, fn)


def read_restart(fn):
    """The state a RestartWriter (or DeviceVerlet.save_restart) wrote."""
    with np.load(fn, allow_pickle=False) as d:
        return dict((k, d[k]) for k in d.files)


class RestartWriter(object):
    """Restart hook of VerletIntegrator: writes the integrator's state to
    `fn` (.npz, replaced atomically) every `step` steps from `start`."""

    def __init__(self, fn, start=0, step=1000):
        self.fn = fn
        self.start = start
        self.step = step

    def expects_call(self, counter):
        return counter >= self.start and (counter - self.start) % self.step == 0

    def __call__(self, iterative):
        if not self.expects_call(iterative.counter):
            return
        from .verlet import VerletHook
        hooks = [h for h in iterative.hooks if isinstance(h, VerletHook)]
        cell = getattr(iterative.ff.system, 'cell', None)
        rvecs = cell.rvecs if cell is not None else np.zeros((0, 3))
        _write_npz(self.fn, restart_state(iterative.counter, iterative.time, iterative.timestep, iterative.pos,
                                          iterative.vel, rvecs, iterative.econs, iterative.cons_err, hooks))
