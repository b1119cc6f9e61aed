"""Plain-text trajectory output for the integrators.

XYZWriter is the reference's XYZ trajectory hook (yaff/sampling/io.py:
113-156): one frame per call (every `step` steps from `start`), the atom
count, a title line with the step counter, the potential energy and the cell
vectors in angstrom, then one line per atom with its element symbol and
Cartesian position in angstrom.  It works as a plain hook of
VerletIntegrator; ``write_frame`` writes a frame from arrays (for example
positions fetched from a DeviceVerlet run).  HDF5 output is not offered
(h5py is not part of this build).
"""
import numpy as np

from .units import angstrom

__all__ = ['XYZWriter', 'SYMBOLS']

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
