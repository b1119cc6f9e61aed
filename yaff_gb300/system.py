"""Periodic cell and system description (host side).

``Cell`` reproduces the reference cell object (yaff/pes/ext.pyx:68-131,
cell.c:37-79): the reciprocal vectors come from the same SVD completion, so
the minimum-image decisions of the device neighbour list match the
reference's bit for bit.  ``System`` keeps the subset of the reference System
(yaff/system.py:50-235) that the force evaluation reads: positions, cell,
charges, radii, masses and the bond graph with its 1-2 .. 1-4 neighbour sets.
"""
import numpy as np

__all__ = ['Cell', 'System', 'SystemView', 'as_system']


class Cell(object):
    """Periodic boundary conditions with 0..3 cell vectors (rows)."""

    def __init__(self, rvecs):
        self.update_rvecs(rvecs)

    def update_rvecs(self, rvecs):
        if rvecs is None or np.asarray(rvecs).size == 0:
            self.nvec = 0
            self._rvecs = np.identity(3)
            self._gvecs = np.identity(3)
        else:
            rvecs = np.ascontiguousarray(rvecs, dtype=np.float64)
            if rvecs.ndim != 2 or rvecs.shape[0] > 3 or rvecs.shape[1] != 3:
                raise TypeError('rvecs must be a C contiguous array with three columns and at most three rows.')
            self.nvec = len(rvecs)
            up, sp, vt = np.linalg.svd(rvecs, full_matrices=True)
            s = np.ones(3, float)
            s[:self.nvec] = sp
            u = np.identity(3, float)
            u[:self.nvec, :self.nvec] = up
            mod = np.dot(u * s, vt)
            mod[:self.nvec] = rvecs
            self._rvecs = np.ascontiguousarray(mod)
            self._gvecs = np.ascontiguousarray(np.dot(u / s, vt))
        g, r = self._gvecs, self._rvecs
        self._rspacings = np.array([1.0 / np.sqrt(g[i, 0] * g[i, 0] + g[i, 1] * g[i, 1] + g[i, 2] * g[i, 2])
                                    for i in range(3)])
        self._gspacings = np.array([1.0 / np.sqrt(r[i, 0] * r[i, 0] + r[i, 1] * r[i, 1] + r[i, 2] * r[i, 2])
                                    for i in range(3)])
        if self.nvec == 3:
            rv = r.ravel()
            self.volume = abs(rv[0] * (rv[4] * rv[8] - rv[5] * rv[7]) + rv[1] * (rv[5] * rv[6] - rv[3] * rv[8]) +
                              rv[2] * (rv[3] * rv[7] - rv[4] * rv[6]))
        elif self.nvec == 2:
            tmp = np.dot(r[0], r[1])
            tmp = np.dot(r[0], r[0]) * np.dot(r[1], r[1]) - tmp * tmp
            self.volume = np.sqrt(tmp) if tmp > 0 else 0.0
        elif self.nvec == 1:
            self.volume = np.sqrt(np.dot(r[0], r[0]))
        else:
            self.volume = 0.0

    @property
    def rvecs(self):
        return self._rvecs[:self.nvec]

    @property
    def gvecs(self):
        return self._gvecs[:self.nvec]

    @property
    def rspacings(self):
        return self._rspacings[:self.nvec]

    @property
    def gspacings(self):
        return self._gspacings[:self.nvec]

    def full_rvecs(self):
        return self._rvecs

    def full_gvecs(self):
        return self._gvecs

    def mic(self, delta):
        """In-place fractional wrap of a relative vector, one cell vector at a
        time (yaff/pes/cell.c:81-106)."""
        for k in range(self.nvec):
            g = self._gvecs[k]
            x = np.ceil(g[0] * delta[0] + g[1] * delta[1] + g[2] * delta[2] - 0.5)
            delta -= x * self._rvecs[k]

    def add_vec(self, delta, r):
        for k in range(self.nvec):
            delta += r[k] * self._rvecs[k]


class System(object):
    """Atoms, cell and topology of a periodic system (atomic units)."""

    def __init__(self, numbers, pos, rvecs=None, charges=None, radii=None, masses=None, bonds=None,
                 ffatypes=None):
        self.numbers = np.asarray(numbers)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
        self.natom = len(self.pos)
        if len(self.numbers) != self.natom:
            raise TypeError('numbers and pos must have the same length')
        self.cell = Cell(rvecs)
        self.charges = None if charges is None else np.ascontiguousarray(charges, dtype=np.float64).copy()
        self.radii = None if radii is None else np.ascontiguousarray(radii, dtype=np.float64).copy()
        self.masses = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64).copy()
        self.ffatypes = ffatypes
        self.bonds = None if bonds is None else np.asarray(bonds, dtype=np.int64).reshape(-1, 2)
        self._device = None
        if self.bonds is not None:
            self._init_derived_bonds()

    def _init_derived_bonds(self):
        """1-2, 1-3, 1-4 and 1-5 neighbour sets by shortest bond path, as in
        yaff/system.py:199-234."""
        n = self.natom
        self.neighs1 = dict((i, set()) for i in range(n))
        for i0, i1 in self.bonds:
            self.neighs1[int(i0)].add(int(i1))
            self.neighs1[int(i1)].add(int(i0))
        self.neighs2 = dict((i, set()) for i in range(n))
        for i0, n0 in self.neighs1.items():
            for i1 in n0:
                for i2 in self.neighs1[i1]:
                    if i2 > i0 and i2 not in self.neighs1[i0]:
                        self.neighs2[i0].add(i2)
                        self.neighs2[i2].add(i0)
        self.neighs3 = dict((i, set()) for i in range(n))
        for i0, n0 in self.neighs1.items():
            for i1 in n0:
                for i3 in self.neighs2[i1]:
                    if i3 != i0 and i3 not in self.neighs1[i0] and i3 not in self.neighs2[i0]:
                        self.neighs3[i0].add(i3)
                        self.neighs3[i3].add(i0)
        self.neighs4 = dict((i, set()) for i in range(n))
        for i0, n0 in self.neighs1.items():
            for i1 in n0:
                for i4 in self.neighs3[i1]:
                    if (i4 != i0 and i4 not in self.neighs1[i0] and i4 not in self.neighs2[i0]
                            and i4 not in self.neighs3[i0]):
                        self.neighs4[i0].add(i4)
                        self.neighs4[i4].add(i0)


class _ViewCell(Cell):
    """The cell of a SystemView: follows the other program's cell object,
    and passes cell changes made through this package on to it."""

    def __init__(self, other):
        self._other = other
        self._src = np.array(other.rvecs, dtype=np.float64)
        Cell.update_rvecs(self, self._src)

    def refresh(self):
        rv = np.asarray(self._other.rvecs, dtype=np.float64)
        if rv.shape != self._src.shape or not np.array_equal(rv, self._src):
            self._src = rv.copy()
            Cell.update_rvecs(self, self._src)

    def update_rvecs(self, rvecs):
        if hasattr(self, '_other') and hasattr(self._other, 'update_rvecs'):
            self._other.update_rvecs(rvecs)
        self._src = np.array(rvecs, dtype=np.float64)
        Cell.update_rvecs(self, self._src)


class SystemView(System):
    """This package's view of another program's System object -- for
    instance the reference's own yaff.system.System (yaff/system.py:50-235)
    -- so that the device parts and neighbour list can be built on it.

    What the force evaluation reads is taken from the other object when it
    is read: the positions (``pos`` is the other object's array; setting it
    sets theirs, so the device path's page-locked position buffer becomes the
    array the other program's ForceField.update_pos writes into), the cell
    (re-derived whenever the other cell's rvecs change, with the same SVD
    completion as the reference Cell), charges, radii and masses.  Bonds and
    the 1-2 .. 1-4 neighbour sets are taken once (they are fixed for a
    System, as in the reference)."""

    def __init__(self, other):
        self._other = other
        natom = getattr(other, 'natom', None)
        self.natom = int(natom) if natom is not None else len(other.pos)
        numbers = getattr(other, 'numbers', None)
        self.numbers = np.zeros(self.natom, int) if numbers is None else np.asarray(numbers)
        self._cell = None
        self.ffatypes = getattr(other, 'ffatypes', None)
        bonds = getattr(other, 'bonds', None)
        self.bonds = None if bonds is None else np.asarray(bonds, dtype=np.int64).reshape(-1, 2)
        self._device = None
        if self.bonds is not None:
            if all(hasattr(other, 'neighs%d' % k) for k in (1, 2, 3)):
                self.neighs1, self.neighs2, self.neighs3 = other.neighs1, other.neighs2, other.neighs3
                self.neighs4 = getattr(other, 'neighs4', None)
                if self.neighs4 is None:
                    self._init_derived_bonds()
            else:
                self._init_derived_bonds()

    @property
    def pos(self):
        return self._other.pos

    @pos.setter
    def pos(self, value):
        self._other.pos = value

    @property
    def cell(self):
        if self._cell is None:
            other_cell = getattr(self._other, 'cell', None)
            self._cell = _ViewCell(other_cell) if other_cell is not None else Cell(None)
        if isinstance(self._cell, _ViewCell):
            self._cell.refresh()
        return self._cell

    @property
    def charges(self):
        q = getattr(self._other, 'charges', None)
        return None if q is None else np.asarray(q, dtype=np.float64)

    @property
    def radii(self):
        r = getattr(self._other, 'radii', None)
        return None if r is None else np.asarray(r, dtype=np.float64)

    @property
    def masses(self):
        m = getattr(self._other, 'masses', None)
        return None if m is None else np.asarray(m, dtype=np.float64)


def as_system(system):
    """`system` when it is this package's System, else the (cached)
    SystemView of the other program's System object: every part, neighbour
    list and scaling table built on the same object shares one view and so
    one device context."""
    if isinstance(system, System):
        return system
    view = getattr(system, '_yaff_gb300_view', None)
    if view is None:
        view = SystemView(system)
        try:
            system._yaff_gb300_view = view
        except AttributeError:
            raise TypeError('cannot attach a device view to %r; pass a yaff_gb300.System' % type(system).__name__)
    return view
