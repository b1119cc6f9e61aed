"""Valence tables: relative vectors, internal coordinates and energy terms.

Host-side table construction with the reference's deduplication rules
(yaff/pes/dlist.py:78-118 add_delta, iclist.py:91-120 add_ic, vlist.py:90-110
add_term); the forward and back passes run on the GPU (yg_valence_compute).
Supported on the device: internal coordinates Bond (kind 0), BendCos (1),
BendAngle (2) and UreyBradley (5); energy term Harmonic (kind 0).
"""
import numpy as np

__all__ = ['DeltaList', 'InternalCoordinateList', 'ValenceList', 'InternalCoordinate', 'Bond', 'BendCos',
           'BendAngle', 'UreyBradley', 'ValenceTerm', 'Harmonic']


class DeltaList(object):
    def __init__(self, system):
        self.system = system
        self.pairs = []
        self.lookup = {}

    @property
    def ndelta(self):
        return len(self.pairs)

    def add_delta(self, i, j):
        """Row and sign of the relative vector i -> j (registered if new)."""
        assert i != j and 0 <= i < self.system.natom and 0 <= j < self.system.natom
        row = self.lookup.get((i, j))
        if row is not None:
            return row, 1
        row = self.lookup.get((j, i))
        if row is not None:
            return row, -1
        row = len(self.pairs)
        self.pairs.append((i, j))
        self.lookup[(i, j)] = row
        return row, 1


class InternalCoordinateList(object):
    def __init__(self, dlist):
        self.dlist = dlist
        self.rows = []       # [kind, i0, s0, i1, s1, i2, s2, i3, s3]
        self.lookup = {}

    @property
    def nic(self):
        return len(self.rows)

    def add_ic(self, ic):
        rows_signs = [self.dlist.add_delta(i, j) for i, j in ic.index_pairs]
        key = (ic.kind,) + sum(rows_signs, ())
        row = self.lookup.get(key)
        if row is None:
            rec = [ic.kind, -1, 0, -1, 0, -1, 0, -1, 0]
            for k, (r, s) in enumerate(rows_signs):
                rec[1 + 2 * k] = r
                rec[2 + 2 * k] = s
            row = len(self.rows)
            self.rows.append(rec)
            self.lookup[key] = row
        ic.iclist = self
        return row


class InternalCoordinate(object):
    kind = None

    def __init__(self, index_pairs):
        self.index_pairs = index_pairs
        self.iclist = None


class Bond(InternalCoordinate):
    """Bond length (kind 0)."""
    kind = 0

    def __init__(self, i, j):
        InternalCoordinate.__init__(self, [(i, j)])


class BendCos(InternalCoordinate):
    """Cosine of the angle i-j-k (kind 1)."""
    kind = 1

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(j, i), (j, k)])


class BendAngle(InternalCoordinate):
    """Angle i-j-k (kind 2)."""
    kind = 2

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(j, i), (j, k)])


class UreyBradley(InternalCoordinate):
    """Distance i-k of the angle i-j-k (kind 5)."""
    kind = 5

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(i, k)])


class ValenceTerm(object):
    kind = None

    def __init__(self, pars, ics):
        self.pars = pars
        self.ics = ics


class Harmonic(ValenceTerm):
    """0.5 K (q - q0)^2 (kind 0)."""
    kind = 0

    def __init__(self, fc, rv, ic):
        ValenceTerm.__init__(self, [fc, rv], [ic])


class ValenceList(object):
    def __init__(self, iclist):
        self.iclist = iclist
        self.terms = []      # (kind, [pars], [ic rows])
        self.version = 0

    @property
    def nv(self):
        return len(self.terms)

    def add_term(self, term):
        if term.kind != 0:
            raise NotImplementedError('only Harmonic valence terms run on the device')
        ic_rows = [self.iclist.add_ic(ic) for ic in term.ics]
        self.terms.append((term.kind, list(term.pars), ic_rows))
        self.version += 1

    def arrays(self):
        dl = self.iclist.dlist
        delta_ij = np.array(dl.pairs, dtype=np.int64).reshape(-1, 2)
        ic_rows = np.array(self.iclist.rows, dtype=np.int64).reshape(-1, 9)
        pars = np.array([t[1][:2] for t in self.terms], dtype=np.float64).reshape(-1, 2)
        vic = np.array([t[2][0] for t in self.terms], dtype=np.int64)
        return delta_ij, ic_rows, pars, vic
