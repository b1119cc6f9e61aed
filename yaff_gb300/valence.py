"""Valence tables: relative vectors, internal coordinates and energy terms.

Host-side table construction with the reference's deduplication rules
(yaff/pes/dlist.py:78-118 add_delta, iclist.py:91-120 add_ic, vlist.py:90-110
add_term); the forward and back passes run on the GPU (yg_valence_compute).
Every internal-coordinate kind of yaff/pes/iclist.py:231-530 (kinds 0-17)
and every energy-term kind of yaff/pes/vlist.py:179-700 (kinds 0-15) is
supported, with the same constructor arguments, the same relative vectors
per coordinate and the same parameter slots.
"""
import numpy as np
from .system import as_system

__all__ = ['DeltaList', 'InternalCoordinateList', 'ValenceList', 'InternalCoordinate', 'Bond', 'BendCos',
           'BendAngle', 'DihedCos', 'DihedAngle', 'UreyBradley', 'OopCos', 'OopMeanCos', 'OopAngle',
           'OopMeanAngle', 'OopDist', 'SqOopDist', 'DihedCos2', 'DihedCos3', 'DihedCos4', 'DihedCos6',
           'PointLineDistance', 'SqPointLineDistance', 'IC_CLASSES',
           'ValenceTerm', 'Harmonic', 'PolyFour', 'Fues', 'Cross', 'Cosine', 'Chebychev1', 'Chebychev2',
           'Chebychev3', 'Chebychev4', 'Chebychev6', 'PolySix', 'MM3Quartic', 'MM3Bend', 'BondDoubleWell',
           'Morse', 'Poly4', 'TERM_CLASSES']


class DeltaList(object):
    def __init__(self, system):
        system = as_system(system)
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
    """An internal coordinate of kind `kind` over the relative vectors
    `index_pairs` (i -> j each)."""
    kind = None

    def __init__(self, index_pairs):
        self.index_pairs = index_pairs
        self.iclist = None


class Bond(InternalCoordinate):
    """Bond length i-j (kind 0)."""
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


class DihedCos(InternalCoordinate):
    """Cosine of the dihedral angle i-j-k-l (kind 3)."""
    kind = 3

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class DihedAngle(InternalCoordinate):
    """Signed dihedral angle i-j-k-l in (-pi, pi] (kind 4)."""
    kind = 4

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class UreyBradley(InternalCoordinate):
    """Distance i-k of the angle i-j-k (kind 5)."""
    kind = 5

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(i, k)])


class OopCos(InternalCoordinate):
    """Cosine of the angle between l->k and the plane of l->i, l->j (kind 6)."""
    kind = 6

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, l), (j, l), (k, l)])


class OopMeanCos(InternalCoordinate):
    """Mean of the three out-of-plane cosines of l's neighbours i, j, k
    (kind 7)."""
    kind = 7

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, l), (j, l), (k, l)])


class OopAngle(InternalCoordinate):
    """Out-of-plane angle of l->k against the plane of l->i, l->j (kind 8)."""
    kind = 8

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, l), (j, l), (k, l)])


class OopMeanAngle(InternalCoordinate):
    """Mean of the three out-of-plane angles (kind 9)."""
    kind = 9

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, l), (j, l), (k, l)])


class OopDist(InternalCoordinate):
    """Signed distance of l from the plane of i, j, k (kind 10)."""
    kind = 10

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, j), (j, k), (k, l)])


class SqOopDist(InternalCoordinate):
    """Squared distance of l from the plane of i, j, k (kind 11)."""
    kind = 11

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(i, j), (j, k), (k, l)])


class DihedCos2(InternalCoordinate):
    """cos(2 phi) of the dihedral i-j-k-l (kind 12)."""
    kind = 12

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class DihedCos3(InternalCoordinate):
    """cos(3 phi) of the dihedral i-j-k-l (kind 13)."""
    kind = 13

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class DihedCos4(InternalCoordinate):
    """cos(4 phi) of the dihedral i-j-k-l (kind 14)."""
    kind = 14

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class DihedCos6(InternalCoordinate):
    """cos(6 phi) of the dihedral i-j-k-l (kind 15)."""
    kind = 15

    def __init__(self, i, j, k, l):
        InternalCoordinate.__init__(self, [(j, i), (j, k), (k, l)])


class PointLineDistance(InternalCoordinate):
    """Distance of k from the line through i and j (kind 16)."""
    kind = 16

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(i, k), (j, k), (i, j)])


class SqPointLineDistance(InternalCoordinate):
    """Squared distance of k from the line through i and j (kind 17)."""
    kind = 17

    def __init__(self, i, j, k):
        InternalCoordinate.__init__(self, [(i, k), (j, k), (i, j)])


IC_CLASSES = {c.kind: c for c in (Bond, BendCos, BendAngle, DihedCos, DihedAngle, UreyBradley, OopCos,
                                  OopMeanCos, OopAngle, OopMeanAngle, OopDist, SqOopDist, DihedCos2,
                                  DihedCos3, DihedCos4, DihedCos6, PointLineDistance, SqPointLineDistance)}


class ValenceTerm(object):
    """An energy term of kind `kind`: up to six parameters (unused slots hold
    -1, as in the reference's table) over one or two internal coordinates."""
    kind = None

    def __init__(self, pars, ics):
        if len(pars) > 6 or not 1 <= len(ics) <= 2:
            raise ValueError('a valence term takes at most six parameters and one or two coordinates')
        self.pars = list(pars)
        self.ics = ics


class Harmonic(ValenceTerm):
    """0.5 K (q - q0)^2 (kind 0)."""
    kind = 0

    def __init__(self, fc, rv, ic):
        ValenceTerm.__init__(self, [fc, rv], [ic])


class PolyFour(ValenceTerm):
    """a0 q + a1 q^2 + a2 q^3 + a3 q^4 (kind 1); fewer than four
    coefficients are padded with zeros."""
    kind = 1

    def __init__(self, pars, ic):
        pars = list(pars)
        if len(pars) > 4:
            raise ValueError('PolyFour term can have maximum 4 parameters, received %i' % len(pars))
        pars += [0.0] * (4 - len(pars))
        ValenceTerm.__init__(self, pars, [ic])


class Fues(ValenceTerm):
    """0.5 K r0^2 (1 + r0/q (r0/q - 2)) (kind 2)."""
    kind = 2

    def __init__(self, fc, rv, ic):
        ValenceTerm.__init__(self, [fc, rv], [ic])


class Cross(ValenceTerm):
    """K (q0 - r0)(q1 - r1) (kind 3)."""
    kind = 3

    def __init__(self, fc, rv0, rv1, ic0, ic1):
        ValenceTerm.__init__(self, [fc, rv0, rv1], [ic0, ic1])


class Cosine(ValenceTerm):
    """0.5 A (1 - cos(m (q - phi0))) (kind 4)."""
    kind = 4

    def __init__(self, m, a, phi0, ic):
        ValenceTerm.__init__(self, [m, a, phi0], [ic])


class _Chebychev(ValenceTerm):
    def __init__(self, A, ic, sign=-1):
        ValenceTerm.__init__(self, [A, sign], [ic])


class Chebychev1(_Chebychev):
    """0.5 A (1 + sign T1(q)) (kind 5)."""
    kind = 5


class Chebychev2(_Chebychev):
    """0.5 A (1 + sign T2(q)) (kind 6)."""
    kind = 6


class Chebychev3(_Chebychev):
    """0.5 A (1 + sign T3(q)) (kind 7)."""
    kind = 7


class Chebychev4(_Chebychev):
    """0.5 A (1 + sign T4(q)) (kind 8)."""
    kind = 8


class Chebychev6(_Chebychev):
    """0.5 A (1 + sign T6(q)) (kind 9)."""
    kind = 9


class PolySix(ValenceTerm):
    """sum_{n=1..6} a_{n-1} q^n (kind 10)."""
    kind = 10

    def __init__(self, pars, ic):
        pars = list(pars)
        if len(pars) > 6:
            raise ValueError('PolySix term can have maximum 6 parameters, received %i' % len(pars))
        pars += [0.0] * (6 - len(pars))
        ValenceTerm.__init__(self, pars, [ic])


class MM3Quartic(ValenceTerm):
    """MM3 quartic bond stretch (kind 11)."""
    kind = 11

    def __init__(self, fc, rv, ic):
        ValenceTerm.__init__(self, [fc, rv], [ic])


class MM3Bend(ValenceTerm):
    """MM3 sextic angle bend (kind 12)."""
    kind = 12

    def __init__(self, fc, rv, ic):
        ValenceTerm.__init__(self, [fc, rv], [ic])


class BondDoubleWell(ValenceTerm):
    """K/(2 (r1 - r2)^4) (q - r1)^2 (q - r2)^4 (kind 13)."""
    kind = 13

    def __init__(self, K, r1, r2, ic):
        ValenceTerm.__init__(self, [K, r1, r2], [ic])


class Morse(ValenceTerm):
    """E0 (exp(-2 k (q - r0)) - 2 exp(-k (q - r0))) (kind 14)."""
    kind = 14

    def __init__(self, E0, k, r1, ic):
        ValenceTerm.__init__(self, [E0, k, r1], [ic])


class Poly4(ValenceTerm):
    """c0 + c1 x + c2 x^2 + c3 x^3 + c4 x^4, x = q - q0 (kind 15)."""
    kind = 15

    def __init__(self, c0, c1, c2, c3, c4, rv, ic):
        ValenceTerm.__init__(self, [c0, c1, c2, c3, c4, rv], [ic])


TERM_CLASSES = {c.kind: c for c in (Harmonic, PolyFour, Fues, Cross, Cosine, Chebychev1, Chebychev2, Chebychev3,
                                    Chebychev4, Chebychev6, PolySix, MM3Quartic, MM3Bend, BondDoubleWell, Morse,
                                    Poly4)}


class ValenceList(object):
    def __init__(self, iclist):
        self.iclist = iclist
        self.terms = []      # (kind, [6 pars], [ic0, ic1])
        self.version = 0

    @property
    def nv(self):
        return len(self.terms)

    def add_term(self, term):
        if term.kind not in TERM_CLASSES:
            raise ValueError('unknown valence term kind %r' % (term.kind,))
        for ic in term.ics:
            if ic.kind not in IC_CLASSES:
                raise ValueError('unknown internal-coordinate kind %r' % (ic.kind,))
        pars = [float(p) for p in term.pars] + [-1.0] * (6 - len(term.pars))
        ic_rows = [self.iclist.add_ic(ic) for ic in term.ics] + [-1] * (2 - len(term.ics))
        self.terms.append((term.kind, pars, ic_rows))
        self.version += 1

    def arrays(self):
        """Device tables: delta (i, j) pairs, coordinate rows (kind, delta
        row and sign x 4), term kinds, term parameters (6 per term) and term
        coordinates (2 per term, -1 when unused)."""
        dl = self.iclist.dlist
        delta_ij = np.array(dl.pairs, dtype=np.int64).reshape(-1, 2)
        ic_rows = np.array(self.iclist.rows, dtype=np.int64).reshape(-1, 9)
        kinds = np.array([t[0] for t in self.terms], dtype=np.int64)
        pars = np.array([t[1] for t in self.terms], dtype=np.float64).reshape(-1, 6)
        vic = np.array([t[2] for t in self.terms], dtype=np.int64).reshape(-1, 2)
        return delta_ij, ic_rows, kinds, pars, vic


def terms_from_rows(rows, ic_classes=None, term_classes=None):
    """Valence terms from the packed rows of a workload description: per term
    [term kind, par0..par5, ic kind, 4 atoms, ic kind, 4 atoms] (-1 where
    unused).  Parameters beyond a term's own count are ignored.  The class
    tables (kind -> class) default to this module's; any classes with the
    same constructor arguments can be given instead."""
    IC_CLASSES_ = IC_CLASSES if ic_classes is None else ic_classes
    TERM_CLASSES_ = TERM_CLASSES if term_classes is None else term_classes
    npars = {0: 2, 1: 4, 2: 2, 3: 3, 4: 3, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 6, 11: 2, 12: 2, 13: 3, 14: 3, 15: 6}
    natoms = {0: 2, 1: 3, 2: 3, 3: 4, 4: 4, 5: 3, 16: 3, 17: 3}
    out = []
    for r in np.asarray(rows, float):
        kind = int(r[0])
        ics = []
        for c in (7, 12):
            ick = int(r[c])
            if ick < 0:
                continue
            atoms = [int(x) for x in r[c + 1:c + 1 + natoms.get(ick, 4)]]
            ics.append(IC_CLASSES_[ick](*atoms))
        pars = list(r[1:1 + npars[kind]])
        cls = TERM_CLASSES_[kind]
        if kind in (1, 10):
            term = cls(pars, ics[0])
        elif kind == 3:
            term = cls(pars[0], pars[1], pars[2], ics[0], ics[1])
        elif 5 <= kind <= 9:
            term = cls(pars[0], ics[0], pars[1])
        else:
            term = cls(*(pars + ics))
        out.append(term)
    return out
