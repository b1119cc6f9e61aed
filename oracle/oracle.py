"""CPU oracle for the force-evaluation path (ctypes front end of yaff_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
and the CPU-baseline leg of bench.py.  The product never imports it.

``OracleForceField(spec)`` evaluates a configs.py spec the way the reference
``ForceField.compute`` does (yaff/pes/ff.py:117-168, :268-273): a neighbour
list update with the reference's skin policy (yaff/pes/nlist.py:144-218), then
each part in turn -- pair terms (pair_pot.c), Ewald reciprocal / correction /
neutralizing (ewald.c, ff.py:653-669) and the valence chain (dlist/iclist/
vlist).  All arithmetic is FP64 in the order of the reference C code.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'yaff_oracle.c')
SRC_MT = os.path.join(HERE, 'yaff_oracle_mt.c')
BUILD_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD_DIR, 'libyaff_oracle.so')
LIB_MT = os.path.join(BUILD_DIR, 'libyaff_oracle_mt.so')

neigh_dtype = np.dtype([('a', 'i8'), ('b', 'i8'), ('d', 'f8'), ('dx', 'f8'), ('dy', 'f8'),
                        ('dz', 'f8'), ('r0', 'i8'), ('r1', 'i8'), ('r2', 'i8')])
scaling_dtype = np.dtype([('a', 'i8'), ('b', 'i8'), ('scale', 'f8'), ('nbond', 'i8')])
delta_dtype = np.dtype([('dx', 'f8'), ('dy', 'f8'), ('dz', 'f8'), ('i', 'i8'), ('j', 'i8'),
                        ('gx', 'f8'), ('gy', 'f8'), ('gz', 'f8')])
iclist_dtype = np.dtype([('kind', 'i8'), ('i0', 'i8'), ('sign0', 'i8'), ('i1', 'i8'),
                         ('sign1', 'i8'), ('i2', 'i8'), ('sign2', 'i8'), ('i3', 'i8'),
                         ('sign3', 'i8'), ('value', 'f8'), ('grad', 'f8')])
vlist_dtype = np.dtype([('kind', 'i8'), ('par0', 'f8'), ('par1', 'f8'), ('par2', 'f8'),
                        ('par3', 'f8'), ('par4', 'f8'), ('par5', 'f8'), ('ic0', 'i8'),
                        ('ic1', 'i8'), ('energy', 'f8')])

_lib = None


def build():
    """Compile yaff_oracle.c and its threaded timing form yaff_oracle_mt.c
    (gcc, no FMA contraction) if stale."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(SRC_MT))
    for out, src, extra in ((LIB, SRC, []), (LIB_MT, SRC_MT, ['-pthread'])):
        if os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        tmp = out + '.%d.tmp' % os.getpid()
        subprocess.check_call(['gcc', '-O2', '-ffp-contract=off', '-fPIC', '-shared'] + extra +
                              ['-o', tmp, src, '-lm'])
        os.replace(tmp, out)
    return LIB


_lib_mt = None


def lib_mt():
    """The threaded whole-evaluation entry points (yaff_oracle_mt.c)."""
    global _lib_mt
    if _lib_mt is None:
        build()
        L = ctypes.CDLL(LIB_MT)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        D = ctypes.c_double
        INT = ctypes.c_int
        L.orc_mt_nlist_build.restype = I64
        L.orc_mt_nlist_build.argtypes = [P, I64, D, P, P, P, INT, I64, I64, P, I64, I64, INT]
        L.orc_mt_pair_compute.restype = D
        L.orc_mt_pair_compute.argtypes = [P, I64, P, I64, INT, P, P, P, P, P, D, D, D, INT, D, P, P, I64, INT]
        L.orc_mt_ewald_reci.restype = D
        L.orc_mt_ewald_reci.argtypes = [P, I64, I64, I64, P, P, P, D, D, P, D, D, P, P, INT]
        _lib_mt = L
    return _lib_mt


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        D = ctypes.c_double
        INT = ctypes.c_int
        L.orc_nlist_build.restype = I64
        L.orc_nlist_build.argtypes = [P, I64, D, P, P, P, INT, I64, I64, P, I64]
        L.orc_nlist_recompute.restype = None
        L.orc_nlist_recompute.argtypes = [P, P, P, P, INT, P, I64]
        L.orc_pair_compute.restype = D
        L.orc_pair_compute.argtypes = [P, I64, P, I64, INT, P, P, P, P, P, D, D, D, INT, D, P, P]
        L.orc_pair_compute_table.restype = D
        L.orc_pair_compute_table.argtypes = [P, I64, P, I64, INT, P, I64, P, P, P, I64, P, D, INT, D, P, P]
        L.orc_ewald_reci.restype = D
        L.orc_ewald_reci.argtypes = [P, I64, I64, I64, P, P, P, D, D, P, D, D, P, P, P]
        L.orc_ewald_corr.restype = D
        L.orc_ewald_corr.argtypes = [P, P, P, P, INT, D, P, I64, D, P, P, I64, I64, I64]
        L.orc_ewald_prefactors.restype = None
        L.orc_ewald_prefactors.argtypes = [P, D, D, P, D, P]
        L.orc_ewald_structurefactors.restype = None
        L.orc_ewald_structurefactors.argtypes = [P, I64, P, P, P, D, P, P]
        L.orc_ewald_deltae.restype = D
        L.orc_ewald_deltae.argtypes = [P, P, P, P, P, I64]
        L.orc_dlist_forward.restype = None
        L.orc_dlist_forward.argtypes = [P, P, P, INT, P, I64]
        L.orc_dlist_back.restype = None
        L.orc_dlist_back.argtypes = [P, P, P, I64]
        L.orc_iclist_forward.restype = INT
        L.orc_iclist_forward.argtypes = [P, P, I64]
        L.orc_iclist_back.restype = INT
        L.orc_iclist_back.argtypes = [P, P, I64]
        L.orc_vlist_forward.restype = D
        L.orc_vlist_forward.argtypes = [P, P, I64]
        L.orc_vlist_back.restype = None
        L.orc_vlist_back.argtypes = [P, P, I64]
        L.orc_mic_vec.restype = None
        L.orc_mic_vec.argtypes = [P, P, P, INT]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleCell(object):
    """Cell vectors, reciprocal vectors, spacings and volume computed the way
    the reference Cell does (yaff/pes/ext.pyx:103-131, cell.c:37-79)."""

    def __init__(self, rvecs):
        rvecs = np.asarray(rvecs, dtype=np.float64)
        if rvecs.size == 0:
            self.nvec = 0
            self.rvecs = np.identity(3)
            self.gvecs = np.identity(3)
        else:
            self.nvec = len(rvecs)
            up, sp, vt = np.linalg.svd(rvecs, full_matrices=True)
            s = np.ones(3)
            s[:self.nvec] = sp
            u = np.identity(3)
            u[:self.nvec, :self.nvec] = up
            mod = np.dot(u * s, vt)
            mod[:self.nvec] = rvecs
            self.rvecs = np.ascontiguousarray(mod)
            self.gvecs = np.ascontiguousarray(np.dot(u / s, vt))
        g = self.gvecs
        r = self.rvecs
        self.rspacings = np.array([1.0 / np.sqrt(g[i, 0] * g[i, 0] + g[i, 1] * g[i, 1] + g[i, 2] * g[i, 2])
                                   for i in range(3)])
        self.gspacings = np.array([1.0 / np.sqrt(r[i, 0] * r[i, 0] + r[i, 1] * r[i, 1] + r[i, 2] * r[i, 2])
                                   for i in range(3)])
        if self.nvec == 3:
            rv = r.ravel()
            self.volume = abs(rv[0] * (rv[4] * rv[8] - rv[5] * rv[7]) +
                              rv[1] * (rv[5] * rv[6] - rv[3] * rv[8]) +
                              rv[2] * (rv[3] * rv[7] - rv[4] * rv[6]))
        else:
            self.volume = 0.0

    def mic(self, delta):
        d = np.ascontiguousarray(delta, dtype=np.float64).copy()
        lib().orc_mic_vec(_p(d), _p(self.rvecs), _p(self.gvecs), self.nvec)
        return d


def build_scalings(natom, bonds, scalings):
    """Sorted exclusion table (a > b, scale, nbond) from the bond graph, as
    the reference Scalings builds it (yaff/pes/scaling.py:58-105)."""
    s1, s2, s3, s4 = scalings
    if bonds is None or len(bonds) == 0:
        return np.zeros(0, scaling_dtype)
    n1 = [set() for _ in range(natom)]
    for i, j in bonds:
        n1[int(i)].add(int(j))
        n1[int(j)].add(int(i))
    # graph distances up to 4 bonds
    shells = []
    for i0 in range(natom):
        dist = {i0: 0}
        front = [i0]
        for depth in range(1, 5):
            nxt = []
            for a in front:
                for b in n1[a]:
                    if b not in dist:
                        dist[b] = depth
                        nxt.append(b)
            front = nxt
        shells.append(dist)
    rows = []
    for i0 in range(natom):
        for i1, depth in shells[i0].items():
            if i1 >= i0 or depth == 0:
                continue
            sc = (None, s1, s2, s3, s4)[depth]
            if sc < 1.0:
                rows.append((i0, i1, sc, depth))
    rows.sort()
    return np.array(rows, dtype=scaling_dtype)


# Pair-potential kinds of the oracle (yaff/pes/pair_pot.c).
PAIR_KINDS = {'lj': 0, 'mm3': 1, 'ei': 2, 'mm3cap': 3, 'grimme': 4, 'exprep': 5, 'qmdffrep': 6, 'ljcross': 7,
              'dampdisp': 8, 'disp68bjdamp': 9}


def type_pair_tables(pdef):
    """Type-pair tables of a table potential after the mixing rules that the
    reference's constructors apply to unset (zero) entries:
    yaff/pes/ext.pyx:1146-1172 (ExpRep/QMDFFRep amplitude and decay),
    :1560-1573 (DampDisp), :1690-1694 (Disp68BJDamp R from C8/C6)."""
    kind = pdef['kind']
    f = lambda k: np.array(pdef[k], dtype=np.float64)   # noqa: E731
    if kind in ('exprep', 'qmdffrep'):
        A, B = f('amp_cross'), f('b_cross')
        n = len(A)
        amps = pdef.get('amps')
        if amps is not None:
            amps = np.asarray(amps, float)
            mix, x = int(pdef['amp_mix']), float(pdef['amp_mix_coeff'])
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if A[i0, i1] == 0.0:
                        if mix == 0:
                            A[i0, i1] = np.sqrt(amps[i0] * amps[i1])
                        elif amps[i0] != 0.0 and amps[i1] != 0.0:
                            a = (np.log(amps[i0]) + np.log(amps[i1])) / 2
                            a *= 1 - x * abs(np.log(amps[i0] / amps[i1]))
                            A[i0, i1] = np.exp(a)
                        A[i1, i0] = A[i0, i1]
        bs = pdef.get('bs')
        if bs is not None:
            bs = np.asarray(bs, float)
            mix, x = int(pdef['b_mix']), float(pdef['b_mix_coeff'])
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if B[i0, i1] == 0.0:
                        if mix == 0:
                            B[i0, i1] = (bs[i0] + bs[i1]) / 2
                        elif amps[i0] != 0.0 and amps[i1] != 0.0:
                            b = (bs[i0] + bs[i1]) / 2
                            b *= 1 - x * abs(np.log(amps[i0] / amps[i1]))
                            B[i0, i1] = b
                        B[i1, i0] = B[i0, i1]
        return A, B
    if kind == 'ljcross':
        return f('eps_cross'), f('sig_cross')
    if kind == 'dampdisp':
        C, B = f('cn_cross'), f('b_cross')
        n = len(C)
        if pdef.get('cns') is not None:
            cns, vols = np.asarray(pdef['cns'], float), np.asarray(pdef['vols'], float)
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if C[i0, i1] == 0.0 and vols[i0] != 0.0 and vols[i1] != 0.0:
                        ratio = vols[i0] / vols[i1]
                        C[i0, i1] = 2.0 * cns[i0] * cns[i1] / (cns[i0] / ratio + cns[i1] * ratio)
                        C[i1, i0] = C[i0, i1]
        if pdef.get('bs') is not None:
            bs = np.asarray(pdef['bs'], float)
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if B[i0, i1] == 0.0 and bs[i0] != 0.0 and bs[i1] != 0.0:
                        B[i0, i1] = 0.5 * (bs[i0] + bs[i1])
                        B[i1, i0] = B[i0, i1]
        return C, B
    if kind == 'disp68bjdamp':
        c6, c8, R = f('c6_cross'), f('c8_cross'), f('R_cross')
        if np.all(R == 0.0):
            m = c6 != 0.0
            R[m] = np.sqrt(c8[m] / c6[m])
        return c6, c8, R
    raise ValueError(kind)


# Relative vectors (i -> j) each internal-coordinate kind reads, from its
# atoms; yaff/pes/iclist.py:231-530.
IC_DELTAS = {
    0: lambda i, j: [(i, j)],
    1: lambda i, j, k: [(j, i), (j, k)],
    2: lambda i, j, k: [(j, i), (j, k)],
    3: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    4: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    5: lambda i, j, k: [(i, k)],
    6: lambda i, j, k, l: [(i, l), (j, l), (k, l)],
    7: lambda i, j, k, l: [(i, l), (j, l), (k, l)],
    8: lambda i, j, k, l: [(i, l), (j, l), (k, l)],
    9: lambda i, j, k, l: [(i, l), (j, l), (k, l)],
    10: lambda i, j, k, l: [(i, j), (j, k), (k, l)],
    11: lambda i, j, k, l: [(i, j), (j, k), (k, l)],
    12: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    13: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    14: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    15: lambda i, j, k, l: [(j, i), (j, k), (k, l)],
    16: lambda i, j, k: [(i, k), (j, k), (i, j)],
    17: lambda i, j, k: [(i, k), (j, k), (i, j)],
}

# Parameters each energy-term kind stores; yaff/pes/vlist.py:179-700.
TERM_NPARS = {0: 2, 1: 4, 2: 2, 3: 3, 4: 3, 5: 2, 6: 2, 7: 2, 8: 2, 9: 2, 10: 6, 11: 2, 12: 2, 13: 3, 14: 3, 15: 6}


class OracleForceField(object):
    """Reference-order FP64 evaluation of a configs.py spec on the CPU.

    threads > 1 runs the neighbour-list build, the point-charge / per-atom
    pair terms and the Ewald reciprocal sum on that many host threads
    (yaff_oracle_mt.c: the same list, sums in a different order); used to
    time whole evaluations of benchmark-sized systems."""

    def __init__(self, spec, threads=1):
        self.spec = spec
        self.threads = int(threads)
        self.natom = len(spec['pos'])
        self.pos = np.ascontiguousarray(spec['pos'], dtype=np.float64).copy()
        self.cell = OracleCell(spec['rvecs'])
        self.nlow = spec.get('nlow', 0)
        nh = spec.get('nhigh', -1)
        self.nhigh = self.natom if nh == -1 else nh
        self.rcut = spec['rcut']
        self.skin = spec['skin']
        self.stab = build_scalings(self.natom, spec.get('bonds'), spec['scalings'])
        self.neighs = np.zeros(16, neigh_dtype)
        self.nneigh = 0
        self.pos_old = None
        self.rebuild_next = True
        self.update_rmax()
        self._setup_valence()
        self.part_energies = {}
        self.part_gpos = {}
        self.part_vtens = {}

    # -- neighbour list (yaff/pes/nlist.py:119-218) --
    def update_rmax(self):
        if self.cell.nvec > 0:
            self.rmax = np.ceil((self.rcut + self.skin) / self.cell.rspacings[:self.cell.nvec] - 0.5).astype(np.int64)
        else:
            self.rmax = np.zeros(0, np.int64)
        self.rebuild_next = True
        if self.spec.get('ewald') is not None:
            self.gmax = np.ceil(self.spec['ewald']['gcut'] / self.cell.gspacings - 0.5).astype(np.int64)

    def need_rebuild(self):
        if self.skin <= 0 or self.pos_old is None or self.rebuild_next:
            return True
        disp = np.sqrt(((self.pos - self.pos_old) ** 2).sum(axis=1).max())
        disp *= 2 * (self.rmax.max() + 1)
        return disp >= self.skin

    def update_nlist(self):
        L = lib()
        if self.need_rebuild():
            rmax3 = np.zeros(3, np.int64)
            rmax3[:len(self.rmax)] = self.rmax
            if self.threads > 1 and len(self.neighs) <= 16 and self.cell.nvec == 3:
                # first threaded build: size the list from the number density
                # (half the atoms within rcut + skin, 10 % margin) instead of
                # letting a whole build run into a 16-row buffer first
                rc = self.rcut + self.skin
                est = 0.55 * self.natom * self.natom / self.cell.volume * 4.0 / 3.0 * np.pi * rc ** 3
                self.neighs = np.zeros(int(est) + 1024, neigh_dtype)
            while True:
                if self.threads > 1:
                    n = lib_mt().orc_mt_nlist_build(_p(self.pos), self.natom, self.rcut + self.skin, _p(rmax3),
                                                    _p(self.cell.rvecs), _p(self.cell.gvecs), self.cell.nvec,
                                                    self.nlow, self.nhigh, _p(self.neighs), len(self.neighs),
                                                    max(self.nneigh, 16 * self.natom), self.threads)
                    if n < 0:
                        raise MemoryError('threaded neighbour-list build: out of memory')
                else:
                    n = L.orc_nlist_build(_p(self.pos), self.natom, self.rcut + self.skin, _p(rmax3),
                                          _p(self.cell.rvecs), _p(self.cell.gvecs), self.cell.nvec,
                                          self.nlow, self.nhigh, _p(self.neighs), len(self.neighs))
                if n <= len(self.neighs):
                    break
                self.neighs = np.zeros(int(n * 1.1) + 16, neigh_dtype)
            self.nneigh = int(n)
            if self.skin > 0:
                self.pos_old = self.pos.copy()
            self.rebuild_next = False
            return True
        L.orc_nlist_recompute(_p(self.pos), _p(self.pos_old), _p(self.cell.rvecs),
                              _p(self.cell.gvecs), self.cell.nvec, _p(self.neighs), self.nneigh)
        return False

    def pair_set(self):
        """Sorted (a, b, r0, r1, r2) rows of the current list (int64 array)."""
        nb = self.neighs[:self.nneigh]
        keys = np.stack([nb['a'], nb['b'], nb['r0'], nb['r1'], nb['r2']], 1)
        order = np.lexsort(keys.T[::-1])
        return keys[order], nb[order]

    # -- valence layers (yaff/pes/dlist.py, iclist.py, vlist.py) --
    def _setup_valence(self):
        spec = self.spec
        bt = spec.get('bond_terms')
        at = spec.get('bend_terms')
        vr = spec.get('valence')
        self.has_valence = any(x is not None and len(x) for x in (bt, at, vr))
        if not self.has_valence:
            return
        deltas = []
        lookup = {}

        def add_delta(i, j):
            row = lookup.get((i, j))
            if row is not None:
                return row, 1
            row = lookup.get((j, i))
            if row is not None:
                return row, -1
            lookup[(i, j)] = len(deltas)
            deltas.append((i, j))
            return len(deltas) - 1, 1

        ics = []
        iclook = {}

        def add_ic(kind, pairs):
            rs = [add_delta(i, j) for i, j in pairs]
            key = (kind,) + sum(rs, ())
            row = iclook.get(key)
            if row is None:
                row = len(ics)
                iclook[key] = row
                rec = [kind, -1, 0, -1, 0, -1, 0, -1, 0]
                for k, (r, s) in enumerate(rs):
                    rec[1 + 2 * k] = r
                    rec[2 + 2 * k] = s
                ics.append(rec)
            return row

        terms = []   # (term kind, pars, ic0, ic1)
        for i, j, K, r0 in (bt if bt is not None else []):
            terms.append((0, [K, r0], add_ic(0, [(int(i), int(j))]), -1))
        for i, j, k, K, t0 in (at if at is not None else []):
            terms.append((0, [K, t0], add_ic(2, [(int(j), int(i)), (int(j), int(k))]), -1))
        for row in (vr if vr is not None else []):
            kind = int(row[0])
            term_ics = []
            for c in (7, 12):
                if row[c] >= 0:
                    ick = int(row[c])
                    atoms = [int(x) for x in row[c + 1:c + 5] if x >= 0]
                    term_ics.append(add_ic(ick, IC_DELTAS[ick](*atoms)))
            pars = list(row[1:1 + TERM_NPARS[kind]])
            if kind in (1, 10):   # PolyFour / PolySix pad their coefficients with zeros
                pars += [0.0] * ((4 if kind == 1 else 6) - len(pars))
            terms.append((kind, pars, term_ics[0], term_ics[1] if len(term_ics) > 1 else -1))
        self.dl = np.zeros(len(deltas), delta_dtype)
        for r, (i, j) in enumerate(deltas):
            self.dl[r]['i'] = i
            self.dl[r]['j'] = j
        self.ic = np.zeros(len(ics), iclist_dtype)
        for r, rec in enumerate(ics):
            self.ic[r] = tuple(rec) + (np.nan, np.nan)
        self.vt = np.zeros(len(terms), vlist_dtype)
        for r, (kind, pars, ic0, ic1) in enumerate(terms):
            p = [float(x) for x in pars] + [-1.0] * (6 - len(pars))
            self.vt[r] = (kind, p[0], p[1], p[2], p[3], p[4], p[5], ic0, ic1, np.nan)

    def compute_valence(self, gpos, vtens):
        L = lib()
        c = self.cell
        L.orc_dlist_forward(_p(self.pos), _p(c.rvecs), _p(c.gvecs), c.nvec, _p(self.dl), len(self.dl))
        assert L.orc_iclist_forward(_p(self.dl), _p(self.ic), len(self.ic)) == 0
        e = L.orc_vlist_forward(_p(self.ic), _p(self.vt), len(self.vt))
        if gpos is not None or vtens is not None:
            L.orc_vlist_back(_p(self.ic), _p(self.vt), len(self.vt))
            assert L.orc_iclist_back(_p(self.dl), _p(self.ic), len(self.ic)) == 0
            L.orc_dlist_back(_p(gpos), _p(vtens), _p(self.dl), len(self.dl))
        return e

    # -- parts --
    def part_names(self):
        names = ['pair_%s' % p['kind'] for p in self.spec['pair']]
        if self.spec.get('ewald') is not None and self.cell.nvec == 3:
            names += ['ewald_reci', 'ewald_cor', 'ewald_neut']
        if self.has_valence:
            names.append('valence')
        return names

    def _pair(self, pdef, gpos, vtens):
        spec = self.spec
        kind = PAIR_KINDS[pdef['kind']]
        tr = spec.get('tr')
        if pdef['kind'] == 'ei':
            tr = None if not pdef.get('smooth', False) else tr
        trk, trp = 0, 0.0
        if tr is not None:
            trk = {'hammer': 1, 'switch3': 2}[tr[0]]
            trp = tr[1]
        if kind >= 5:
            tabs = type_pair_tables(pdef)
            types = np.ascontiguousarray(pdef['ffatype_ids'], dtype=np.int64)
            scales = None
            if pdef['kind'] == 'disp68bjdamp':
                scales = np.array([float(pdef.get(k, d)) for k, d in
                                   (('c6_scale', 1.0), ('c8_scale', 1.0), ('bj_a', 0.0), ('bj_b', 0.0))])
            return lib().orc_pair_compute_table(
                _p(self.neighs), self.nneigh, _p(self.stab), len(self.stab), kind, _p(types), len(tabs[0]),
                _p(tabs[0]), _p(tabs[1]), _p(tabs[2] if len(tabs) > 2 else None),
                int(pdef.get('power', 6)), _p(scales), self.rcut, trk, trp, _p(gpos), _p(vtens))
        sig = pdef.get('r0') if kind == 4 else pdef.get('sigmas')
        eps = pdef.get('c6') if kind == 4 else pdef.get('epsilons')
        op = pdef.get('onlypaulis')
        q = spec['charges']
        radii = pdef.get('radii')
        if kind == 2 and radii is None:
            radii = np.zeros(self.natom)
        ew = spec.get('ewald')
        alpha = ew['alpha'] if (ew is not None and self.cell.nvec == 3) else 0.0
        keep = [np.ascontiguousarray(x) if x is not None else None for x in (sig, eps, op, q, radii)]
        if keep[2] is not None:
            keep[2] = keep[2].astype(np.int32)
        if self.threads > 1:
            return lib_mt().orc_mt_pair_compute(
                _p(self.neighs), self.nneigh, _p(self.stab), len(self.stab), kind,
                _p(keep[0]), _p(keep[1]), _p(keep[2]), _p(keep[3]), _p(keep[4]),
                alpha, spec.get('dielectric', 1.0), self.rcut, trk, trp, _p(gpos), _p(vtens), self.natom,
                self.threads)
        return lib().orc_pair_compute(
            _p(self.neighs), self.nneigh, _p(self.stab), len(self.stab), kind,
            _p(keep[0]), _p(keep[1]), _p(keep[2]), _p(keep[3]), _p(keep[4]),
            alpha, spec.get('dielectric', 1.0), self.rcut, trk, trp, _p(gpos), _p(vtens))

    def compute(self, gpos=None, vtens=None):
        """Total energy; gpos and vtens (if given) are ADDED to, like the
        reference ForcePart.compute.  Per-part results are kept in
        part_energies / part_gpos / part_vtens."""
        spec = self.spec
        self.update_nlist()
        L = lib()
        total = 0.0
        for name in self.part_names():
            g = np.zeros((self.natom, 3)) if gpos is not None else None
            v = np.zeros((3, 3)) if vtens is not None else None
            if name.startswith('pair_'):
                pdef = [p for p in spec['pair'] if 'pair_' + p['kind'] == name][0]
                e = self._pair(pdef, g, v)
            elif name == 'ewald_reci':
                ew = spec['ewald']
                work = np.zeros(2 * self.natom) if g is not None else None
                if self.threads > 1:
                    e = lib_mt().orc_mt_ewald_reci(
                        _p(self.pos), self.natom, self.nlow, self.nhigh, _p(np.ascontiguousarray(spec['charges'])),
                        _p(self.cell.rvecs), _p(self.cell.gvecs), self.cell.volume, ew['alpha'], _p(self.gmax),
                        ew['gcut'], spec.get('dielectric', 1.0), _p(g), _p(v), self.threads)
                else:
                    e = L.orc_ewald_reci(_p(self.pos), self.natom, self.nlow, self.nhigh,
                                         _p(np.ascontiguousarray(spec['charges'])), _p(self.cell.rvecs),
                                         _p(self.cell.gvecs), self.cell.volume, ew['alpha'], _p(self.gmax),
                                         ew['gcut'], spec.get('dielectric', 1.0), _p(g), _p(work), _p(v))
            elif name == 'ewald_cor':
                ew = spec['ewald']
                e = L.orc_ewald_corr(_p(self.pos), _p(np.ascontiguousarray(spec['charges'])),
                                     _p(self.cell.rvecs), _p(self.cell.gvecs), self.cell.nvec,
                                     ew['alpha'], _p(self.stab), len(self.stab),
                                     spec.get('dielectric', 1.0), _p(g), _p(v), self.natom,
                                     self.nlow, self.nhigh)
            elif name == 'ewald_neut':
                e = self._neut(v)
            elif name == 'valence':
                e = self.compute_valence(g, v)
            else:
                raise AssertionError(name)
            if np.isnan(e):
                raise ValueError('The energy is not-a-number (nan).')
            self.part_energies[name] = e
            self.part_gpos[name] = g
            self.part_vtens[name] = v
            if gpos is not None:
                gpos += g
            if vtens is not None:
                vtens += v
            total += e
        return total

    def _neut(self, vtens):
        """Neutralizing background, yaff/pes/ff.py:633-669 (point charges)."""
        q = self.spec['charges']
        alpha = self.spec['ewald']['alpha']
        fac = q[:].sum() ** 2 / alpha ** 2
        fac -= q[:self.nlow].sum() ** 2 / alpha ** 2
        fac -= q[self.nhigh:].sum() ** 2 / alpha ** 2
        pref = fac * np.pi / (2.0 * self.spec.get('dielectric', 1.0))
        fac = pref / self.cell.volume
        if vtens is not None:
            vtens.ravel()[::4] -= fac
        return fac

    def update_rvecs(self, rvecs):
        """New cell: rmax and gmax follow, the next list is a full rebuild
        (yaff/pes/ff.py:97-103, nlist.py:102-110, ff.py:381-386)."""
        self.cell = OracleCell(rvecs)
        self.update_rmax()

    def update_pos(self, pos):
        self.pos[:] = pos
