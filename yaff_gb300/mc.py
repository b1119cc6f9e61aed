"""Monte Carlo trial energies on the GPU.

Drop-in forms of the reference's structure-factor functions
(compute_ewald_prefactors / structurefactors / deltae, yaff/pes/ext.pyx:
2727-2900 on ewald.c:441-522) and of ForcePartEwaldReciprocalInteraction
(yaff/pes/ff.py:1060-1255), plus ``MCTrials``: batched trial energies of
rigid-guest insertions, deletions and translations for many chains at once
(the trial path of yaff/sampling/mctrials.py:69-126 with the reference MC's
reci_ei = 'ewald_interaction', mc.py:596-597), with the chains' positions and
structure factors resident in HBM.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr

__all__ = ['compute_ewald_prefactors', 'compute_ewald_structurefactors', 'compute_ewald_deltae',
           'ForcePartEwaldReciprocalInteraction', 'MCTrials', 'INSERT', 'DELETE', 'TRANSLATE']

INSERT, DELETE, TRANSLATE = 0, 1, 2


def _dense_shape(gmax):
    return (2 * int(gmax[0]) + 1, 2 * int(gmax[1]) + 1, int(gmax[2]) + 1)


def compute_ewald_prefactors(unitcell, alpha, gmax, gcut, prefactors):
    """fac1 exp(-k^2/4 alpha^2)/k^2 of the half sphere |k| <= 2 pi gcut into
    prefactors (shape (2gmax0+1, 2gmax1+1, gmax2+1); ext.pyx:2727-2772)."""
    assert unitcell.nvec == 3
    assert alpha > 0
    assert gmax.flags['C_CONTIGUOUS']
    assert gmax.shape[0] == 3
    assert prefactors.flags['C_CONTIGUOUS']
    assert prefactors.shape == _dense_shape(gmax)
    lib = _lib.load()
    g = np.ascontiguousarray(gmax, dtype=np.int64)
    gv = np.ascontiguousarray(unitcell.full_gvecs())
    check(lib.yg_ewald_prefactors(ptr(gv), float(unitcell.volume), float(alpha), ptr(g), float(gcut),
                                  ptr(prefactors)), 'yg_ewald_prefactors')


def compute_ewald_structurefactors(pos, charges, unitcell, alpha, gmax, gcut, cosfacs, sinfacs):
    """ADDS q cos(k.r) and q sin(k.r) of the atoms to cosfacs / sinfacs
    (ext.pyx:2775-2841); evaluated on the GPU in FP64."""
    assert pos.flags['C_CONTIGUOUS']
    assert pos.shape[1] == 3
    assert charges.flags['C_CONTIGUOUS']
    assert charges.shape[0] == pos.shape[0]
    assert unitcell.nvec == 3
    assert alpha > 0
    assert gmax.flags['C_CONTIGUOUS']
    assert gmax.shape[0] == 3
    for a in (cosfacs, sinfacs):
        assert a.flags['C_CONTIGUOUS']
        assert a.shape == _dense_shape(gmax)
    lib = _lib.load()
    g = np.ascontiguousarray(gmax, dtype=np.int64)
    rv = np.ascontiguousarray(unitcell.full_rvecs())
    gv = np.ascontiguousarray(unitcell.full_gvecs())
    p = np.ascontiguousarray(pos, dtype=np.float64)
    q = np.ascontiguousarray(charges, dtype=np.float64)
    check(lib.yg_ewald_structurefactors(ptr(p), len(p), ptr(q), ptr(rv), ptr(gv), float(unitcell.volume), ptr(g),
                                        float(gcut), ptr(cosfacs), ptr(sinfacs), None),
          'yg_ewald_structurefactors')


def compute_ewald_deltae(prefactors, deltacosfacs, cosfacs, deltasinfacs, sinfacs):
    """2 sum prefactors (cosfacs deltacosfacs + sinfacs deltasinfacs)
    (ext.pyx:2844-2900)."""
    assert deltacosfacs.flags['C_CONTIGUOUS']
    for a in (cosfacs, deltasinfacs, sinfacs):
        assert a.flags['C_CONTIGUOUS']
        assert a.shape == deltacosfacs.shape
    nk = deltacosfacs.size
    lib = _lib.load()
    out = ctypes.c_double()
    pf = np.ascontiguousarray(prefactors, dtype=np.float64)
    check(lib.yg_ewald_deltae(ptr(pf), ptr(deltacosfacs), ptr(cosfacs), ptr(deltasinfacs), ptr(sinfacs), nk,
                              ctypes.byref(out)), 'yg_ewald_deltae')
    return out.value


class ForcePartEwaldReciprocalInteraction(object):
    """Reciprocal-space interaction energy between a resident set of atoms
    and atoms added or removed (ff.py:1060-1255): same constructor, cached
    cosfacs/sinfacs arrays and methods; the structure factors and energy
    differences are evaluated on the GPU."""

    def __init__(self, cell, alpha, gcut, pos=None, charges=None, dielectric=1.0):
        self.name = 'ewald_reciprocal_interaction'
        self.energy = 0.0
        self.gpos = np.zeros((0, 3), float)
        self.vtens = np.zeros((3, 3), float)
        if not cell.nvec == 3:
            raise TypeError('The system must have a 3D periodic cell.')
        self.cell = cell
        self.rvecs0 = self.cell.rvecs.copy()
        self.alpha = alpha
        self.gcut = gcut
        self.dielectric = dielectric
        self.initialize()
        if pos is not None:
            assert charges is not None
            self.compute_structurefactors(pos, charges, self.cosfacs, self.sinfacs)

    def update_gmax(self):
        self.gmax = np.ceil(self.gcut / self.cell.gspacings - 0.5).astype(int)

    def initialize(self):
        self.update_gmax()
        self.prefactors = np.zeros(_dense_shape(self.gmax))
        compute_ewald_prefactors(self.cell, self.alpha, np.ascontiguousarray(self.gmax, dtype=np.int64),
                                 self.gcut, self.prefactors)
        self.cosfacs = np.zeros(self.prefactors.shape)
        self.sinfacs = np.zeros(self.prefactors.shape)
        self.rvecs0 = self.cell.rvecs.copy()

    def compute_structurefactors(self, pos, charges, cosfacs, sinfacs):
        if not np.all(self.cell.rvecs == self.rvecs0):
            self.initialize()
        compute_ewald_structurefactors(np.ascontiguousarray(pos, dtype=np.float64),
                                       np.ascontiguousarray(charges, dtype=np.float64), self.cell, self.alpha,
                                       np.ascontiguousarray(self.gmax, dtype=np.int64), self.gcut, cosfacs, sinfacs)

    def compute_deltae(self, cosfacs, sinfacs):
        e = compute_ewald_deltae(self.prefactors, cosfacs, self.cosfacs, sinfacs, self.sinfacs)
        return e / self.dielectric

    def insertion_energy(self, pos, charges, cosfacs=None, sinfacs=None, sign=1):
        assert sign in [-1, 1]
        if cosfacs is None:
            assert sinfacs is None
            cosfacs = np.zeros(self.prefactors.shape)
            sinfacs = np.zeros(self.prefactors.shape)
        else:
            cosfacs[:] = 0.0
            sinfacs[:] = 0.0
        self.compute_structurefactors(pos, charges, cosfacs, sinfacs)
        if sign == -1:
            self.cosfacs[:] -= cosfacs
            self.sinfacs[:] -= sinfacs
        return sign * self.compute_deltae(cosfacs, sinfacs)

    def compute(self, gpos=None, vtens=None):
        return 0.0


class MCTrials(object):
    """Batched MC trial energies of one rigid framework and many chains.

    framework / guest: dicts with 'pos' (framework only), 'charges',
    'sigmas', 'epsilons' (LJ, Lorentz-Berthelot mixing); cell: a Cell;
    rcut, alpha, gcut, dielectric as in the reference's generator
    (alpha = 3.5/rcut, gcut = 1.1 alpha); close_contact: the reference MC's
    close-contact distance (default 0.4 A; negative: off).  ``trials``
    returns U(after) - U(before) per trial against the chains' current
    states; ``apply`` accepts trials of the last batch.
    """

    def __init__(self, framework, guest, cell, rcut, alpha, gcut, nchain, max_guests, dielectric=1.0,
                 close_contact=None, precision='mixed', stream=None):
        from .units import angstrom
        _lib.require_cuda()
        self.lib = _lib.load()
        self.cell = cell
        self.M = len(guest['charges'])
        self.nchain = int(nchain)
        self.max_guests = int(max_guests)
        cc = 0.4 * angstrom if close_contact is None else float(close_contact)
        rmax = np.ascontiguousarray(np.ceil(rcut / cell.rspacings - 0.5).astype(np.int64))
        self.gmax = np.ascontiguousarray(np.ceil(gcut / cell.gspacings - 0.5).astype(np.int64))
        rv = np.ascontiguousarray(cell.full_rvecs())
        gv = np.ascontiguousarray(cell.full_gvecs())
        f = {k: np.ascontiguousarray(framework[k], dtype=np.float64) for k in ('pos', 'charges', 'sigmas', 'epsilons')}
        g = {k: np.ascontiguousarray(guest[k], dtype=np.float64) for k in ('charges', 'sigmas', 'epsilons')}
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = ctypes.c_void_p()
        check(self.lib.yg_mc_create(ptr(rv), ptr(gv), float(cell.volume), ptr(rmax), float(rcut), float(alpha),
                                    float(gcut), ptr(self.gmax), float(dielectric), cc, len(f['pos']),
                                    ptr(f['pos']), ptr(f['charges']), ptr(f['sigmas']), ptr(f['epsilons']), self.M,
                                    ptr(g['charges']), ptr(g['sigmas']), ptr(g['epsilons']), self.nchain,
                                    self.max_guests, prec, None if stream is None else ctypes.c_void_p(stream),
                                    ctypes.byref(h)), 'yg_mc_create')
        self.handle = h

    def __del__(self):
        self.destroy()

    def destroy(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            self.lib.yg_mc_destroy(h)
        self.handle = None

    def set_precision(self, precision):
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        check(self.lib.yg_mc_set_precision(self.handle, prec), 'yg_mc_set_precision')

    def set_chain(self, chain, guest_pos):
        gp = np.ascontiguousarray(guest_pos, dtype=np.float64).reshape(-1, self.M, 3)
        check(self.lib.yg_mc_set_chain(self.handle, int(chain), len(gp), ptr(gp) if len(gp) else None),
              'yg_mc_set_chain')

    def get_chain(self, chain):
        """(guest positions, cosfacs, sinfacs) of a chain; the structure
        factors in the reference's dense layout."""
        n = ctypes.c_int64()
        check(self.lib.yg_mc_get_chain(self.handle, int(chain), ctypes.byref(n), None, None, None), 'yg_mc_get_chain')
        pos = np.zeros((max(n.value, 1), self.M, 3))
        cos = np.zeros(_dense_shape(self.gmax))
        sin = np.zeros(_dense_shape(self.gmax))
        check(self.lib.yg_mc_get_chain(self.handle, int(chain), ctypes.byref(n), ptr(pos), ptr(cos), ptr(sin)),
              'yg_mc_get_chain')
        return pos[:n.value], cos, sin

    def prefactors(self):
        out = np.zeros(_dense_shape(self.gmax))
        n = ctypes.c_int64()
        check(self.lib.yg_mc_prefactors(self.handle, ptr(out), ctypes.byref(n)), 'yg_mc_prefactors')
        return out

    def trials(self, chain, kind, guest, newpos):
        chain = np.ascontiguousarray(chain, dtype=np.int32)
        kind = np.ascontiguousarray(kind, dtype=np.int32)
        guest = np.ascontiguousarray(guest, dtype=np.int32)
        newpos = np.ascontiguousarray(newpos, dtype=np.float64).reshape(len(chain), self.M, 3)
        out = np.zeros(len(chain))
        check(self.lib.yg_mc_trials(self.handle, len(chain), ptr(chain), ptr(kind), ptr(guest), ptr(newpos),
                                    ptr(out)), 'yg_mc_trials')
        return out

    def apply(self, trial_index):
        idx = np.ascontiguousarray(trial_index, dtype=np.int32)
        check(self.lib.yg_mc_apply(self.handle, len(idx), ptr(idx)), 'yg_mc_apply')

    def launch_count(self):
        return int(self.lib.yg_mc_launch_count(self.handle))
