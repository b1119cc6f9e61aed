"""Pair potentials and truncation schemes (parameter holders).

Same constructors, names and attributes as the reference's extension classes
(yaff/pes/ext.pyx:524-620 Hammer/Switch3, :747-819 PairPotLJ, :822-908
PairPotMM3, :911-997 PairPotMM3CAP, :1000-1035 PairPotGrimme, :1038-1194
PairPotExpRep, :1197-1354 PairPotQMDFFRep, :1357-1443 PairPotLJCross,
:1446-1590 PairPotDampDisp, :1593-1767 PairPotDisp68BJDamp, :1770-1857
PairPotEI), including the mixing rules that fill the type-pair tables.  The evaluation itself happens on the GPU
through ForcePartPair; ``compute`` on a rows array is not offered (the device
list never leaves the GPU in the hot path).
"""
import numpy as np

from . import _lib

__all__ = ['Truncation', 'Hammer', 'Switch3', 'PairPot', 'PairPotLJ', 'PairPotMM3', 'PairPotEI', 'PairPotMM3CAP',
           'PairPotGrimme', 'PairPotExpRep', 'PairPotQMDFFRep', 'PairPotLJCross', 'PairPotDampDisp',
           'PairPotDisp68BJDamp']


class Truncation(object):
    kind = _lib.TR_NONE
    par = 0.0

    def trunc_fn(self, d, rcut):
        """(h, dh/dd) at distance d (host evaluation, for checks)."""
        raise NotImplementedError


class Hammer(Truncation):
    """exp(tau/(d - rcut)) below rcut, 0 above (yaff/pes/truncation.c:30-41)."""
    kind = _lib.TR_HAMMER

    def __init__(self, tau):
        self.tau = float(tau)
        self.par = self.tau

    def trunc_fn(self, d, rcut):
        if d < rcut:
            x = d - rcut
            h = np.exp(self.tau / x)
            return h, -h * self.tau / x / x
        return 0.0, 0.0

    def get_log(self):
        return 'hammer %s' % self.tau


class Switch3(Truncation):
    """Cubic switch 3x^2 - 2x^3 over the last `width` before rcut
    (yaff/pes/truncation.c:59-76)."""
    kind = _lib.TR_SWITCH3

    def __init__(self, width):
        self.width = float(width)
        self.par = self.width

    def trunc_fn(self, d, rcut):
        if d < rcut:
            x = rcut - d
            if x > self.width:
                return 1.0, 0.0
            x /= self.width
            return (3 - 2 * x) * x * x, -6 * x * (1 - x) / self.width
        return 0.0, 0.0

    def get_log(self):
        return 'switch3 %s' % self.width


# Gauss-Legendre rule for the switching interval of the tail integrals (the
# integrand r^2 V(r) (1 - S(r)) is smooth there; 48 nodes reach FP64 rounding)
_GL_X, _GL_W = np.polynomial.legendre.leggauss(48)


def _tail_cut(terms, rc):
    """sum over terms of int_rc^inf r^2 V_term(r) dr, in closed form:
    ('pow', A, n): A r^-n; ('exp', A, b): A exp(-b r); ('expr', A, b):
    A exp(-b r) / r.  A and the parameter are arrays over type pairs."""
    out = 0.0
    for form, A, q in terms:
        A = np.asarray(A, float)
        q = np.asarray(q, float)
        if form == 'pow':
            out = out + A * rc ** (3.0 - q) / (q - 3.0)
        else:
            b = np.where(q > 0, q, 1.0)
            e = np.exp(-b * rc)
            if form == 'exp':
                v = A * e * (rc * rc / b + 2.0 * rc / (b * b) + 2.0 / (b * b * b))
            else:
                v = A * e * (rc / b + 1.0 / (b * b))
            out = out + np.where((q > 0) & (A != 0), v, 0.0)
    return out


def _tail_switch(terms, rc, width):
    """sum over terms of int_{rc-w}^{rc} r^2 V(r) (1 - S(r)) dr with the cubic
    switch S = 3x^2 - 2x^3, x = (rc - r)/w (Gauss-Legendre)."""
    r = rc - 0.5 * width * (1.0 - _GL_X)          # nodes on [rc - w, rc]
    x = (rc - r) / width
    f = r * r * (1.0 - (3.0 - 2.0 * x) * x * x) * (0.5 * width * _GL_W)
    out = 0.0
    for form, A, q in terms:
        A = np.asarray(A, float)[..., None]
        q = np.asarray(q, float)[..., None]
        if form == 'pow':
            v = A * r ** (-q)
        elif form == 'exp':
            v = np.where(A != 0, A * np.exp(-q * r), 0.0)
        else:
            v = np.where(A != 0, A * np.exp(-q * r) / r, 0.0)
        out = out + (v * f).sum(-1)
    return out


class PairPot(object):
    name = None
    kind = None

    def __init__(self, rcut, tr):
        if not rcut > 0:
            raise ValueError('rcut must be positive')
        self._rcut = float(rcut)
        self.tr = tr

    @property
    def rcut(self):
        return self._rcut

    def get_truncation(self):
        return self.tr

    def log(self):
        pass

    # -- tail corrections (yaff/pes/ext.pyx:665-687, pair_pot.c:178-254) --
    def _tail_params(self, natom):
        """(natom, k) per-atom parameters that fix the pair terms."""
        raise NotImplementedError('Tail corrections are not defined for %s' % self.name)

    def _tail_terms(self, A, B):
        """Long-range model of the pair potential for parameter rows A, B."""
        raise NotImplementedError

    def _tail_value(self, A, B, r):
        """The untruncated pair potential at distance r."""
        raise NotImplementedError

    def _tail_switch_compat(self, A, B, rc, width):
        """Deviation of the reference's Switch3 tail integral from the exact
        one, where the reference's closed form has one (default: none)."""
        return 0.0

    def prepare_tailcorrections(self, natom, nlow=0, nhigh=-1):
        """(C0, C1) summed over all ordered atom pairs (i, j), i = j included,
        except pairs with both atoms below nlow or both at or above nhigh:
        C0 = sum int r^2 V(r) (1 - h(r)) dr (h the truncation: a step at rcut,
        or Switch3), C1 = -C0 - U(rcut) rcut^3 / 3 without truncation, -C0
        with Switch3.  Atoms are grouped by their parameters, so the cost is
        quadratic in the number of distinct parameter sets only."""
        if nhigh == -1:
            nhigh = natom
        if not (0 <= nlow <= nhigh <= natom):
            raise ValueError('invalid nlow / nhigh')
        if self.tr is not None and not isinstance(self.tr, Switch3):
            raise NotImplementedError('Tail corrections not supported for %s' % self.tr.get_log())
        P = np.asarray(self._tail_params(natom), float).reshape(natom, -1)
        keys, inv = np.unique(P, axis=0, return_inverse=True)
        inv = inv.ravel()
        nkey = len(keys)
        cnt = [np.bincount(inv[lo:hi], minlength=nkey).astype(float)
               for lo, hi in ((0, nlow), (nlow, nhigh), (nhigh, natom))]
        tot = cnt[0] + cnt[1] + cnt[2]
        mult = np.outer(tot, tot) - np.outer(cnt[0], cnt[0]) - np.outer(cnt[2], cnt[2])
        ia, ib = np.nonzero(mult)
        if len(ia) == 0:
            return 0.0, 0.0
        A, B, m = keys[ia], keys[ib], mult[ia, ib]
        terms = self._tail_terms(A, B)
        rc = self.rcut
        c0 = _tail_cut(terms, rc)
        if self.tr is not None:
            c0 = c0 + _tail_switch(terms, rc, self.tr.width) + self._tail_switch_compat(A, B, rc, self.tr.width)
        e = float((m * c0).sum())
        if self.tr is None:
            w = -e - float((m * self._tail_value(A, B, rc)).sum()) * rc ** 3 / 3.0
        else:
            w = -e
        return e, w


class PairPotLJ(PairPot):
    """4 eps_ij ((sigma_ij/d)^12 - (sigma_ij/d)^6), sigma_ij = (sigma_i +
    sigma_j)/2, eps_ij = sqrt(eps_i eps_j)."""
    name = 'lj'
    kind = _lib.POT_LJ

    def __init__(self, sigmas, epsilons, rcut, tr=None):
        PairPot.__init__(self, rcut, tr)
        self.sigmas = np.ascontiguousarray(sigmas, dtype=np.float64)
        self.epsilons = np.ascontiguousarray(epsilons, dtype=np.float64)
        if self.sigmas.shape != self.epsilons.shape:
            raise TypeError('sigmas and epsilons must have the same shape')

    def _device_arrays(self, natom):
        assert len(self.sigmas) == natom
        return {'sigma': self.sigmas, 'epsilon': self.epsilons, 'onlypauli': None, 'radii': None,
                'alpha': 0.0, 'dielectric': 1.0}

    def _tail_params(self, natom):
        return np.stack([self.sigmas, self.epsilons], 1)

    @staticmethod
    def _mix(A, B):
        return 0.5 * (A[:, 0] + B[:, 0]), np.sqrt(A[:, 1] * B[:, 1])

    def _tail_terms(self, A, B):
        sig, eps = self._mix(A, B)
        return [('pow', 4 * eps * sig ** 12, 12.0), ('pow', -4 * eps * sig ** 6, 6.0)]

    def _tail_value(self, A, B, r):
        sig, eps = self._mix(A, B)
        x = (sig / r) ** 6
        return 4.0 * eps * (x * (x - 1.0))


class PairPotMM3(PairPot):
    """eps_ij (1.84e5 exp(-12 d/sigma_ij) - 2.25 (sigma_ij/d)^6) with
    sigma_ij = sigma_i + sigma_j (the reference's MM3 code sums the sigmas,
    yaff/pes/pair_pot.c:325-328) and the only-Pauli switch."""
    name = 'mm3'
    kind = _lib.POT_MM3

    def __init__(self, sigmas, epsilons, onlypaulis, rcut, tr=None):
        PairPot.__init__(self, rcut, tr)
        self.sigmas = np.ascontiguousarray(sigmas, dtype=np.float64)
        self.epsilons = np.ascontiguousarray(epsilons, dtype=np.float64)
        self.onlypaulis = np.ascontiguousarray(onlypaulis, dtype=np.int32)
        if not (self.sigmas.shape == self.epsilons.shape == self.onlypaulis.shape):
            raise TypeError('sigmas, epsilons and onlypaulis must have the same shape')

    def _device_arrays(self, natom):
        assert len(self.sigmas) == natom
        return {'sigma': self.sigmas, 'epsilon': self.epsilons, 'onlypauli': self.onlypaulis, 'radii': None,
                'alpha': 0.0, 'dielectric': 1.0}

    def _tail_params(self, natom):
        return np.stack([self.sigmas, self.epsilons, self.onlypaulis.astype(float)], 1)

    def _tail_terms(self, A, B):
        # the capped form shares MM3's long-range model (pair_pot.c:361-365)
        sig, eps = A[:, 0] + B[:, 0], np.sqrt(A[:, 1] * B[:, 1])
        r6 = np.where(A[:, 2] + B[:, 2] == 0, 1.0, 0.0)
        return [('exp', 1.84e5 * eps, 12.0 / sig), ('pow', -2.25 * r6 * eps * sig ** 6, 6.0)]

    def _tail_value(self, A, B, r):
        sig, eps = A[:, 0] + B[:, 0], np.sqrt(A[:, 1] * B[:, 1])
        ex = 1.84e5 * np.exp(-12.0 * r / sig)
        v = np.where(A[:, 2] + B[:, 2] == 0, eps * (ex - 2.25 * (sig / r) ** 6), eps * ex)
        if self.kind == _lib.POT_MM3CAP:
            x = r / sig
            v = np.where((A[:, 2] + B[:, 2] == 0) & (x <= 0.355114), eps * (5799.303156 - 12182.86986 * x), v)
        return v


class PairPotEI(PairPot):
    """Real-space electrostatics q_i q_j erfc(alpha d)/d / dielectric (point
    charges, or Gaussian charges when radii are given)."""
    name = 'ei'
    kind = _lib.POT_EI

    def __init__(self, charges, alpha, rcut, tr=None, dielectric=1.0, radii=None):
        PairPot.__init__(self, rcut, tr)
        self.charges = np.ascontiguousarray(charges, dtype=np.float64)
        self.alpha = float(alpha)
        self.dielectric = float(dielectric)
        self.radii = np.zeros(self.charges.shape) if radii is None else np.ascontiguousarray(radii, dtype=np.float64)

    def _device_arrays(self, natom):
        assert len(self.charges) == natom
        return {'sigma': None, 'epsilon': None, 'onlypauli': None, 'radii': self.radii,
                'alpha': self.alpha, 'dielectric': self.dielectric}


class PairPotMM3CAP(PairPotMM3):
    """MM3 with the energy capped linearly below d = 0.355114 sigma_ij (for
    Monte Carlo insertions); above the cap identical to MM3."""
    name = 'mm3cap'
    kind = _lib.POT_MM3CAP


class PairPotGrimme(PairPot):
    """-1.1 f(d) c6_ij / d^6 with f = 1/(1 + exp(-20 (d/r0_ij - 1))),
    r0_ij = r0_i + r0_j, c6_ij = sqrt(c6_i c6_j)."""
    name = 'grimme'
    kind = _lib.POT_GRIMME

    def __init__(self, r0, c6, rcut, tr=None):
        PairPot.__init__(self, rcut, tr)
        self.r0 = np.ascontiguousarray(r0, dtype=np.float64)
        self.c6 = np.ascontiguousarray(c6, dtype=np.float64)
        if self.r0.shape != self.c6.shape:
            raise TypeError('r0 and c6 must have the same shape')

    def _device_arrays(self, natom):
        assert len(self.r0) == natom
        return {'sigma': self.r0, 'epsilon': self.c6, 'onlypauli': None, 'radii': None,
                'alpha': 0.0, 'dielectric': 1.0}

    def _tail_params(self, natom):
        return np.stack([self.r0, self.c6], 1)

    def _tail_terms(self, A, B):
        # undamped long-range model -1.1 c6 / r^6 (tailcorr.c:229-256)
        return [('pow', -1.1 * np.sqrt(A[:, 1] * B[:, 1]), 6.0)]

    def _tail_value(self, A, B, r):
        r0, c6 = A[:, 0] + B[:, 0], np.sqrt(A[:, 1] * B[:, 1])
        f = 1.0 / (1.0 + np.exp(-20.0 * (r / r0 - 1.0)))
        return -1.1 * f * c6 / r ** 6


class _TypeTablePot(PairPot):
    """A pair potential whose parameters are tables over pairs of atom types."""
    type_table = True

    def __init__(self, ffatype_ids, rcut, tr):
        PairPot.__init__(self, rcut, tr)
        self.ffatype_ids = np.ascontiguousarray(ffatype_ids, dtype=np.int64)

    @staticmethod
    def _square(a, n=None):
        a = np.array(a, dtype=np.float64, order='C')
        if a.ndim != 2 or a.shape[0] != a.shape[1] or (n is not None and a.shape[0] != n):
            raise TypeError('cross-parameter tables must be square, one row per atom type')
        return a

    def _check_types(self, n):
        if len(self.ffatype_ids) and (self.ffatype_ids.min() < 0 or self.ffatype_ids.max() >= n):
            raise ValueError('atom type index out of range')

    def _tail_params(self, natom):
        return self.ffatype_ids.astype(float)[:, None]

    def _tab(self, A, B, k):
        return self._cross[k][A[:, 0].astype(np.int64), B[:, 0].astype(np.int64)]

    def _device_table(self, natom):
        assert len(self.ffatype_ids) == natom
        return {'ffatype_ids': self.ffatype_ids, 'cross0': self._cross[0], 'cross1': self._cross[1],
                'cross2': self._cross[2] if len(self._cross) > 2 else None, 'power': getattr(self, 'power', 0),
                'scales': getattr(self, '_scales', None)}


class _RepPot(_TypeTablePot):
    def __init__(self, ffatype_ids, amp_cross, b_cross, rcut, tr=None, amps=None, amp_mix=-1, amp_mix_coeff=-1,
                 bs=None, b_mix=-1, b_mix_coeff=-1):
        _TypeTablePot.__init__(self, ffatype_ids, rcut, tr)
        amp_cross = self._square(amp_cross)
        n = amp_cross.shape[0]
        b_cross = self._square(b_cross, n)
        self._check_types(n)
        if amps is not None:
            amps = np.asarray(amps, dtype=np.float64)
            if len(amps) != n or amp_mix not in (0, 1) or not 0 <= amp_mix_coeff <= 1:
                raise ValueError('invalid amplitude mixing arguments')
            self._mix_amp(n, amp_cross, amps, amp_mix, amp_mix_coeff)
        if not (amp_cross == amp_cross.T).all():
            raise ValueError('amp_cross must be symmetric')
        if bs is not None:
            bs = np.asarray(bs, dtype=np.float64)
            if len(bs) != n or b_mix not in (0, 1) or not 0 <= b_mix_coeff <= 1:
                raise ValueError('invalid decay mixing arguments')
            self._mix_b(n, b_cross, bs, b_mix, b_mix_coeff, amps)
        if not (b_cross == b_cross.T).all():
            raise ValueError('b_cross must be symmetric')
        self.amp_cross = amp_cross
        self.b_cross = b_cross
        self._cross = (amp_cross, b_cross)

    @staticmethod
    def _mix_amp(n, amp_cross, amps, amp_mix, coeff):
        # unset (zero) entries: geometric mean (amp_mix 0) or the corrected
        # geometric rule ln A_ij = (ln A_i + ln A_j)/2 (1 - x |ln(A_i/A_j)|)
        for i0 in range(n):
            for i1 in range(i0 + 1):
                if amp_cross[i0, i1] == 0.0:
                    if amp_mix == 0:
                        amp_cross[i0, i1] = np.sqrt(amps[i0] * amps[i1])
                    elif amps[i0] != 0.0 and amps[i1] != 0.0:
                        a = (np.log(amps[i0]) + np.log(amps[i1])) / 2
                        a *= 1 - coeff * abs(np.log(amps[i0] / amps[i1]))
                        amp_cross[i0, i1] = np.exp(a)
                    amp_cross[i1, i0] = amp_cross[i0, i1]

    @staticmethod
    def _mix_b(n, b_cross, bs, b_mix, coeff, amps):
        # unset entries: arithmetic mean (b_mix 0) or the corrected rule
        # B_ij = (B_i + B_j)/2 (1 - x |ln(A_i/A_j)|)
        for i0 in range(n):
            for i1 in range(i0 + 1):
                if b_cross[i0, i1] == 0.0:
                    if b_mix == 0:
                        b_cross[i0, i1] = (bs[i0] + bs[i1]) / 2
                    elif amps[i0] != 0.0 and amps[i1] != 0.0:
                        b = (bs[i0] + bs[i1]) / 2
                        b *= 1 - coeff * abs(np.log(amps[i0] / amps[i1]))
                        b_cross[i0, i1] = b
                    b_cross[i1, i0] = b_cross[i0, i1]


    def _tail_terms(self, A, B):
        amp, b = self._tab(A, B, 0), self._tab(A, B, 1)
        amp = np.where(b == 0.0, 0.0, amp)
        return [('exp' if self.kind == _lib.POT_EXPREP else 'expr', amp, b)]

    def _tail_value(self, A, B, r):
        amp, b = self._tab(A, B, 0), self._tab(A, B, 1)
        ok = (amp != 0.0) & (b != 0.0)
        v = amp * np.exp(-np.where(ok, b, 0.0) * r)
        if self.kind == _lib.POT_QMDFFREP:
            v = v / r
        return np.where(ok, v, 0.0)


class PairPotExpRep(_RepPot):
    """A_ij exp(-B_ij d) over atom-type pairs."""
    name = 'exprep'
    kind = _lib.POT_EXPREP

    def _tail_switch_compat(self, A, B, rc, width):
        # The reference's Switch3 integral truncates rcut^2 to an integer in
        # one of its terms (yaff/pes/tailcorr.c:358); its value differs from
        # the exact one by 6 A exp(-B rc) (floor(rc^2) - rc^2) / (B^3 w^2).
        # Kept so that the energies equal the reference's.
        amp, b = self._tab(A, B, 0), self._tab(A, B, 1)
        ok = b > 0
        bb = np.where(ok, b, 1.0)
        d = 6.0 * amp * np.exp(-bb * rc) * (np.floor(rc * rc) - rc * rc) / (bb ** 3 * width * width)
        return np.where(ok, d, 0.0)


class PairPotQMDFFRep(_RepPot):
    """A_ij exp(-B_ij d) / d over atom-type pairs."""
    name = 'qmdffrep'
    kind = _lib.POT_QMDFFREP


class PairPotLJCross(_TypeTablePot):
    """4 eps_ij ((sig_ij/d)^12 - (sig_ij/d)^6) over atom-type pairs."""
    name = 'ljcross'
    kind = _lib.POT_LJCROSS

    def __init__(self, ffatype_ids, eps_cross, sig_cross, rcut, tr=None):
        _TypeTablePot.__init__(self, ffatype_ids, rcut, tr)
        self.eps_cross = self._square(eps_cross)
        self.sig_cross = self._square(sig_cross, self.eps_cross.shape[0])
        self._check_types(self.eps_cross.shape[0])
        self._cross = (self.eps_cross, self.sig_cross)

    def _tail_terms(self, A, B):
        eps, sig = self._tab(A, B, 0), self._tab(A, B, 1)
        return [('pow', 4 * eps * sig ** 12, 12.0), ('pow', -4 * eps * sig ** 6, 6.0)]

    def _tail_value(self, A, B, r):
        eps, sig = self._tab(A, B, 0), self._tab(A, B, 1)
        x = (sig / r) ** 6
        return 4.0 * eps * (x * (x - 1.0))


class PairPotDampDisp(_TypeTablePot):
    """-C_ij f_n(B_ij d) / d^n with the Tang-Toennies damping f_n (undamped
    where B_ij = 0), over atom-type pairs."""
    name = 'dampdisp'
    kind = _lib.POT_DAMPDISP

    def __init__(self, ffatype_ids, cn_cross, b_cross, rcut, tr=None, cns=None, bs=None, vols=None, power=6):
        _TypeTablePot.__init__(self, ffatype_ids, rcut, tr)
        cn_cross = self._square(cn_cross)
        n = cn_cross.shape[0]
        b_cross = self._square(b_cross, n)
        self._check_types(n)
        if cns is not None or vols is not None:
            if cns is None or vols is None:
                raise ValueError('cns and vols are needed together')
            cns = np.asarray(cns, dtype=np.float64)
            vols = np.asarray(vols, dtype=np.float64)
            # unset entries: 2 C_i C_j / (C_i v_j/v_i + C_j v_i/v_j)
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if cn_cross[i0, i1] == 0.0 and vols[i0] != 0.0 and vols[i1] != 0.0:
                        ratio = vols[i0] / vols[i1]
                        cn_cross[i0, i1] = 2.0 * cns[i0] * cns[i1] / (cns[i0] / ratio + cns[i1] * ratio)
                        cn_cross[i1, i0] = cn_cross[i0, i1]
        if bs is not None:
            bs = np.asarray(bs, dtype=np.float64)
            for i0 in range(n):
                for i1 in range(i0 + 1):
                    if b_cross[i0, i1] == 0.0 and bs[i0] != 0.0 and bs[i1] != 0.0:
                        b_cross[i0, i1] = 0.5 * (bs[i0] + bs[i1])
                        b_cross[i1, i0] = b_cross[i0, i1]
        if not 0 <= int(power) <= 30:
            raise ValueError('power must be in [0, 30]')
        self.power = int(power)
        self.cn_cross = cn_cross
        self.b_cross = b_cross
        self._cross = (cn_cross, b_cross)

    def _tail_terms(self, A, B):
        # undamped long-range model -C / r^n (tailcorr.c:523-553)
        return [('pow', -self._tab(A, B, 0), float(self.power))]

    def _tail_value(self, A, B, r):
        cn, b = self._tab(A, B, 0), self._tab(A, B, 1)
        n = self.power
        disp = -cn / r ** n
        x = b * r
        poly = np.zeros_like(x)
        term = np.ones_like(x)
        for k in range(n + 1):
            if k:
                term = term * x / k
            poly = poly + term
        damp = np.where(b == 0.0, 1.0, 1.0 - poly * np.exp(-x))
        return np.where(cn == 0.0, 0.0, damp * disp)


class PairPotDisp68BJDamp(_TypeTablePot):
    """-s6 C6_ij / (d^6 + R^6) - s8 C8_ij / (d^8 + R^8), R = a R_ij + b
    (Becke-Johnson damping), over atom-type pairs."""
    name = 'disp68bjdamp'
    kind = _lib.POT_DISP68BJ

    def __init__(self, ffatype_ids, c6_cross, c8_cross, R_cross, rcut, tr=None, c6s=None, c8s=None, Rs=None,
                 c6_scale=1.0, c8_scale=1.0, bj_a=0.0, bj_b=0.0):
        _TypeTablePot.__init__(self, ffatype_ids, rcut, tr)
        c6_cross = self._square(c6_cross)
        n = c6_cross.shape[0]
        c8_cross = self._square(c8_cross, n)
        R_cross = self._square(R_cross, n)
        self._check_types(n)
        if c6s is not None or c8s is not None or Rs is not None:
            raise NotImplementedError('per-type c6s / c8s / Rs mixing is not defined for this potential')
        if np.all(R_cross == 0.0):
            mask = c6_cross != 0.0
            R_cross[mask] = np.sqrt(c8_cross[mask] / c6_cross[mask])
        self.c6_cross, self.c8_cross, self.R_cross = c6_cross, c8_cross, R_cross
        self.c6_scale, self.c8_scale, self.bj_a, self.bj_b = float(c6_scale), float(c8_scale), float(bj_a), float(bj_b)
        self._cross = (c6_cross, c8_cross, R_cross)
        self._scales = np.array([self.c6_scale, self.c8_scale, self.bj_a, self.bj_b])

    def _tail_terms(self, A, B):
        # undamped long-range model (tailcorr.c:596-625)
        return [('pow', -self.c6_scale * self._tab(A, B, 0), 6.0), ('pow', -self.c8_scale * self._tab(A, B, 1), 8.0)]

    def _tail_value(self, A, B, r):
        R = self.bj_a * self._tab(A, B, 2) + self.bj_b
        return (-self.c6_scale * self._tab(A, B, 0) / (r ** 6 + R ** 6)
                - self.c8_scale * self._tab(A, B, 1) / (r ** 8 + R ** 8))
