"""Pair potentials and truncation schemes (parameter holders).

Same constructors, names and attributes as the reference's extension classes
(yaff/pes/ext.pyx:524-620 Hammer/Switch3, :747-819 PairPotLJ, :822-908
PairPotMM3, :1770-1857 PairPotEI).  The evaluation itself happens on the GPU
through ForcePartPair; ``compute`` on a rows array is not offered (the device
list never leaves the GPU in the hot path).
"""
import numpy as np

from . import _lib

__all__ = ['Truncation', 'Hammer', 'Switch3', 'PairPot', 'PairPotLJ', 'PairPotMM3', 'PairPotEI']


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
