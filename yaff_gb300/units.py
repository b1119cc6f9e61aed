"""Unit constants (atomic units: bohr, hartree, electron charge, a.u. time).

yaff works internally in atomic units and takes its unit constants from
``molmod.units``.  molmod is not a dependency of this package, so the values
below are this package's own harness constants (CODATA 2010 inputs).  They are
used on both sides of every parity check, so parity never depends on them.
"""
import math

# base SI quantities of the atomic unit system (CODATA 2010)
_BOHR_M = 0.52917721092e-10
_HARTREE_J = 4.35974434e-18
_AUTIME_S = 2.418884326505e-17
_ELECTRON_MASS_KG = 9.10938291e-31
_AVOGADRO = 6.02214129e23
_KB_J_PER_K = 1.3806488e-23
_AMU_KG = 1.660538921e-27

meter = 1.0 / _BOHR_M
angstrom = 1e-10 * meter
nanometer = 1e-9 * meter
bohr = 1.0

joule = 1.0 / _HARTREE_J
kjmol = 1e3 * joule / _AVOGADRO
kcalmol = 4.184 * kjmol
electronvolt = 1.602176565e-19 * joule
hartree = 1.0

second = 1.0 / _AUTIME_S
femtosecond = 1e-15 * second
picosecond = 1e-12 * second
nanosecond = 1e-9 * second

kilogram = 1.0 / _ELECTRON_MASS_KG
amu = _AMU_KG * kilogram

kelvin = 1.0
boltzmann = _KB_J_PER_K * joule          # hartree per kelvin

deg = math.pi / 180.0
rad = 1.0

pascal = joule / meter**3
bar = 1e5 * pascal
atm = 101325.0 * pascal

__all__ = [
    'meter', 'angstrom', 'nanometer', 'bohr', 'joule', 'kjmol', 'kcalmol',
    'electronvolt', 'hartree', 'second', 'femtosecond', 'picosecond',
    'nanosecond', 'kilogram', 'amu', 'kelvin', 'boltzmann', 'deg', 'rad',
    'pascal', 'bar', 'atm',
]
