"""Seeded synthetic systems for the force-evaluation workloads.

Every generator returns a *spec*: a plain dict of numpy arrays and scalars in
atomic units that fully describes a system and its force field.  The same spec
builds the GPU force field (``yaff_gb300.build_forcefield``) and, in tests,
the CPU oracle, so both sides always see identical inputs.

Spec keys
---------
name           str
pos            (N, 3) float64, bohr
rvecs          (3, 3) float64 rows = cell vectors (or shape (0, 3))
charges        (N,) float64 or None
masses         (N,) float64 (a.u. of mass)
bonds          (nb, 2) int64 or None
pair           list of dicts: {'kind': 'lj', 'sigmas', 'epsilons'} |
               {'kind': 'mm3' or 'mm3cap', 'sigmas', 'epsilons', 'onlypaulis'} |
               {'kind': 'ei', 'radii' (optional)} | {'kind': 'grimme', 'r0', 'c6'} |
               type-pair tables over 'ffatype_ids': {'kind': 'exprep' or
               'qmdffrep', 'amp_cross', 'b_cross', mixing keys} | {'kind':
               'ljcross', 'eps_cross', 'sig_cross'} | {'kind': 'dampdisp',
               'cn_cross', 'b_cross', 'power', mixing keys} | {'kind':
               'disp68bjdamp', 'c6_cross', 'c8_cross', 'R_cross', 'c6_scale',
               'c8_scale', 'bj_a', 'bj_b'}
rcut, skin     float (bohr)
tr             None | ('switch3', width) | ('hammer', tau)
ewald          None | {'alpha': a, 'gcut': g}      (reciprocal + corr + neut)
dielectric     float
scalings       (scale1, scale2, scale3, scale4)
bond_terms     (nbt, 4): i, j, K, r0      harmonic bonds (Bond + Harmonic)
bend_terms     (nat, 5): i, j, k, K, th0  harmonic bends (BendAngle + Harmonic)
valence        (nv, 17) packed valence terms: term kind, par0..par5, then
               per internal coordinate its kind and 4 atoms (-1 unused)
nlow, nhigh    ints (nhigh = -1 means N)
tailcorr       bool (optional): a tail correction per non-EI pair part
"""
import hashlib
import math
import os

import numpy as np

from .units import angstrom, kjmol, amu, deg

MASS_O = 15.999 * amu
MASS_H = 1.008 * amu
MASS_GENERIC = 12.011 * amu


def triclinic_rvecs(a, b, c, alpha, beta, gamma):
    """Cell vectors (rows) for lengths a, b, c and angles alpha, beta, gamma
    (radians), a along x and b in the xy plane."""
    ca, cb, cg = math.cos(alpha), math.cos(beta), math.cos(gamma)
    sg = math.sin(gamma)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = math.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [cx, cy, cz]])


def ewald_params(rcut, alpha_scale=3.5, gcut_scale=1.1):
    """alpha = alpha_scale / rcut and gcut = gcut_scale * alpha, the rule of the
    reference's force-field generator (yaff/pes/generator.py:210, :229)."""
    alpha = alpha_scale / rcut
    return {'alpha': alpha, 'gcut': gcut_scale * alpha}


def _base_spec(name, pos, rvecs):
    n = len(pos)
    return {
        'name': name, 'pos': np.ascontiguousarray(pos, dtype=np.float64),
        'rvecs': np.ascontiguousarray(rvecs, dtype=np.float64),
        'charges': None, 'masses': np.full(n, MASS_GENERIC), 'bonds': None,
        'pair': [], 'rcut': 0.0, 'skin': 0.0, 'tr': None, 'ewald': None,
        'dielectric': 1.0, 'scalings': (0.0, 0.0, 1.0, 1.0),
        'bond_terms': np.zeros((0, 4)), 'bend_terms': np.zeros((0, 5)),
        'nlow': 0, 'nhigh': -1,
    }


def lattice_lj_ei(nside=10, spacing=2.5, jitter=0.3, rcut=12.0, skin=0.0, seed=0,
                  name=None):
    """Simple-cubic lattice of alternating A/B atoms with LJ + EI + Ewald.

    The 1,000-atom default is the plain FP64 workload: 10x10x10 lattice,
    2.5 A spacing, +-0.3 A uniform jitter (seed 0) in a 25 A cube; A: +0.5 e,
    sigma 3.0 A, eps 0.5 kJ/mol; B: -0.5 e, sigma 3.2 A, eps 0.8 kJ/mol
    (Lorentz-Berthelot via the LJ mixing rule); rcut 12 A, skin 0,
    alpha_scale 3.5, gcut_scale 1.1, no exclusions.
    """
    rng = np.random.default_rng(seed)
    g = np.arange(nside, dtype=float)
    grid = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    pos = (grid * spacing + rng.uniform(-jitter, jitter, grid.shape)) * angstrom
    box = nside * spacing * angstrom
    spec = _base_spec(name or 'lattice%d' % (nside ** 3), pos, np.eye(3) * box)
    n = len(pos)
    isb = (np.arange(n) % 2 == 1)
    spec['charges'] = np.where(isb, -0.5, 0.5)
    sig = np.where(isb, 3.2, 3.0) * angstrom
    eps = np.where(isb, 0.8, 0.5) * kjmol
    spec['pair'] = [{'kind': 'lj', 'sigmas': sig, 'epsilons': eps}, {'kind': 'ei'}]
    spec['rcut'] = rcut * angstrom
    spec['skin'] = skin * angstrom
    spec['ewald'] = ewald_params(spec['rcut'])
    return spec


def _random_rotations(rng, n):
    """n uniformly random rotation matrices (from uniform unit quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def water_geometry():
    """Body-frame coordinates (O, H, H) of the 3-site water: O-H 0.96 A,
    H-O-H 104.5 deg, O at the origin."""
    half = 0.5 * 104.5 * deg
    r = 0.96 * angstrom
    return np.array([[0.0, 0.0, 0.0],
                     [r * math.sin(half), 0.0, r * math.cos(half)],
                     [-r * math.sin(half), 0.0, r * math.cos(half)]])


def flexible_water(nside=20, box=62.1, jitter=0.2, rcut=10.0, skin=1.0, seed=1,
                   name=None):
    """Flexible 3-site water box with LJ (O only) + EI + Ewald + valence.

    The default is the 8,000-molecule (24,000-atom) NVE workload: molecule
    centres on a jittered 20^3 lattice in a 62.1 A cube, seeded uniformly
    random orientations, q(O) -0.82 e, q(H) +0.41 e, LJ on O (sigma 3.166 A,
    eps 0.65 kJ/mol), harmonic bonds K 4000 kJ/mol/A^2, r0 1.0 A, harmonic
    bends K 300 kJ/mol/rad^2, theta0 109.47 deg, 1-2 and 1-3 pairs excluded,
    rcut 10 A, skin 1 A.
    """
    rng = np.random.default_rng(seed)
    spacing = box / nside
    g = np.arange(nside, dtype=float)
    centres = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    centres = (centres * spacing + rng.uniform(-jitter, jitter, centres.shape)) * angstrom
    nmol = len(centres)
    rot = _random_rotations(rng, nmol)
    body = water_geometry()
    pos = (centres[:, None, :] + np.einsum('mij,aj->mai', rot, body)).reshape(-1, 3)
    spec = _base_spec(name or 'water%d' % nmol, pos, np.eye(3) * box * angstrom)
    n = 3 * nmol
    iso = (np.arange(n) % 3 == 0)
    spec['charges'] = np.where(iso, -0.82, 0.41)
    spec['masses'] = np.where(iso, MASS_O, MASS_H)
    sig = np.where(iso, 3.166 * angstrom, 0.0)
    eps = np.where(iso, 0.65 * kjmol, 0.0)
    spec['pair'] = [{'kind': 'lj', 'sigmas': sig, 'epsilons': eps}, {'kind': 'ei'}]
    o = 3 * np.arange(nmol)
    spec['bonds'] = np.stack([np.stack([o, o + 1], 1), np.stack([o, o + 2], 1)], 1).reshape(-1, 2)
    kb = 4000.0 * kjmol / angstrom ** 2
    spec['bond_terms'] = np.column_stack([spec['bonds'].astype(float),
                                          np.full(2 * nmol, kb), np.full(2 * nmol, 1.0 * angstrom)])
    ka = 300.0 * kjmol
    spec['bend_terms'] = np.column_stack([(o + 1).astype(float), o.astype(float), (o + 2).astype(float),
                                          np.full(nmol, ka), np.full(nmol, 109.47 * deg)])
    spec['scalings'] = (0.0, 0.0, 1.0, 1.0)
    spec['rcut'] = rcut * angstrom
    spec['skin'] = skin * angstrom
    spec['ewald'] = ewald_params(spec['rcut'])
    return spec


def _valence_row(term_kind, pars, ic0, ic1=None):
    """One packed valence row: [term kind, par0..par5, ic kind, 4 atoms,
    ic kind, 4 atoms], -1 where unused."""
    row = [float(term_kind)] + [float(p) for p in pars] + [-1.0] * (6 - len(pars))
    for ic in (ic0, ic1):
        if ic is None:
            row += [-1.0] * 5
        else:
            row += [float(ic[0])] + [float(a) for a in ic[1]] + [-1.0] * (4 - len(ic[1]))
    return row


def valence_molecules(nside=2, box=15.0, seed=7, rcut=6.0, skin=0.5, name=None):
    """Periodic box of branched 5-atom molecules carrying every valence kind.

    Molecule a-b-c-d with a branch b-e (bonds 1.45-1.6 A, bends 95-125 deg,
    the dihedral a-b-c-d uniform in (-180, 180] deg so that the cosine and the
    sine branches of the dihedral angle both occur), centres on a jittered
    nside^3 lattice of a mildly triclinic 15 A cell so that molecules straddle
    the cell faces.  Terms: every internal-coordinate kind 0-17 and every
    energy-term kind 0-15 of the reference valence tables, several sharing a
    coordinate; LJ (sigma 3.0 A, eps 0.2 kJ/mol) with 1-2 and 1-3 pairs
    excluded, rcut 6 A, skin 0.5 A.
    """
    rng = np.random.default_rng(seed)
    nmol = nside ** 3
    g = np.arange(nside, dtype=float)
    centres = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    centres = centres * (box / nside) + rng.uniform(-1.0, 1.0, centres.shape)
    rvecs = np.array([[box, 0.0, 0.0], [0.1 * box, box, 0.0], [-0.07 * box, 0.13 * box, box]])
    centres = centres @ (rvecs / box)
    rot = _random_rotations(rng, nmol)
    pos = []
    for m in range(nmol):
        r = rng.uniform(1.45, 1.6, 4)
        th = rng.uniform(95.0, 125.0, 3) * math.pi / 180
        phi = rng.uniform(-math.pi, math.pi, 2)
        b = np.zeros(3)
        c = np.array([r[1], 0.0, 0.0])
        a = r[0] * np.array([math.cos(th[0]), math.sin(th[0]), 0.0])
        # d: bend th[1] at c, dihedral phi[0] about b-c
        u = np.array([-math.cos(th[1]), math.sin(th[1]) * math.cos(phi[0]), math.sin(th[1]) * math.sin(phi[0])])
        d = c + r[2] * u
        # e: bend th[2] at b against c, rotated out of the a-b-c plane
        e = r[3] * np.array([math.cos(th[2]), math.sin(th[2]) * math.cos(phi[1] + math.pi),
                             math.sin(th[2]) * math.sin(phi[1] + math.pi)])
        mol = np.array([a, b, c, d, e])
        mol -= mol.mean(0)
        pos.append(centres[m] + mol @ rot[m].T)
    pos = np.concatenate(pos) * angstrom
    spec = _base_spec(name or 'valence%d' % (5 * nmol), pos, rvecs * angstrom)
    n = len(pos)
    spec['pair'] = [{'kind': 'lj', 'sigmas': np.full(n, 3.0 * angstrom), 'epsilons': np.full(n, 0.2 * kjmol)}]
    spec['rcut'] = rcut * angstrom
    spec['skin'] = skin * angstrom
    spec['scalings'] = (0.0, 0.0, 1.0, 1.0)
    A = angstrom
    kb, kt = 2000 * kjmol / A ** 2, 300 * kjmol
    rows, bonds = [], []
    for m in range(nmol):
        a, b, c, d, e = 5 * m + np.arange(5)
        bonds += [(a, b), (b, c), (c, d), (b, e)]
        B = lambda i, j: (0, (i, j))          # noqa: E731
        rows += [
            _valence_row(0, [kb, 1.5 * A], B(a, b)),                                  # Harmonic
            _valence_row(1, [0.0, kb, -0.3 * kb / A, 0.05 * kb / A ** 2], B(a, b)),   # PolyFour, shared bond
            _valence_row(2, [kb, 1.52 * A], B(b, c)),                                 # Fues
            _valence_row(11, [kb, 1.55 * A], B(c, d)),                                # MM3Quartic
            _valence_row(13, [50 * kjmol, 1.45 * A, 1.65 * A], B(c, d)),              # BondDoubleWell
            _valence_row(14, [400 * kjmol, 2.0 / A, 1.5 * A], B(b, e)),               # Morse
            _valence_row(10, [0.01, 0.02, -0.003, 1e-4, 2e-6, -1e-7], B(b, c)),       # PolySix
            _valence_row(15, [0.1, 0.0, kb, 0.1 * kb / A, 0.01 * kb / A ** 2, 1.5 * A], B(b, e)),  # Poly4
            _valence_row(0, [kt, 110 * deg], (2, (a, b, c))),                         # BendAngle
            _valence_row(12, [kt, 112 * deg], (2, (c, b, e))),                        # MM3Bend
            _valence_row(5, [20 * kjmol, -1.0], (1, (a, b, e))),                      # Chebychev1 on BendCos
            _valence_row(0, [kt, -0.3], (1, (b, c, d))),                              # BendCos
            _valence_row(0, [kb, 2.5 * A], (5, (a, b, c))),                           # UreyBradley
            _valence_row(3, [0.3 * kb, 1.5 * A, 110 * deg], B(a, b), (2, (a, b, c))),  # Cross
            _valence_row(3, [-0.2 * kb, 1.5 * A, 1.52 * A], B(a, b), B(b, c)),        # Cross of two bonds
            _valence_row(4, [3, 10 * kjmol, 15 * deg], (4, (a, b, c, d))),            # Cosine on DihedAngle
            _valence_row(0, [5 * kjmol, 60 * deg], (4, (e, b, c, d))),                # Harmonic on DihedAngle
            _valence_row(6, [8 * kjmol, -1.0], (3, (a, b, c, d))),                    # Chebychev2 on DihedCos
            _valence_row(7, [6 * kjmol, 1.0], (3, (a, b, c, d))),                     # Chebychev3
            _valence_row(8, [4 * kjmol, -1.0], (3, (e, b, c, d))),                    # Chebychev4
            _valence_row(9, [2 * kjmol, 1.0], (3, (e, b, c, d))),                     # Chebychev6
            _valence_row(0, [3 * kjmol, 0.2], (12, (a, b, c, d))),                    # DihedCos2
            _valence_row(0, [3 * kjmol, -0.1], (13, (a, b, c, d))),                   # DihedCos3
            _valence_row(0, [3 * kjmol, 0.3], (14, (e, b, c, d))),                    # DihedCos4
            _valence_row(0, [3 * kjmol, -0.4], (15, (e, b, c, d))),                   # DihedCos6
            _valence_row(0, [40 * kjmol, 0.7], (6, (a, c, e, b))),                    # OopCos
            _valence_row(0, [40 * kjmol, 0.8], (7, (a, c, e, b))),                    # OopMeanCos
            _valence_row(0, [40 * kjmol, 30 * deg], (8, (a, c, e, b))),               # OopAngle
            _valence_row(0, [40 * kjmol, 25 * deg], (9, (a, c, e, b))),               # OopMeanAngle
            _valence_row(0, [kb, 0.2 * A], (10, (a, c, e, b))),                       # OopDist
            _valence_row(1, [0.0, kb, 0.0, 0.0], (11, (a, c, e, b))),                 # PolyFour on SqOopDist
            _valence_row(0, [kb, 0.8 * A], (16, (a, c, b))),                          # PointLineDistance
            _valence_row(0, [kb / A ** 2, 0.5 * A ** 2], (17, (a, c, e))),            # SqPointLineDistance
        ]
    spec['bonds'] = np.array(bonds, dtype=np.int64)
    spec['valence'] = np.array(rows, dtype=np.float64)
    return spec


def pair_potentials(variant='a', natom=300, box=16.0, dmin=1.5, rcut=7.0, skin=0.5, seed=11, name=None):
    """A dense periodic box (triclinic, 16 A edges) with three atom types and
    three pair parts of the potentials beyond LJ / MM3 / EI, in atomic units.

    variant 'a': MM3CAP (minimum separation 1.5 A, so that pairs fall below
      the cap at d = 0.355 sigma_ij; some atoms only-Pauli), Grimme and ExpRep
      with the geometric / arithmetic mixing rules filling unset table
      entries, no truncation;
    variant 'b': QMDFFRep, LJCross, DampDisp (power 6, Tang-Toennies damped,
      one undamped type pair; C6 mixed from per-type C6 and volumes), Switch3
      truncation over 2 A;
    variant 'c': Disp68BJDamp (Becke-Johnson R from C8/C6), DampDisp (power
      8) and ExpRep with the corrected mixing rules, Hammer truncation.
    """
    rng = np.random.default_rng(seed + ord(variant))
    rvecs = triclinic_rvecs(box, box, box, 80 * deg, 85 * deg, 95 * deg) * angstrom
    pos = _rsa_fill(rng, rvecs, natom, dmin * angstrom)
    spec = _base_spec(name or 'pairpot%s%d' % (variant, natom), pos, rvecs)
    types = np.arange(natom) % 3
    A = angstrom
    spec['rcut'] = rcut * A
    spec['skin'] = skin * A
    if variant == 'a':
        sig = np.array([1.9, 1.7, 1.6])[types] * A
        eps = np.array([0.4, 0.25, 0.3])[types] * kjmol
        spec['pair'] = [
            {'kind': 'mm3cap', 'sigmas': sig, 'epsilons': eps, 'onlypaulis': (np.arange(natom) % 7 == 0).astype(np.int32)},
            {'kind': 'grimme', 'r0': np.array([1.5, 1.4, 1.3])[types] * A, 'c6': np.array([20.0, 12.0, 9.0])[types]},
            {'kind': 'exprep', 'ffatype_ids': types.astype(np.int64),
             'amp_cross': np.array([[60.0, 0.0, 0.0], [0.0, 40.0, 35.0], [0.0, 35.0, 30.0]]),
             'b_cross': np.array([[2.1, 0.0, 0.0], [0.0, 2.0, 0.0], [0.0, 0.0, 1.9]]),
             'amps': np.array([60.0, 40.0, 30.0]), 'amp_mix': 0, 'amp_mix_coeff': 0.0,
             'bs': np.array([2.1, 2.0, 1.9]), 'b_mix': 0, 'b_mix_coeff': 0.0},
        ]
    elif variant == 'b':
        spec['tr'] = ('switch3', 2.0 * A)
        spec['pair'] = [
            {'kind': 'qmdffrep', 'ffatype_ids': types.astype(np.int64),
             'amp_cross': np.array([[90.0, 70.0, 60.0], [70.0, 50.0, 45.0], [60.0, 45.0, 40.0]]),
             'b_cross': np.array([[2.2, 2.1, 2.0], [2.1, 2.0, 1.9], [2.0, 1.9, 1.8]])},
            {'kind': 'ljcross', 'ffatype_ids': types.astype(np.int64),
             'eps_cross': np.array([[0.5, 0.3, 0.4], [0.3, 0.2, 0.25], [0.4, 0.25, 0.35]]) * kjmol,
             'sig_cross': np.array([[3.2, 3.0, 3.1], [3.0, 2.8, 2.9], [3.1, 2.9, 3.0]]) * A},
            {'kind': 'dampdisp', 'ffatype_ids': types.astype(np.int64), 'power': 6,
             'cn_cross': np.array([[30.0, 0.0, 20.0], [0.0, 15.0, 12.0], [20.0, 12.0, 10.0]]),
             'b_cross': np.array([[1.8, 1.7, 0.0], [1.7, 1.6, 1.65], [0.0, 1.65, 1.5]]),
             'cns': np.array([30.0, 15.0, 10.0]), 'vols': np.array([1.2, 1.0, 0.9]),
             'bs': np.array([1.8, 1.6, 0.0])},
        ]
    else:
        spec['tr'] = ('hammer', 0.8 * A)
        spec['pair'] = [
            {'kind': 'disp68bjdamp', 'ffatype_ids': types.astype(np.int64),
             'c6_cross': np.array([[30.0, 22.0, 18.0], [22.0, 16.0, 13.0], [18.0, 13.0, 11.0]]),
             'c8_cross': np.array([[900.0, 700.0, 600.0], [700.0, 520.0, 450.0], [600.0, 450.0, 400.0]]),
             'R_cross': np.zeros((3, 3)), 'c6_scale': 1.0, 'c8_scale': 0.8, 'bj_a': 0.45, 'bj_b': 2.5},
            {'kind': 'dampdisp', 'ffatype_ids': types.astype(np.int64), 'power': 8,
             'cn_cross': np.array([[800.0, 600.0, 500.0], [600.0, 450.0, 400.0], [500.0, 400.0, 350.0]]),
             'b_cross': np.array([[1.8, 0.0, 1.7], [0.0, 1.6, 0.0], [1.7, 0.0, 1.5]]),
             'bs': np.array([1.8, 1.6, 1.5])},
            {'kind': 'exprep', 'ffatype_ids': types.astype(np.int64),
             'amp_cross': np.array([[0.0, 0.0, 45.0], [0.0, 0.0, 0.0], [45.0, 0.0, 0.0]]),
             'b_cross': np.zeros((3, 3)),
             'amps': np.array([60.0, 40.0, 30.0]), 'amp_mix': 1, 'amp_mix_coeff': 0.3,
             'bs': np.array([2.1, 2.0, 1.9]), 'b_mix': 1, 'b_mix_coeff': 0.2},
        ]
    return spec


def tail_corrections(variant='a'):
    """Small boxes with a tail correction per non-electrostatic pair part:
    'a' the MM3CAP / Grimme / ExpRep box untruncated (150 atoms, nlow 20,
    nhigh 130), 'b' the QMDFFRep / LJCross / DampDisp(7) box with Switch3, 'c'
    the Disp68BJDamp / DampDisp(8) / ExpRep box with Switch3 instead of
    Hammer, 'lj' the 216-atom LJ + EI lattice untruncated (rcut 6 A), 'mm3'
    a 200-atom triclinic MM3 + EI box with Switch3 (2 A)."""
    if variant in ('a', 'b', 'c'):
        spec = pair_potentials(variant, natom=150, name='tailcorr%s150' % variant)
        if variant == 'a':
            spec['nlow'], spec['nhigh'] = 20, 130
        if variant == 'b':
            # the reference's Switch3 tail integral of DampDisp divides by
            # (power - 6) (tailcorr.c:555-594), NaN at power 6
            spec['pair'][2]['power'] = 7
        if variant == 'c':
            spec['tr'] = ('switch3', 1.5 * angstrom)
    elif variant == 'lj':
        spec = lattice_lj_ei(nside=6, spacing=2.5, rcut=6.0, name='tailcorrlj216')
    else:
        spec = triclinic_mm3_ei(natom=200, rcut=6.0, skin=0.5, name='tailcorrmm3200')
        spec['tr'] = ('switch3', 2.0 * angstrom)
    spec['tailcorr'] = True
    return spec


_CACHE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), '_build', 'cache')


def _cached(kind, key, make):
    """Positions generated by `make`, cached on disk under the package's
    build folder keyed by the generator parameters (the insertion of the
    50,000-atom system takes tens of seconds)."""
    tag = hashlib.sha256(repr((kind, key)).encode()).hexdigest()[:24]
    path = os.path.join(_CACHE_DIR, '%s_%s.npy' % (kind, tag))
    if os.path.exists(path):
        try:
            return np.load(path)
        except (OSError, ValueError):
            pass
    arr = make()
    try:
        os.makedirs(_CACHE_DIR, exist_ok=True)
        tmp = path + '.%d.tmp.npy' % os.getpid()
        np.save(tmp, arr)
        os.replace(tmp, path)
    except OSError:
        pass
    return arr


def _rsa_fill(rng, rvecs, natom, dmin, batch=1024, maxper=8):
    """Random sequential insertion of natom points with minimum image distance
    dmin in the periodic cell rvecs (rows).

    Trial points come in seeded batches.  A trial is rejected when it lies
    within dmin of an accepted point (checked against the 27 surrounding
    cells of a fractional grid whose cells are at least dmin wide) or of an
    earlier trial of the same batch that passed that check; the survivors are
    accepted in order.  Deterministic for a given seed."""
    gvecs = np.linalg.inv(rvecs).T
    spac = 1.0 / np.linalg.norm(gvecs, axis=1)
    ng = np.maximum((spac / dmin).astype(int), 1)
    ncell = int(np.prod(ng))
    cells = -np.ones((ncell, maxper), np.int64)
    counts = np.zeros(ncell, np.int64)
    frac_out = np.zeros((natom + 1, 3))
    dmin2 = dmin * dmin
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    count = 0
    accept = 1.0
    while count < natom:
        # batch size adapts to the acceptance rate (about 1000 survivors each)
        batch = int(min(16384, max(1024, 1000.0 / max(accept, 1e-3))))
        f = rng.random((batch, 3))
        c = (f * ng).astype(np.int64) % ng
        nc = (c[:, None, :] + offs[None, :, :]) % ng
        nid = nc[..., 0] + ng[0] * (nc[..., 1] + ng[1] * nc[..., 2])
        cand = cells[nid]                                   # (B, 27, maxper)
        mask = cand >= 0
        df = frac_out[np.where(mask, cand, natom)] - f[:, None, None, :]
        df -= np.round(df)
        dd = df @ rvecs
        d2 = np.einsum('bcpi,bcpi->bcp', dd, dd)
        keep = ~((mask & (d2 < dmin2)).any(axis=(1, 2)))
        idx = np.nonzero(keep)[0]
        if len(idx) > 1:
            fk = f[idx]
            dk = fk[None, :, :] - fk[:, None, :]
            dk -= np.round(dk)
            dc = dk @ rvecs
            close = np.einsum('ijk,ijk->ij', dc, dc) < dmin2
            close = np.tril(close, -1)                       # i conflicts with an earlier j
            idx = idx[~close.any(axis=1)]
        accept = max(len(idx), 1) / float(batch)
        for t in idx:
            if count >= natom:
                break
            cid = c[t, 0] + ng[0] * (c[t, 1] + ng[1] * c[t, 2])
            if counts[cid] >= maxper:
                continue
            cells[cid, counts[cid]] = count
            counts[cid] += 1
            frac_out[count] = f[t]
            count += 1
    return frac_out[:natom] @ rvecs


def triclinic_mm3_ei(natom=50000, density=50000 / 5.0313e5, angle=75.0, dmin=1.8,
                     rcut=12.0, skin=1.0, seed=2, name=None, a=None):
    """Triclinic exp-6 (MM3) + EI + Ewald system.

    The default is the 50,000-atom precision-sweep workload: a=b=c=82 A,
    alpha=beta=gamma=75 deg, three species (atom i has species i % 3) with
    charges +1.2/-0.6/-0.6 e, MM3 sigma 3.4/3.0/3.0 A, eps 0.3/0.25/0.25
    kJ/mol (the reference's MM3 mixing sums the sigmas), placed by seeded
    random sequential insertion with a 1.8 A minimum separation; rcut 12 A,
    skin 1 A, alpha_scale 3.5, gcut_scale 1.1.  50,000 is not a multiple of
    three, so the 1:1:1 ratio leaves a net charge of +0.6 e, which the
    neutralizing-background part accounts for.  Smaller natom keep the number
    density and shrink the cell.
    """
    rng = np.random.default_rng(seed)
    ang = angle * deg
    if a is None:
        if natom == 50000 and abs(density - 50000 / 5.0313e5) < 1e-12:
            a = 82.0
        else:
            unit = triclinic_rvecs(1.0, 1.0, 1.0, ang, ang, ang)
            a = (natom / density / abs(np.linalg.det(unit))) ** (1.0 / 3.0)
    rvecs = triclinic_rvecs(a, a, a, ang, ang, ang) * angstrom
    pos = _cached('rsa', (natom, a, angle, dmin, seed), lambda: _rsa_fill(rng, rvecs, natom, dmin * angstrom))
    spec = _base_spec(name or 'triclinic%d' % natom, pos, rvecs)
    sp = np.arange(natom) % 3
    spec['charges'] = np.array([1.2, -0.6, -0.6])[sp]
    spec['pair'] = [{'kind': 'mm3', 'sigmas': np.array([3.4, 3.0, 3.0])[sp] * angstrom,
                     'epsilons': np.array([0.3, 0.25, 0.25])[sp] * kjmol,
                     'onlypaulis': np.zeros(natom, np.int32)},
                    {'kind': 'ei'}]
    spec['rcut'] = rcut * angstrom
    spec['skin'] = skin * angstrom
    spec['ewald'] = ewald_params(spec['rcut'])
    return spec


def lattice_1000():
    """1,000-atom LJ + EI + Ewald lattice (plain FP64 parity workload)."""
    return lattice_lj_ei(name='lattice1000')


def water_24000():
    """8,000-molecule (24,000-atom) flexible water NVE workload."""
    return flexible_water(name='water24000')


def triclinic_50000():
    """50,000-atom triclinic MM3 + EI + Ewald workload (the headline)."""
    return triclinic_mm3_ei(name='triclinic50000')


def serving_request(natom, seed, rcut=10.0, density=0.064):
    """One request of the batched-replica serving workload: an LJ + EI +
    Ewald lattice-like system of natom atoms in a cube at 0.064 atoms/A^3
    with rcut 10 A (A/B parameters of the 1,000-atom lattice)."""
    rng = np.random.default_rng(seed)
    box = (natom / density) ** (1.0 / 3.0)
    nside = int(math.ceil(natom ** (1.0 / 3.0)))
    spacing = box / nside
    g = np.arange(nside, dtype=float)
    grid = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    sel = rng.permutation(len(grid))[:natom]
    pos = (grid[np.sort(sel)] + 0.5) * spacing
    pos = (pos + rng.uniform(-0.12, 0.12, pos.shape) * spacing) * angstrom
    spec = _base_spec('request%d_%d' % (natom, seed), pos, np.eye(3) * box * angstrom)
    isb = (np.arange(natom) % 2 == 1)
    spec['charges'] = np.where(isb, -0.5, 0.5)
    if natom % 2 == 1:
        spec['charges'] = spec['charges'].copy()
        spec['charges'][-1] = 0.0
    spec['pair'] = [{'kind': 'lj', 'sigmas': np.where(isb, 3.2, 3.0) * angstrom,
                     'epsilons': np.where(isb, 0.8, 0.5) * kjmol}, {'kind': 'ei'}]
    spec['rcut'] = rcut * angstrom
    spec['ewald'] = ewald_params(spec['rcut'])
    return spec


def natom_of(spec):
    return len(spec['pos'])


def nhigh_of(spec):
    nh = spec.get('nhigh', -1)
    return natom_of(spec) if nh == -1 else nh


def mc_framework(natom=2000, box=30.0, jitter=0.3, seed=4):
    """Rigid framework of the MC trial-energy workload: natom sites of a
    13^3 simple-cubic grid in a 30 A cube (seeded choice, uniform jitter of
    +-0.3 A), charges +-0.4 e alternating (neutral), LJ sigma 3.3 A,
    eps 0.4 kJ/mol."""
    rng = np.random.default_rng(seed)
    nside = int(math.ceil(natom ** (1.0 / 3.0)))
    spacing = box / nside
    g = np.arange(nside, dtype=float)
    grid = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    sel = np.sort(rng.permutation(len(grid))[:natom])
    pos = ((grid[sel] + 0.5) * spacing + rng.uniform(-jitter, jitter, (natom, 3))) * angstrom
    q = np.where(np.arange(natom) % 2 == 0, 0.4, -0.4)
    return {'pos': pos, 'charges': q, 'sigmas': np.full(natom, 3.3 * angstrom),
            'epsilons': np.full(natom, 0.4 * kjmol), 'rvecs': np.eye(3) * box * angstrom}


def mc_guest():
    """The rigid guest: the 3-site water of the NVE workload (O, H, H)."""
    return {'pos': water_geometry(), 'charges': np.array([-0.82, 0.41, 0.41]),
            'sigmas': np.array([3.166 * angstrom, 0.0, 0.0]),
            'epsilons': np.array([0.65 * kjmol, 0.0, 0.0])}


def mc_place_guests(rng, n, rvecs):
    """n rigid waters at uniformly random centres and orientations."""
    body = mc_guest()['pos']
    frac = rng.uniform(0.0, 1.0, (n, 3))
    centres = frac @ rvecs
    rot = _random_rotations(rng, n)
    return centres[:, None, :] + np.einsum('mij,aj->mai', rot, body)


def mc_workload(nchain=256, max_guests=400, seed=5, rcut=12.0):
    """The MC trial-energy workload: one framework, nchain chains with
    seeded loadings uniform in [0, max_guests] rigid waters placed at random,
    rcut 12 A, Ewald alpha 3.5/rcut and gcut 1.1 alpha."""
    rng = np.random.default_rng(seed)
    fw = mc_framework()
    loads = rng.integers(0, max_guests + 1, nchain)
    chains = [mc_place_guests(rng, int(n), fw['rvecs']) for n in loads]
    ew = ewald_params(rcut * angstrom)
    return {'framework': fw, 'guest': mc_guest(), 'chains': chains, 'rcut': rcut * angstrom,
            'alpha': ew['alpha'], 'gcut': ew['gcut'], 'max_guests': max_guests,
            'close_contact': 0.4 * angstrom}


def mc_trial_batch(rng, work, chains_state, ntrial_per_chain=64, chain_ids=None, max_shift=1.0):
    """Random trials for the given chains: a third each of insertions
    (random position and orientation), deletions and translations (shift
    uniform in a cube of +-max_shift A) of a random guest; deletions and
    translations become insertions on an empty chain.  Returns (chain, kind,
    guest, newpos) arrays."""
    rv = work['framework']['rvecs']
    ids = range(len(chains_state)) if chain_ids is None else chain_ids
    ch, kind, guest, newpos = [], [], [], []
    for c in ids:
        n = len(chains_state[c])
        k = rng.integers(0, 3, ntrial_per_chain)
        if n == 0:
            k[:] = 0
        g = rng.integers(0, max(n, 1), ntrial_per_chain)
        ins = mc_place_guests(rng, ntrial_per_chain, rv)
        shift = rng.uniform(-max_shift, max_shift, (ntrial_per_chain, 1, 3)) * angstrom
        npos = np.where((k == 2)[:, None, None], (chains_state[c][g] if n else ins) + shift, ins)
        ch.append(np.full(ntrial_per_chain, c))
        kind.append(k)
        guest.append(np.where(k == 0, -1, g))
        newpos.append(npos)
    return (np.concatenate(ch).astype(np.int32), np.concatenate(kind).astype(np.int32),
            np.concatenate(guest).astype(np.int32), np.ascontiguousarray(np.concatenate(newpos)))
