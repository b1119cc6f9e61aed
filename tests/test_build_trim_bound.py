"""The lower bound the candidate sweep uses to trim each stencil row to an
atom's reach (yaff_gb300/csrc/yg_nlist.cu, trim_row), restated on the host
and checked against the exact distance from the atom to the cell.

For an atom at phi (cell widths from its cell's corner) and the cell at
offset o, every point of that cell is d = sum_k Delta_k M_k with Delta_k in
[o_k - phi_k, o_k - phi_k + 1] (M_k = the grid cell's edge vectors).  The
kernel keeps a cell unless |p| - sum_k |u.M_k| / 2 reaches the limit, with p
the centre offset and u = p / |p|, formed along a row as a quadratic in the
x offset; a row is empty when its slab bound along axis 1 or 2 reaches the
limit.  Both must be lower bounds of min |d| over the cell, which
scipy.optimize.lsq_linear gives exactly (a box-constrained least-squares
problem).  Random triclinic cells, grids and positions; no GPU."""
import numpy as np
import pytest


def _cell(rng):
    a, b, c = rng.uniform(20.0, 60.0, 3)
    al, be, ga = np.radians(rng.uniform(60.0, 120.0, 3))
    rv = np.zeros((3, 3))
    rv[0] = [a, 0, 0]
    rv[1] = [b * np.cos(ga), b * np.sin(ga), 0]
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    rv[2] = [cx, cy, np.sqrt(max(c * c - cx * cx - cy * cy, 1e-6))]
    return rv


def _row_bound(M, phi, o1, o2, o0):
    """trim_row's per-cell test value, formed as the kernel forms it (FP64)."""
    c1, c2 = o1 - phi[1] + 0.5, o2 - phi[2] + 0.5
    q = c1 * M[1] + c2 * M[2]
    qq, qm = q @ q, M @ q
    g0 = M @ M[0]
    c0 = o0 - phi[0] + 0.5
    pp = c0 * (c0 * g0[0] + 2.0 * qm[0]) + qq
    ext = abs(c0 * g0[0] + qm[0]) + abs(c0 * g0[1] + qm[1]) + abs(c0 * g0[2] + qm[2])
    if not pp > 0.0:
        return -np.inf
    return np.sqrt(pp) - 0.5 * ext / np.sqrt(pp)


def _slab(w, phi, k, ok):
    a = ok - phi[k]
    return w[k] * max(0.0, a, -a - 1.0)


@pytest.mark.parametrize('seed', range(6))
def test_trim_bounds_never_exceed_the_atom_to_cell_distance(seed):
    from scipy.optimize import lsq_linear
    rng = np.random.default_rng(seed)
    rv = _cell(rng)
    n = rng.integers(3, 12, 3)
    M = rv / n[:, None]                      # grid cell edge vectors
    gv = np.linalg.inv(rv).T
    w = 1.0 / np.linalg.norm(gv, axis=1) / n  # slab widths along the plane normals
    worst = np.inf
    for _ in range(60):
        phi = rng.uniform(0.0, 1.0, 3)
        o = rng.integers(-5, 6, 3)
        lo = o - phi
        res = lsq_linear(M.T, np.zeros(3), bounds=(lo, lo + 1.0), method='bvls')
        dmin = np.linalg.norm(M.T @ res.x)
        b_dir = _row_bound(M, phi, o[1], o[2], o[0])
        b_slab = max(_slab(w, phi, 1, o[1]), _slab(w, phi, 2, o[2]))
        assert b_dir <= dmin * (1 + 1e-12) + 1e-9, (b_dir, dmin)
        assert b_slab <= dmin * (1 + 1e-12) + 1e-9, (b_slab, dmin)
        worst = min(worst, dmin - max(b_dir, b_slab))
    assert worst >= -1e-9
