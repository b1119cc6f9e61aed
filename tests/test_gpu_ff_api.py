"""GPU: ForceField.compute's add-into convention on the fused device path
(yaff/pes/ff.py:117-168): the gradient and virial are ADDED to the caller's
arrays, and the force field's own gpos / vtens (fetched from the device on
access) hold this evaluation's totals."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_compute_adds_into_caller_arrays_and_keeps_totals():
    import yaff_gb300 as ygb
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=600)
    ff = ygb.build_forcefield(spec, precision='mixed')
    n = len(spec['pos'])
    g0 = np.zeros((n, 3))
    v0 = np.zeros((3, 3))
    e0 = ff.compute(g0, v0)
    assert np.array_equal(ff.gpos, g0)
    assert np.array_equal(ff.vtens, v0)
    base_g = np.random.default_rng(1).normal(size=(n, 3))
    base_v = np.random.default_rng(2).normal(size=(3, 3))
    g1 = base_g.copy()
    v1 = base_v.copy()
    e1 = ff.compute(g1, v1)
    assert e1 == e0
    assert np.allclose(g1, base_g + g0, rtol=0, atol=1e-12 * np.abs(g0).max())
    assert np.allclose(v1, base_v + v0, rtol=0, atol=1e-12 * np.abs(v0).max())
    assert np.array_equal(ff.gpos, g0)
    # energy only: no arrays touched, the force field keeps the previous
    # gradient and virial (as yaff's ForcePart does)
    e2 = ff.compute()
    assert e2 == e0
    assert np.array_equal(ff.gpos, g0)
    assert np.array_equal(ff.vtens, v0)
