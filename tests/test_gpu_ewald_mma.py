"""GPU: the mixed-precision reciprocal sum on the tensor cores (warp MMA with
FP16 hi/lo split operands) against the FP64 form of the same workload.

Tolerances are those of the mixed form in the parity suite: energy 1e-6
relative, gradient 1e-5 relative RMS, virial 1e-6 relative to its largest
entry.  The 3,000-atom triclinic box has enough atoms for several S-pass
chunks and a force pass split into column ranges; the nlow/nhigh case runs
the three-group form (three structure factors, three weight sets)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reci(spec, precision, nlow=None, nhigh=None):
    import yaff_gb300 as ygb
    if nlow is not None:
        spec = dict(spec)
        spec['nlow'], spec['nhigh'] = nlow, nhigh
    ff = ygb.build_forcefield(spec, precision=precision)
    n = len(spec['pos'])
    gpos = np.zeros((n, 3))
    vt = np.zeros((3, 3))
    ff.compute(gpos, vt)
    part = [p for p in ff.parts if p.name == 'ewald_reci'][0]
    dev = ygb.device_of(ff.system)
    tensor, nk = ctypes.c_int(), ctypes.c_int64()
    dev.lib.yg_ewald_info(dev.ctx, ctypes.byref(tensor), ctypes.byref(nk))
    return part.energy, part.gpos.copy(), part.vtens.copy(), tensor.value, nk.value


def _compare(ref, mix):
    e0, g0, v0 = ref[:3]
    e1, g1, v1 = mix[:3]
    assert abs(e1 - e0) <= 1e-6 * abs(e0)
    grms = np.sqrt(((g1 - g0) ** 2).mean()) / np.sqrt((g0 ** 2).mean())
    assert grms <= 1e-5, grms
    assert np.abs(v1 - v0).max() <= 1e-6 * np.abs(v0).max()


def test_tensor_core_reciprocal_matches_fp64():
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=3000)
    ref = _reci(spec, 'fp64')
    mix = _reci(spec, 'mixed')
    assert mix[3] == 1 and mix[4] == ref[4] > 1000   # the tensor-core layout was used
    _compare(ref, mix)


def test_tensor_core_reciprocal_three_groups():
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=3000)
    ref = _reci(spec, 'fp64', nlow=700, nhigh=2300)
    mix = _reci(spec, 'mixed', nlow=700, nhigh=2300)
    assert mix[3] == 1
    _compare(ref, mix)
