"""GPU: the mixed-precision reciprocal sum on the tensor cores against the
FP64 form of the same workload.

Two tensor-core forms of the force pass compute the same sums: the tcgen05
kernel (MMAs issued by one thread into tensor-memory accumulators, operands
in shared memory; yg_ewald_info reports 2) and the warp-level MMA kernel
(yg_ewald_force_path(ctx, 1); reports 1).  Tolerances are those of the
mixed form in the parity suite: energy 1e-6 relative, gradient 1e-5
relative RMS, virial 1e-6 relative to its largest entry; the two force-pass
kernels agree with each other within 2e-6 relative RMS (both FP16-split
products with FP32 accumulation, summed in different orders).  The
3,000-atom triclinic box has enough atoms for several 128-atom blocks and
the force pass split into tile ranges; the nlow/nhigh case runs the
three-group form (three structure factors, three weight sets).  The
structure-factor (S) pass has the same two forms (yg_ewald_sfac_path: 1
warp-level MMA, the automatic choice; 2 tcgen05); every combination is
compared with FP64."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reci(spec, precision, nlow=None, nhigh=None, force_path=0, sfac_path=0):
    import yaff_gb300 as ygb
    if nlow is not None:
        spec = dict(spec)
        spec['nlow'], spec['nhigh'] = nlow, nhigh
    ff = ygb.build_forcefield(spec, precision=precision)
    dev = ygb.device_of(ff.system)
    assert dev.lib.yg_ewald_force_path(dev.ctx, force_path) == 0
    assert dev.lib.yg_ewald_sfac_path(dev.ctx, sfac_path) == 0
    n = len(spec['pos'])
    gpos = np.zeros((n, 3))
    vt = np.zeros((3, 3))
    ff.compute(gpos, vt)
    part = [p for p in ff.parts if p.name == 'ewald_reci'][0]
    tensor, nk = ctypes.c_int(), ctypes.c_int64()
    dev.lib.yg_ewald_info(dev.ctx, ctypes.byref(tensor), ctypes.byref(nk))
    return part.energy, part.gpos.copy(), part.vtens.copy(), tensor.value, nk.value


def _rel_rms(a, b):
    return np.sqrt(((a - b) ** 2).mean()) / np.sqrt((b ** 2).mean())


def _compare(ref, mix):
    e0, g0, v0 = ref[:3]
    e1, g1, v1 = mix[:3]
    assert abs(e1 - e0) <= 1e-6 * abs(e0)
    assert _rel_rms(g1, g0) <= 1e-5, _rel_rms(g1, g0)
    assert np.abs(v1 - v0).max() <= 1e-6 * np.abs(v0).max()


@pytest.mark.parametrize('force_path,sfac_path', [(0, 1), (1, 1), (0, 2), (1, 2)])
def test_tensor_core_reciprocal_matches_fp64(force_path, sfac_path):
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=3000)
    ref = _reci(spec, 'fp64')
    mix = _reci(spec, 'mixed', force_path=force_path, sfac_path=sfac_path)
    assert mix[3] == (2 if force_path == 0 else 1) and mix[4] == ref[4] > 1000
    _compare(ref, mix)


@pytest.mark.parametrize('force_path,sfac_path', [(0, 1), (1, 1), (0, 2), (1, 2)])
def test_tensor_core_reciprocal_three_groups(force_path, sfac_path):
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=3000)
    ref = _reci(spec, 'fp64', nlow=700, nhigh=2300)
    mix = _reci(spec, 'mixed', nlow=700, nhigh=2300, force_path=force_path, sfac_path=sfac_path)
    assert mix[3] == (2 if force_path == 0 else 1)
    _compare(ref, mix)


@pytest.mark.parametrize('natom,nlow,nhigh', [(3000, None, None), (3000, 700, 2300), (999, 0, 998)])
def test_tcgen05_and_warp_mma_s_passes_agree(natom, nlow, nhigh):
    """The two S-pass kernels sum the same FP16-split products over the same
    atom chunks in different orders (tcgen05: 32-atom TMEM accumulations;
    warp MMA: 16-atom register accumulations): energies within 2e-7
    relative, gradients within 1e-6 relative RMS, virials within 1e-6 of the
    largest entry (the FP64 bound of each; measured 2.9e-7 at 3,000 atoms).
    999 atoms leave a ragged last stage (a single 16-atom K-step) and one atom
    in the top group."""
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=natom)
    a = _reci(spec, 'mixed', nlow=nlow, nhigh=nhigh, sfac_path=2)
    b = _reci(spec, 'mixed', nlow=nlow, nhigh=nhigh, sfac_path=1)
    assert abs(a[0] - b[0]) <= 2e-7 * abs(b[0]), (a[0], b[0])
    assert _rel_rms(a[1], b[1]) <= 1e-6, _rel_rms(a[1], b[1])
    assert np.abs(a[2] - b[2]).max() <= 1e-6 * np.abs(b[2]).max()


def test_tcgen05_and_warp_mma_force_passes_agree():
    from yaff_gb300 import configs
    spec = configs.triclinic_mm3_ei(natom=3000)
    a = _reci(spec, 'mixed', force_path=0)
    b = _reci(spec, 'mixed', force_path=1)
    assert a[3] == 2 and b[3] == 1
    assert a[0] == b[0]   # same structure factors and energy kernel
    assert _rel_rms(a[1], b[1]) <= 2e-6, _rel_rms(a[1], b[1])
