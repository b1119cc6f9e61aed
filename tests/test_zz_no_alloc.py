"""GPU: the allocation-free Ewald correction entry point.

Callers that cannot let this library allocate device memory -- an engine that
owns all device memory through its own pool, or a step loop that must never
block on an allocation -- use yg_ewald_corr_noalloc, whose only scratch is a
fixed array inside the library.  These tests call it through the C ABI on
caller-owned device buffers and compare energy, gradient and virial with the
context-based entry point (yg_ewald_corr) on two calls in a row, within 1e-10
relative (both are FP64; only the order of the gradient atomics differs).
They also cover a table spanning several blocks of the row kernel, a NULL
gradient, an nlow/nhigh subset, a corrupt row (skipped on the device, NaN
energy) and that a call leaves the device's free memory unchanged.
This file is collected last so that a failing run has already run every
other test.
"""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _golden_ff():
    import yaff_gb300
    spec, data = gc.load('water64')
    return yaff_gb300.build_forcefield(spec, precision='fp64'), data


def _water_ff(nside=6, nlow=0, nhigh=-1):
    """648-atom flexible water: 648 scaling rows, three blocks of the row
    kernel."""
    import yaff_gb300
    from yaff_gb300 import configs
    spec = configs.flexible_water(nside=nside, box=62.1 * nside / 20, rcut=8.0, skin=0.5, name='water_noalloc')
    spec['nlow'] = nlow
    spec['nhigh'] = nhigh
    return yaff_gb300.build_forcefield(spec, precision='fp64'), spec


class _Buffers(object):
    """Caller-owned device buffers of one call, allocated up front."""

    def __init__(self, ff, pos, stab=None):
        import torch
        system = ff.system
        st = ff.part_ewald_cor.scalings.stab if stab is None else stab
        dev = torch.device('cuda')
        self.n = system.natom
        self.nstab = len(st)
        self.pos = torch.tensor(pos, dtype=torch.float64, device=dev)
        self.q = torch.tensor(system.charges, dtype=torch.float64, device=dev)
        self.a = torch.tensor(np.ascontiguousarray(st['a']), dtype=torch.int64, device=dev)
        self.b = torch.tensor(np.ascontiguousarray(st['b']), dtype=torch.int64, device=dev)
        self.s = torch.tensor(np.ascontiguousarray(st['scale']), dtype=torch.float64, device=dev)
        self.e = torch.full((1,), float('nan'), dtype=torch.float64, device=dev)
        self.g = torch.full((self.n, 3), float('nan'), dtype=torch.float64, device=dev)   # must be overwritten
        self.v = torch.full((9,), float('nan'), dtype=torch.float64, device=dev)
        self.rv = np.ascontiguousarray(system.cell.full_rvecs())
        self.gv = np.ascontiguousarray(system.cell.full_gvecs())
        torch.cuda.synchronize()


def _call(ff, buf, nstab=None, with_gpos=True, nlow=None, nhigh=None):
    import torch
    from yaff_gb300 import _lib
    cor = ff.part_ewald_cor
    lib = _lib.load()
    rc = lib.yg_ewald_corr_noalloc(buf.pos.data_ptr(), buf.q.data_ptr(), buf.n, buf.a.data_ptr(), buf.b.data_ptr(),
                                   buf.s.data_ptr(), buf.nstab if nstab is None else nstab, buf.rv.ctypes.data,
                                   buf.gv.ctypes.data, float(ff.system.cell.volume), float(cor.alpha),
                                   float(cor.dielectric), cor.nlow if nlow is None else nlow,
                                   cor.nhigh if nhigh is None else nhigh, buf.e.data_ptr(),
                                   buf.g.data_ptr() if with_gpos else None, buf.v.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc


def _reference(ff, pos):
    n = ff.system.natom
    ff.update_pos(pos)
    g = np.zeros((n, 3))
    v = np.zeros((3, 3))
    e = ff.part_ewald_cor.compute(g, v)
    return e, g, v


def _check(ff, buf, e_ref, g_ref, v_ref, with_gpos=True):
    from yaff_gb300 import _lib
    e = float(buf.e.cpu()[0])
    assert abs(e - e_ref) <= TOL * abs(e_ref), (e, e_ref)
    if with_gpos:
        assert _rel(buf.g.cpu().numpy(), g_ref) <= TOL
    assert _rel(buf.v.cpu().numpy().reshape(3, 3), v_ref) <= TOL
    assert _lib.YG_OK == 0


def test_noalloc_matches_context_entry_two_calls():
    from yaff_gb300 import _lib
    ff, data = _golden_ff()
    assert len(ff.part_ewald_cor.scalings.stab) > 0
    for step in (0, 1):
        pos = data['step%d_pos' % step]
        e_ref, g_ref, v_ref = _reference(ff, pos)
        buf = _Buffers(ff, pos)
        assert _call(ff, buf) == _lib.YG_OK, _lib.load().yg_last_error()
        _check(ff, buf, e_ref, g_ref, v_ref)


def test_noalloc_several_blocks_two_calls():
    # 648 scaling rows: the row kernel runs three blocks and the finishing
    # kernel sums their partials in a fixed order
    from yaff_gb300 import _lib
    ff, spec = _water_ff()
    assert len(ff.part_ewald_cor.scalings.stab) > 512
    rng = np.random.default_rng(3)
    for step in range(2):
        pos = spec['pos'] + rng.uniform(-0.05, 0.05, spec['pos'].shape)
        e_ref, g_ref, v_ref = _reference(ff, pos)
        buf = _Buffers(ff, pos)
        assert _call(ff, buf) == _lib.YG_OK, _lib.load().yg_last_error()
        _check(ff, buf, e_ref, g_ref, v_ref)


def test_noalloc_null_gradient_and_subset():
    # nlow / nhigh restrict the self term and drop the rows inside the outer
    # groups, as ForcePartEwaldCorrection(nlow, nhigh) does; no gradient asked
    from yaff_gb300 import _lib
    ff, spec = _water_ff(nlow=99, nhigh=501)
    pos = spec['pos']
    e_ref, g_ref, v_ref = _reference(ff, pos)
    buf = _Buffers(ff, pos)
    assert _call(ff, buf, with_gpos=False) == _lib.YG_OK, _lib.load().yg_last_error()
    _check(ff, buf, e_ref, g_ref, v_ref, with_gpos=False)
    assert np.isnan(buf.g.cpu().numpy()).all()   # untouched
    # nhigh = -1 stands for natom, as in the reference
    ff2, spec2 = _water_ff(nlow=99, nhigh=-1)
    e2, g2, v2 = _reference(ff2, pos)
    buf2 = _Buffers(ff2, pos)
    assert _call(ff2, buf2, nhigh=-1) == _lib.YG_OK, _lib.load().yg_last_error()
    _check(ff2, buf2, e2, g2, v2)


def test_noalloc_allocates_nothing():
    import torch
    from yaff_gb300 import _lib
    ff, spec = _water_ff()
    pos = spec['pos']
    buf = _Buffers(ff, pos)
    assert _call(ff, buf) == _lib.YG_OK   # first call on the device: resolves the scratch address
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _call(ff, buf) == _lib.YG_OK
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_corrupt_row_is_skipped():
    # a row with an atom index past natom is not dereferenced; the call
    # reports it as a NaN energy, and the next good call is clean again
    from yaff_gb300 import _lib
    ff, data = _golden_ff()
    pos = data['step0_pos']
    stab = ff.part_ewald_cor.scalings.stab.copy()
    stab['a'][5] = ff.system.natom + 1000
    stab['b'][7] = stab['a'][7]
    buf = _Buffers(ff, pos, stab=stab)
    assert _call(ff, buf) == _lib.YG_OK
    assert np.isnan(float(buf.e.cpu()[0]))
    e_ref, g_ref, v_ref = _reference(ff, pos)
    good = _Buffers(ff, pos)
    assert _call(ff, good) == _lib.YG_OK
    _check(ff, good, e_ref, g_ref, v_ref)


def test_noalloc_rejects_oversized_table():
    from yaff_gb300 import _lib
    ff, data = _golden_ff()
    buf = _Buffers(ff, data['step0_pos'])
    assert _call(ff, buf, nstab=(1 << 20) + 1) == _lib.YG_ERR_CAPACITY
    assert b'max' in _lib.load().yg_last_error()
