"""GPU: the allocation-free Ewald correction entry point.

Callers that cannot let this library allocate device memory -- an engine that
owns all device memory through its own pool, or a step loop that must never
block on an allocation -- use yg_ewald_corr_noalloc, whose only scratch is a
fixed array inside the library.  These tests call it through the C ABI on
caller-owned device buffers and compare energy, gradient and virial with the
context-based entry point (yg_ewald_corr) on two calls in a row, within 1e-10
relative (both are FP64; only the order of the gradient atomics differs).
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


def _setup():
    import torch
    import yaff_gb300
    from yaff_gb300 import _lib
    spec, data = gc.load('water64')
    ff = yaff_gb300.build_forcefield(spec, precision='fp64')
    return torch, _lib, ff, data


def _noalloc(torch, _lib, ff, pos, nstab=None):
    cor = ff.part_ewald_cor
    system = ff.system
    st = cor.scalings.stab
    n = system.natom
    dev = torch.device('cuda')
    dpos = torch.tensor(pos, dtype=torch.float64, device=dev)
    dq = torch.tensor(system.charges, dtype=torch.float64, device=dev)
    da = torch.tensor(np.ascontiguousarray(st['a']), dtype=torch.int64, device=dev)
    db = torch.tensor(np.ascontiguousarray(st['b']), dtype=torch.int64, device=dev)
    ds = torch.tensor(np.ascontiguousarray(st['scale']), dtype=torch.float64, device=dev)
    de = torch.full((1,), float('nan'), dtype=torch.float64, device=dev)
    dg = torch.full((n, 3), float('nan'), dtype=torch.float64, device=dev)   # must be overwritten
    dv = torch.full((9,), float('nan'), dtype=torch.float64, device=dev)
    rv = np.ascontiguousarray(system.cell.full_rvecs())
    gv = np.ascontiguousarray(system.cell.full_gvecs())
    lib = _lib.load()
    rc = lib.yg_ewald_corr_noalloc(dpos.data_ptr(), dq.data_ptr(), n, da.data_ptr(), db.data_ptr(), ds.data_ptr(),
                                   len(st) if nstab is None else nstab, rv.ctypes.data, gv.ctypes.data,
                                   float(system.cell.volume), float(cor.alpha), float(cor.dielectric), cor.nlow,
                                   cor.nhigh, de.data_ptr(), dg.data_ptr(), dv.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, float(de.cpu()[0]), dg.cpu().numpy(), dv.cpu().numpy().reshape(3, 3)


def test_noalloc_matches_context_entry_two_calls():
    torch, _lib, ff, data = _setup()
    cor = ff.part_ewald_cor
    n = ff.system.natom
    assert len(cor.scalings.stab) > 0
    for step in (0, 1):
        pos = data['step%d_pos' % step]
        ff.update_pos(pos)
        g_ref = np.zeros((n, 3))
        v_ref = np.zeros((3, 3))
        e_ref = cor.compute(g_ref, v_ref)
        rc, e, g, v = _noalloc(torch, _lib, ff, pos)
        assert rc == _lib.YG_OK, _lib.load().yg_last_error()
        assert abs(e - e_ref) <= TOL * abs(e_ref)
        assert _rel(g, g_ref) <= TOL
        assert _rel(v, v_ref) <= TOL


def test_noalloc_rejects_oversized_table():
    torch, _lib, ff, data = _setup()
    rc, e, g, v = _noalloc(torch, _lib, ff, data['step0_pos'], nstab=(1 << 20) + 1)
    assert rc == _lib.YG_ERR_CAPACITY
    assert b'max' in _lib.load().yg_last_error()
