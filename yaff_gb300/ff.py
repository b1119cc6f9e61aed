"""Force-field parts with the reference's ForcePart / ForceField interface.

Mirrors yaff/pes/ff.py:
  * ForcePart.compute(gpos=None, vtens=None) zeros the part's own buffers,
    evaluates, raises ValueError on NaN energy/gpos/vtens and ADDS into the
    caller's arrays (ff.py:117-168);
  * ForceField(system, parts, nlist) updates the neighbour list when the
    positions changed and sums its parts (ff.py:178-273), with the parts
    reachable as ``ff.part_<name>``;
  * ForcePartPair, ForcePartEwaldReciprocal / Correction / Neutralizing and
    ForcePartValence take the reference's constructor arguments.

GPU specifics: when every part of a ForceField lives on the same device
system, ``ForceField.compute`` runs the fused path -- one position upload,
one pass of the pair kernel for all pair parts, the Ewald and valence
kernels, and a single device-to-host copy of the summed result.  The parts'
own ``gpos``/``vtens`` are then fetched from the device only when read.
"""
import numpy as np

from . import _lib
from ._lib import check
from .device import device_of
from .system import as_system
from .valence import DeltaList, InternalCoordinateList, ValenceList

__all__ = ['ForcePart', 'ForceField', 'ForcePartPair', 'ForcePartEwaldReciprocal', 'ForcePartEwaldCorrection',
           'ForcePartEwaldNeutralizing', 'ForcePartTailCorrection', 'ForcePartValence']


class ForcePart(object):
    """Base class: anything that computes an energy, gradient and virial."""
    device_slot = None

    def __init__(self, name, system):
        system = as_system(system)
        self.name = name
        self.system = system
        self.energy = 0.0
        self._gpos = np.zeros((system.natom, 3), float)
        self._vtens = np.zeros((3, 3), float)
        self._lazy = None
        self.clear()

    def _fetch(self):
        if self._stale:
            # cleared results read as NaN (filled on first access, not per step)
            self._stale = False
            self._gpos[:] = np.nan
            self._vtens[:] = np.nan
            self._gpos_zero = False
        if self._lazy is not None:
            dev, slot, want_g, want_v = self._lazy
            self._lazy = None
            dev.get_part(slot, self._gpos if want_g else None, self._vtens if want_v else None)

    @property
    def gpos(self):
        self._fetch()
        return self._gpos

    @gpos.setter
    def gpos(self, value):
        self._lazy = None
        self._stale = False
        self._gpos = value
        self._gpos_zero = False

    @property
    def vtens(self):
        self._fetch()
        return self._vtens

    @vtens.setter
    def vtens(self, value):
        self._lazy = None
        self._stale = False
        self._vtens = value

    def clear(self):
        """The cached results no longer hold: energy, gpos and vtens read as
        NaN until the next compute."""
        self._lazy = None
        self.energy = np.nan
        self._stale = True

    def update_rvecs(self, rvecs):
        self.clear()

    def update_pos(self, pos):
        self.clear()

    def compute(self, gpos=None, vtens=None):
        """Energy; the gradient and virial are ADDED to gpos / vtens."""
        self._lazy = None
        self._stale = False
        my_gpos = None
        if gpos is not None:
            my_gpos = self._gpos
            my_gpos[:] = 0.0
        my_vtens = None
        if vtens is not None:
            my_vtens = self._vtens
            my_vtens[:] = 0.0
        self.energy = self._internal_compute(my_gpos, my_vtens)
        if np.isnan(self.energy):
            raise ValueError('The energy is not-a-number (nan).')
        if gpos is not None:
            if np.isnan(my_gpos).any():
                raise ValueError('Some gpos element(s) is/are not-a-number (nan).')
            gpos += my_gpos
        if vtens is not None:
            if np.isnan(my_vtens).any():
                raise ValueError('Some vtens element(s) is/are not-a-number (nan).')
            vtens += my_vtens
        return self.energy

    def _internal_compute(self, gpos, vtens):
        raise NotImplementedError

    # fused-path hooks (GPU parts)
    def _launch(self, want_grad):
        raise NotImplementedError


class ForceField(ForcePart):
    """A complete force field: a neighbour list and a list of parts."""

    def __init__(self, system, parts, nlist=None):
        system = as_system(system)
        ForcePart.__init__(self, 'all', system)
        self._host_vtens = None
        self._total_mask = 0
        self.parts = []
        self.nlist = nlist
        self.needs_nlist_update = nlist is not None
        for part in parts:
            self.add_part(part)

    def add_part(self, part):
        self.parts.append(part)
        name = 'part_%s' % part.name
        if name in self.__dict__:
            raise ValueError('The part %s occurs twice in the force field.' % name)
        self.__dict__[name] = part

    def update_rvecs(self, rvecs):
        ForcePart.update_rvecs(self, rvecs)
        self.system.cell.update_rvecs(rvecs)
        for part in self.parts:
            part.update_rvecs(rvecs)
        if self.nlist is not None:
            self.nlist.update_rmax()
            self.needs_nlist_update = True

    def update_pos(self, pos):
        ForcePart.update_pos(self, pos)
        self.system.pos[:] = pos
        for part in self.parts:
            part.update_pos(pos)
        if self.nlist is not None:
            self.needs_nlist_update = True

    def _device_parts(self):
        """The device system when every part can run fused on it, else None."""
        dev = None
        for part in self.parts:
            if part.device_slot is None and not getattr(part, 'host_scalar', False):
                return None
        if self.system.cell.nvec != 3:
            return None
        dev = device_of(self.system)
        return dev

    def _internal_compute(self, gpos, vtens, add=False):
        dev = self._device_parts()
        if dev is None:
            if self.needs_nlist_update:
                self.nlist.update()
                self.needs_nlist_update = False
            return sum([part.compute(gpos, vtens) for part in self.parts])
        # fused device path: positions first, then the reciprocal sum (it
        # needs no neighbour list and runs on its own stream while the list
        # is updated and the pair terms are evaluated); the readback at the
        # end synchronizes before the caller gets control back
        dev.upload_positions(wait=False)
        # the parts' set-up checks (charges) run once per evaluation
        self._ncall = getattr(self, '_ncall', 0) + 1
        dev.call_key = (id(self), self._ncall)
        try:
            try:
                return self._fused_compute(dev, gpos, vtens, add, defer=True)
            except _lib.YaffGBError as exc:
                if exc.status != _lib.YG_ERR_CAPACITY or self.nlist is None:
                    raise
                # the enqueued rebuild overflowed a row (its capacity has grown);
                # nothing reached the caller's arrays: rebuild and evaluate again
                self.nlist._pending = False
                self.nlist.rebuild_next = True
                self.needs_nlist_update = True
                return self._fused_compute(dev, gpos, vtens, add, defer=False)
        finally:
            dev.call_key = None

    def _fused_compute(self, dev, gpos, vtens, add, defer=False):
        want_grad = (gpos is not None) or (vtens is not None)
        mask = 0
        for part in self.parts:
            if isinstance(part, ForcePartEwaldReciprocal):
                part._launch(want_grad)
                mask |= 1 << part.device_slot
        if self.needs_nlist_update:
            # the rebuild is enqueued without waiting for its row count: the
            # pair terms follow it on the stream at once; the readback below
            # reports an overflow before anything is added to gpos / vtens
            self.nlist.update(upload=False, defer=defer)
            self.needs_nlist_update = False
        pair_parts = [p for p in self.parts if isinstance(p, ForcePartPair)]
        if pair_parts:
            slots = [p._register() for p in pair_parts]
            pmask = 0
            for s in slots:
                pmask |= 1 << s
            check(dev.lib.yg_pair_compute(dev.ctx, pmask, int(want_grad)), 'yg_pair_compute')
            mask |= pmask
        host_energy = 0.0
        host_vtens = np.zeros((3, 3)) if vtens is not None else None
        for part in self.parts:
            if isinstance(part, (ForcePartPair, ForcePartEwaldReciprocal)) or getattr(part, 'host_scalar', False):
                continue
            part._launch(want_grad)
            mask |= 1 << part.device_slot
        # the summed gradient and virial land directly in the caller's arrays
        # (added to them with add=True); NaN in the gradient is detected on
        # the device
        if add:
            energy, part_e = dev.get_total_add(mask, gpos, vtens)
        else:
            energy, part_e = dev.get_total_into(mask, gpos, vtens)
        self._total_mask = mask
        for part in self.parts:
            if getattr(part, 'host_scalar', False):
                # position independent, no gradient (ff.py:653-669, :1052-1058)
                pv = np.zeros((3, 3)) if vtens is not None else None
                e = part._internal_compute(None, pv)
                part.energy = e
                part._lazy = None
                part._stale = False
                if not getattr(part, '_gpos_zero', False):
                    # no gradient: zeroed once, not per call (1.2 MB at 50,000 atoms)
                    part._gpos[:] = 0.0
                    part._gpos_zero = True
                if pv is not None:
                    part._vtens[:] = pv
                    host_vtens += pv
                host_energy += e
                continue
            slot = part._slot_index()
            part.energy = part_e[slot]
            part._lazy = (dev, slot, gpos is not None, vtens is not None)
        energy += host_energy
        if vtens is not None:
            vtens += host_vtens
        self._host_vtens = host_vtens
        return energy

    def compute(self, gpos=None, vtens=None):
        """Energy; the gradient and virial are ADDED to gpos / vtens.  On the
        fused device path they are added to the caller's arrays straight from
        the library's page-locked readback (one pass over gpos); the force
        field's own `gpos` / `vtens` are fetched from the device on access."""
        if self._device_parts() is None:
            return ForcePart.compute(self, gpos, vtens)
        if (gpos is None or vtens is None) and self._lazy is not None:
            # yaff keeps the previous gpos / vtens when this call does not
            # compute them: take them from the device before they are replaced
            self._fetch()
        self._lazy = None
        self._stale = False
        self.energy = self._internal_compute(gpos, vtens, add=True)
        if np.isnan(self.energy):
            raise ValueError('The energy is not-a-number (nan).')
        if vtens is not None and np.isnan(vtens).any():
            raise ValueError('Some vtens element(s) is/are not-a-number (nan).')
        self._lazy = ('total', self._device_parts(), self._total_mask, gpos is not None, vtens is not None)
        return self.energy

    def _fetch(self):
        if self._lazy is not None and self._lazy[0] == 'total':
            _, dev, mask, want_g, want_v = self._lazy
            self._lazy = None
            dev.get_total_into(mask, self._gpos if want_g else None, self._vtens if want_v else None)
            if want_v and self._host_vtens is not None:
                self._vtens += self._host_vtens
            return
        ForcePart._fetch(self)

    def device_md_terms(self):
        """(result-slot mask, constant energy) for an integrator that sums the
        force on the device: the slots the fused path fills, and the
        energy of the host-evaluated parts (neutralizing background, tail
        corrections), which does not depend on the positions.  Valid after one compute()."""
        dev = self._device_parts()
        if dev is None:
            raise NotImplementedError('the on-device integrator needs every part on the fused device path')
        mask = 0
        const = 0.0
        for part in self.parts:
            if getattr(part, 'host_scalar', False):
                const += part.compute()
            elif isinstance(part, ForcePartPair):
                mask |= 1 << part._register()
            else:
                mask |= 1 << part.device_slot
        return dev, mask, const


class ForcePartPair(ForcePart):
    """A pairwise non-bonding term evaluated over the shared neighbour list."""
    device_slot = 'pair'

    def __init__(self, system, nlist, scalings, pair_pot):
        system = as_system(system)
        ForcePart.__init__(self, 'pair_%s' % pair_pot.name, system)
        self.nlist = nlist
        self.scalings = scalings
        self.pair_pot = pair_pot
        self.nlist.request_rcut(pair_pot.rcut)
        self._slot = None
        self._register()

    def _register(self):
        dev = device_of(self.system)
        dev.set_scalings(self.scalings)
        self._slot = dev.register_pair(self)
        return self._slot

    def _slot_index(self):
        return _lib.PART_PAIR0 + self._slot

    def _internal_compute(self, gpos, vtens):
        dev = device_of(self.system)
        slot = self._register()
        want = int(gpos is not None or vtens is not None)
        check(dev.lib.yg_pair_compute(dev.ctx, 1 << slot, want), 'yg_pair_compute')
        return dev.get_part(_lib.PART_PAIR0 + slot, gpos, vtens)


def _check_nlow_nhigh(system, nlow, nhigh):
    if nlow < 0:
        raise ValueError('nlow must be a positive number, received %d.' % nlow)
    if nhigh == -1:
        nhigh = system.natom
    if nhigh < nlow:
        raise ValueError('nhigh must not be smaller than nlow, received %d.' % nhigh)
    return nlow, nhigh


class ForcePartEwaldReciprocal(ForcePart):
    """Long-range (reciprocal-space) electrostatics of a 3D periodic system."""
    device_slot = _lib.PART_EWALD_RECI

    def __init__(self, system, alpha, gcut=0.35, dielectric=1.0, nlow=0, nhigh=-1):
        system = as_system(system)
        ForcePart.__init__(self, 'ewald_reci', system)
        if not system.cell.nvec == 3:
            raise TypeError('The system must have a 3D periodic cell.')
        if system.charges is None:
            raise ValueError('The system does not have charges.')
        self.alpha = alpha
        self.gcut = gcut
        self.dielectric = dielectric
        self.nlow, self.nhigh = _check_nlow_nhigh(system, nlow, nhigh)
        self.update_gmax()

    def update_gmax(self):
        self.gmax = np.ceil(self.gcut / self.system.cell.gspacings - 0.5).astype(int)
        self._setup_key = None

    def update_rvecs(self, rvecs):
        ForcePart.update_rvecs(self, rvecs)
        self.update_gmax()

    def _slot_index(self):
        return self.device_slot

    def _setup(self, dev):
        dev.sync_cell()
        dev.sync_charges()
        key = (self.alpha, self.gcut, tuple(self.gmax), self.dielectric, self.nlow, self.nhigh, dev._cell_key)
        if key != getattr(dev, 'ewald_key', None):
            gmax = np.ascontiguousarray(self.gmax, dtype=np.int64)
            check(dev.lib.yg_ewald_setup(dev.ctx, float(self.alpha), float(self.gcut), _lib.ptr(gmax),
                                         float(self.dielectric), self.nlow, self.nhigh), 'yg_ewald_setup')
            dev.ewald_key = key

    def _launch(self, want_grad):
        dev = device_of(self.system)
        self._setup(dev)
        check(dev.lib.yg_ewald_reci(dev.ctx, int(want_grad)), 'yg_ewald_reci')

    def _internal_compute(self, gpos, vtens):
        dev = device_of(self.system)
        dev.upload_positions()
        self._launch(gpos is not None or vtens is not None)
        return dev.get_part(self.device_slot, gpos, vtens)


class ForcePartEwaldCorrection(ForcePart):
    """Self-energy and excluded-pair correction of the Ewald sum."""
    device_slot = _lib.PART_EWALD_CORR

    def __init__(self, system, alpha, scalings, dielectric=1.0, nlow=0, nhigh=-1):
        system = as_system(system)
        ForcePart.__init__(self, 'ewald_cor', system)
        if not system.cell.nvec == 3:
            raise TypeError('The system must have a 3D periodic cell')
        if system.charges is None:
            raise ValueError('The system does not have charges.')
        self.alpha = alpha
        self.dielectric = dielectric
        self.nlow, self.nhigh = _check_nlow_nhigh(system, nlow, nhigh)
        self.scalings = scalings
        self.gcut = 1.0

    def _slot_index(self):
        return self.device_slot

    def _launch(self, want_grad):
        dev = device_of(self.system)
        dev.sync_cell()
        dev.sync_charges()
        dev.set_scalings(self.scalings)
        key = getattr(dev, 'ewald_key', None)
        if key is None or key[0] != self.alpha or key[3] != self.dielectric or key[4:6] != (self.nlow, self.nhigh):
            # the correction only needs alpha / dielectric / nlow / nhigh; set a
            # trivial reciprocal grid when no reciprocal part configured one
            gmax = np.zeros(3, np.int64)
            check(dev.lib.yg_ewald_setup(dev.ctx, float(self.alpha), 1e-300 + 1e-9, _lib.ptr(gmax),
                                         float(self.dielectric), self.nlow, self.nhigh), 'yg_ewald_setup')
            dev.ewald_key = (self.alpha, None, None, self.dielectric, self.nlow, self.nhigh, dev._cell_key)
        check(dev.lib.yg_ewald_corr(dev.ctx, int(want_grad)), 'yg_ewald_corr')

    def _internal_compute(self, gpos, vtens):
        dev = device_of(self.system)
        dev.upload_positions()
        self._launch(gpos is not None or vtens is not None)
        return dev.get_part(self.device_slot, gpos, vtens)


class ForcePartEwaldNeutralizing(ForcePart):
    """Neutralizing-background term of a charged periodic system (host FP64,
    yaff/pes/ff.py:590-669)."""
    host_scalar = True

    def __init__(self, system, alpha, dielectric=1.0, nlow=0, nhigh=-1, fluctuating_charges=False):
        system = as_system(system)
        ForcePart.__init__(self, 'ewald_neut', system)
        if not system.cell.nvec == 3:
            raise TypeError('The system must have a 3D periodic cell')
        if system.charges is None:
            raise ValueError('The system does not have charges.')
        self.alpha = alpha
        self.dielectric = dielectric
        self.nlow, self.nhigh = _check_nlow_nhigh(system, nlow, nhigh)
        self.fluctuating_charges = fluctuating_charges
        if not fluctuating_charges:
            self.prefactor = self._fac() * np.pi / (2.0 * self.dielectric)

    def _fac(self):
        q = self.system.charges
        fac = q[:].sum() ** 2 / self.alpha ** 2
        fac -= q[:self.nlow].sum() ** 2 / self.alpha ** 2
        fac -= q[self.nhigh:].sum() ** 2 / self.alpha ** 2
        r = self.system.radii
        if r is not None:
            fac -= q.sum() * np.sum(q * r ** 2)
            fac += q[:self.nlow].sum() * np.sum(q[:self.nlow] * r[:self.nlow] ** 2)
            fac += q[self.nhigh:].sum() * np.sum(q[self.nhigh:] * r[self.nhigh:] ** 2)
        return fac

    def _internal_compute(self, gpos, vtens):
        if not self.fluctuating_charges:
            fac = self.prefactor / self.system.cell.volume
        else:
            fac = self._fac() * np.pi / (2.0 * self.system.cell.volume * self.dielectric)
        if vtens is not None:
            vtens.ravel()[::4] -= fac
        return fac


class ForcePartTailCorrection(ForcePart):
    """Long-range correction of a truncated pair potential, assuming a
    homogeneous system beyond the cutoff: energy 2 pi C0 / V and virial
    diagonal 2 pi C1 / V, with C0 and C1 summed once over atom pairs by
    ``pair_pot.prepare_tailcorrections`` (yaff/pes/ff.py:1012-1058).  Host
    FP64 scalars, no gradient; the energy depends on the volume only."""
    host_scalar = True

    def __init__(self, system, part_pair, nlow=0, nhigh=-1):
        system = as_system(system)
        if system.cell.nvec != 3:
            raise ValueError('Tail corrections can only be applied to 3D periodic systems')
        if part_pair.name in ['pair_ei', 'pair_eidip']:
            raise ValueError('Tail corrections are divergent for %s' % part_pair.name)
        ForcePart.__init__(self, 'tailcorr_%s' % part_pair.name, system)
        self.nlow, self.nhigh = _check_nlow_nhigh(system, nlow, nhigh)
        self.ecorr, self.wcorr = part_pair.pair_pot.prepare_tailcorrections(system.natom, self.nlow, self.nhigh)

    def _internal_compute(self, gpos, vtens):
        if vtens is not None:
            w = 2.0 * np.pi * self.wcorr / self.system.cell.volume
            vtens[0, 0] += w
            vtens[1, 1] += w
            vtens[2, 2] += w
        return 2.0 * np.pi * self.ecorr / self.system.cell.volume


class ForcePartValence(ForcePart):
    """Covalent terms through the relative-vector / internal-coordinate /
    energy-term chain, evaluated and back-propagated on the GPU."""
    device_slot = _lib.PART_VALENCE

    def __init__(self, system, comlist=None):
        system = as_system(system)
        ForcePart.__init__(self, 'valence', system)
        if comlist is not None:
            raise NotImplementedError('centre-of-mass layers are not supported on the device')
        self.dlist = DeltaList(system)
        self.iclist = InternalCoordinateList(self.dlist)
        self.vlist = ValenceList(self.iclist)
        self._uploaded = None

    def add_term(self, term):
        self.vlist.add_term(term)

    def _slot_index(self):
        return self.device_slot

    def _launch(self, want_grad):
        dev = device_of(self.system)
        dev.sync_cell()
        key = (id(self.vlist), self.vlist.version)
        if getattr(dev, 'valence_key', None) != key:
            dij, ics, kinds, pars, vic = self.vlist.arrays()
            check(dev.lib.yg_set_valence(dev.ctx, _lib.ptr(np.ascontiguousarray(dij)), len(dij),
                                         _lib.ptr(np.ascontiguousarray(ics)), len(ics),
                                         _lib.ptr(np.ascontiguousarray(kinds)), _lib.ptr(np.ascontiguousarray(pars)),
                                         _lib.ptr(np.ascontiguousarray(vic)), len(kinds)), 'yg_set_valence')
            dev.valence_key = key
        check(dev.lib.yg_valence_compute(dev.ctx, int(want_grad)), 'yg_valence_compute')

    def _internal_compute(self, gpos, vtens):
        dev = device_of(self.system)
        dev.upload_positions()
        self._launch(gpos is not None or vtens is not None)
        return dev.get_part(self.device_slot, gpos, vtens)
