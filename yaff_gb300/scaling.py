"""Short-range scaling (exclusion) table, the reference's Scalings
(yaff/pes/scaling.py:58-105): rows (a > b, scale, nbond) for 1-2, 1-3, 1-4
and 1-5 pairs whose scale is below one, sorted by (a, b)."""
import numpy as np
from .system import as_system

__all__ = ['Scalings', 'scaling_dtype']

scaling_dtype = np.dtype([('a', 'i8'), ('b', 'i8'), ('scale', 'f8'), ('nbond', 'i8')])


class Scalings(object):
    def __init__(self, system, scale1=0.0, scale2=0.0, scale3=1.0, scale4=1.0):
        system = as_system(system)
        for name, s in (('scale1', scale1), ('scale2', scale2), ('scale3', scale3), ('scale4', scale4)):
            if s < -1 or s > 1:
                raise ValueError('%s must be in the range [-1,1].' % name)
        self.scale1 = scale1
        self.scale2 = scale2
        self.scale3 = scale3
        self.scale4 = scale4
        stab = []
        if system.bonds is not None:
            for i0 in range(system.natom):
                for nb, sc, neigh in ((1, scale1, system.neighs1), (2, scale2, system.neighs2),
                                      (3, scale3, system.neighs3), (4, scale4, system.neighs4)):
                    if sc < 1.0:
                        for i1 in neigh[i0]:
                            if i0 > i1:
                                stab.append((i0, i1, sc, nb))
        stab.sort()
        self.stab = np.array(stab, dtype=scaling_dtype)
