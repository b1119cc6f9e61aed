"""yaff_gb300 -- GB300-native force evaluation behind yaff's ForceField API.

The hot path of a yaff force evaluation (neighbour list, the pair terms LJ /
MM3 / EI and MM3CAP / Grimme / ExpRep / QMDFFRep / LJCross / DampDisp /
Disp68BJDamp, Ewald reciprocal / correction / neutralizing terms, the valence
chain with every internal-coordinate and energy-term kind) runs as hand-written sm_103a CUDA kernels in libyaffgb.so,
reached through its C ABI (include/yaffgb.h).  The Python classes keep the
reference's constructors and ``compute(gpos, vtens)`` semantics.  Around it:
velocity Verlet on the host or fully device-resident (``verlet``), a
serving loop for many small systems (``serve``) and batched Monte Carlo
trial energies with the reference's structure-factor functions (``mc``).
"""
from .system import Cell, System, SystemView, as_system
from .pair import (Hammer, Switch3, PairPotLJ, PairPotMM3, PairPotEI, PairPotMM3CAP, PairPotGrimme, PairPotExpRep,
                   PairPotQMDFFRep, PairPotLJCross, PairPotDampDisp, PairPotDisp68BJDamp)
from .scaling import Scalings
from .nlist import NeighborList, neigh_dtype
from .valence import (Bond, BendCos, BendAngle, DihedCos, DihedAngle, UreyBradley, OopCos, OopMeanCos, OopAngle,
                      OopMeanAngle, OopDist, SqOopDist, DihedCos2, DihedCos3, DihedCos4, DihedCos6,
                      PointLineDistance, SqPointLineDistance, Harmonic, PolyFour, Fues, Cross, Cosine, Chebychev1,
                      Chebychev2, Chebychev3, Chebychev4, Chebychev6, PolySix, MM3Quartic, MM3Bend,
                      BondDoubleWell, Morse, Poly4)
from .ff import (ForcePart, ForceField, ForcePartPair, ForcePartEwaldReciprocal, ForcePartEwaldCorrection,
                 ForcePartEwaldNeutralizing, ForcePartTailCorrection, ForcePartValence)
from .device import DeviceSystem, device_of, set_default_precision, get_default_precision
from .builder import build_system, build_forcefield
from .verlet import VerletIntegrator, DeviceVerlet, get_random_vel
from .mc import (ForcePartEwaldReciprocalInteraction, MCTrials, compute_ewald_prefactors,
                 compute_ewald_structurefactors, compute_ewald_deltae)
from . import configs, units

__version__ = '0.1.0'
