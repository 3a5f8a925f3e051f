"""jump_gb300: GB300-native (sm_103a) explicit MPM step (USL, linear hat basis)
behind the solver surface of jump (vinhphunguyen/jump).

The public names mirror the reference's modules: Grid (Grid2D, Grid3D),
Solid (Solid2D, Solid3D, particle generators), Material (ElasticMaterial,
NeoHookeanMaterial, ElastoPlasticMaterial), Algorithm (USL), Basis
(LinearBasis), BodyForce (ConstantBodyForce2D/3D), Fix (EmptyFix,
EnergiesFix, DisplacementFix), Output (OvitoOutput) and Problem
(solve_explicit_dynamics_2D/3D).  The compute path is libjumpmpm.so
(C ABI in include/jump_mpm.h); there is no CPU fallback.
"""
from .algorithm import (USL, MUSL, LinearBasis, QuadBsplineBasis, CubicBsplineBasis,
                        ConstantBodyForce2D, ConstantBodyForce3D)
from .grid import Grid2D, Grid3D, to_1D_index
from .material import (ElasticMaterial, NeoHookeanMaterial, ElastoPlasticMaterial, JohnsonCookMaterial,
                       VoceMaterial, RigidMaterial, JohnsonCookDamage, JohnsonCookMaterialWithDamage)
from .solid import (Solid2D, Solid3D, assign_velocity, move, julia_range, buildParticleForCircle,
                    buildParticleForRing, buildParticleForSphere, buildParticleForCylinder,
                    buildParticleForRectangle, buildParticleForBlock)
from .fix import EmptyFix, EnergiesFix, DisplacementFix, compute, closeFile
from .output import EmptyOutput, OvitoOutput, plotParticles_2D, plotParticles_3D
from .dirichlet import fix_Dirichlet_grid
from .problem import solve_explicit_dynamics_2D, solve_explicit_dynamics_3D
from .engine import Descriptors, MPMContext
from ._capi import MPMError

__all__ = [n for n in dir() if not n.startswith("_")]
