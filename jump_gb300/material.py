"""Material types of jump's explicit step (Material.jl:29-172), host side.

Only the parameters and per-particle state live here; the constitutive
updates themselves (update_stress!, Material.jl:68-275) run in the fused
grid-to-particle kernel.  ``lambda`` is a Python keyword, so the Lame
constant is stored as ``lambda_`` and also reachable as ``getattr(m, "lambda")``.
"""
from __future__ import annotations

import math

import numpy as np

from . import _capi
from .arrays import matrix_array


class MaterialType:
    kind = None
    density = 0.0

    def __getattr__(self, name):
        if name == "lambda":
            return self.lambda_
        raise AttributeError(name)


def _lame(E, nu):
    lam = E * nu / (1 + nu) / (1 - 2 * nu)  # Material.jl:54
    mu = E / 2 / (1 + nu)  # Material.jl:55
    return lam, mu


class RigidMaterial(MaterialType):
    """A rigid solid: RigidMaterial(vx, vy, density) as the reference drivers build it
    (Main_LateralCompressionTube.jl:116-117), with the fields the USL solver reads
    (SolveExplicitSolidMechanics2D.jl:453-461: vx, vy, fixed); vz for 3D.  The
    reference type itself holds only the density (Material.jl:29-31).

    RigidMaterial(vx, vy, density) or RigidMaterial(vx, vy, vz, density), and
    ``fixed=True`` for a body that zeroes every nodal momentum component under it.
    """
    kind = _capi.MPM_MAT_RIGID

    def __init__(self, *args, fixed: bool = False):
        if len(args) == 1:  # RigidMaterial(density), the reference type
            self.vx = self.vy = self.vz = 0.0
            self.density = float(args[0])
        elif len(args) == 3:
            self.vx, self.vy, self.density = (float(a) for a in args)
            self.vz = 0.0
        elif len(args) == 4:
            self.vx, self.vy, self.vz, self.density = (float(a) for a in args)
        else:
            raise TypeError("RigidMaterial(vx, vy[, vz], density) or RigidMaterial(density)")
        self.fixed = bool(fixed)
        self.E = self.nu = 0.0


class ElasticMaterial(MaterialType):
    """ElasticMaterial(E,nu,density,Gf,l,parCount) or ElasticMaterial(E,nu,rho,parCount),
    Material.jl:37-64."""
    kind = _capi.MPM_MAT_ELASTIC

    def __init__(self, E, nu, density, *rest):
        if len(rest) == 3:
            Gf, l0, parCount = rest
        elif len(rest) == 1:
            Gf, l0, parCount = 0.0, 0.0, rest[0]
        else:
            raise TypeError("ElasticMaterial(E,nu,density,Gf,l,parCount) or (E,nu,rho,parCount)")
        self.E, self.nu, self.density = float(E), float(nu), float(density)
        self.lambda_, self.mu = _lame(self.E, self.nu)
        self.Gf, self.l0 = float(Gf), float(l0)
        self.fac = 0.5 / self.E
        self.vmStr = np.zeros(int(parCount))
        self.dam = np.zeros(int(parCount))
        self.c_dil = math.sqrt((self.lambda_ + 2 * self.mu) / self.density)
        self.fy = 0.0
        self.k1 = 0.0


class NeoHookeanMaterial(MaterialType):
    """NeoHookeanMaterial(E,nu,density,parCount), Material.jl:100-117."""
    kind = _capi.MPM_MAT_NEOHOOKEAN

    def __init__(self, E, nu, density, parCount):
        self.E, self.nu, self.density = float(E), float(nu), float(density)
        self.lambda_, self.mu = _lame(self.E, self.nu)
        self.vmStr = np.zeros(int(parCount))
        self.fy = 0.0
        self.k1 = 0.0


class JohnsonCookMaterial(MaterialType):
    """JohnsonCookMaterial(E,nu,density,A,B,C,n,eps0dot,m,chi,Cp,cellsize,parCount),
    Material.jl:279-330; 3D stress update Material.jl:386-443.  State per
    particle: alpha (equivalent plastic strain), alphadot (its filtered rate),
    vmStr.  m, chi and Cp enter no stress update."""
    kind = _capi.MPM_MAT_JOHNSON_COOK

    def __init__(self, E, nu, density, A, B, C, n, eps0dot, m, chi, Cp, cellsize, parCount):
        self.E, self.nu, self.density = float(E), float(nu), float(density)
        self.lambda_, self.mu = _lame(self.E, self.nu)
        self.kappa = self.lambda_ + self.mu
        self.A, self.B, self.C, self.n = float(A), float(B), float(C), float(n)
        self.epsdot0, self.m, self.chi, self.Cp = float(eps0dot), float(m), float(chi), float(Cp)
        self.cellsize = float(cellsize)
        self.signal_velocity = math.sqrt((self.lambda_ + 2 * self.mu) / self.density)
        self.delta = self.chi / (self.density * self.Cp) if self.Cp != 0 else math.inf
        k = int(parCount)
        self.alpha = np.zeros(k)
        self.alphadot = np.zeros(k)
        self.vmStr = np.zeros(k)
        self.fy = 0.0
        self.k1 = 0.0


class VoceMaterial(MaterialType):
    """VoceMaterial(E,nu,density,A,B,C,chi,Cp,cellsize,parCount), Material.jl:336-383;
    3D stress update Material.jl:445-493 (yield A - B exp(-C alpha))."""
    kind = _capi.MPM_MAT_VOCE

    def __init__(self, E, nu, density, A, B, C, chi, Cp, cellsize, parCount):
        self.E, self.nu, self.density = float(E), float(nu), float(density)
        self.lambda_, self.mu = _lame(self.E, self.nu)
        self.kappa = self.lambda_ + self.mu
        self.A, self.B, self.C = float(A), float(B), float(C)
        self.n, self.epsdot0 = 0.0, 0.0
        self.chi, self.Cp, self.cellsize = float(chi), float(Cp), float(cellsize)
        self.signal_velocity = math.sqrt((self.lambda_ + 2 * self.mu) / self.density)
        k = int(parCount)
        self.alpha = np.zeros(k)
        self.alphadot = np.zeros(k)
        self.vmStr = np.zeros(k)
        self.fy = 0.0
        self.k1 = 0.0


class JohnsonCookDamage:
    """JohnsonCookDamage(d1,d2,d3,d4,d5,epsdot0,Tr,Tm,parCount), Material.jl:495-509:
    Johnson-Cook failure strain constants, reference and melting temperatures,
    and the per-particle temperature ``temp`` (starts at Tr)."""

    def __init__(self, d1, d2, d3, d4, d5, epsdot0, Tr, Tm, parCount):
        self.d1, self.d2, self.d3, self.d4, self.d5 = (float(d1), float(d2), float(d3), float(d4), float(d5))
        self.epsdot0, self.Tr, self.Tm = float(epsdot0), float(Tr), float(Tm)
        self.Tmr = self.Tm - self.Tr
        self.temp = np.full(int(parCount), self.Tr)


class JohnsonCookMaterialWithDamage(MaterialType):
    """JohnsonCookMaterialWithDamage(strength, damage), Material.jl:551-564; 3D stress
    update Material.jl:566-646 with compute_damage (:511-549).  State per
    particle: the strength part's alpha, alphadot and vmStr, ``damage_init``,
    ``dam`` and the damage part's ``temp``.  The strength part's constants
    (E, nu, A, B, C, n, ...) are reachable on this object too."""
    kind = _capi.MPM_MAT_JOHNSON_COOK_DAMAGE

    def __init__(self, strength, damage):
        if not isinstance(strength, JohnsonCookMaterial) or not isinstance(damage, JohnsonCookDamage):
            raise TypeError("JohnsonCookMaterialWithDamage(strength::JohnsonCookMaterial, damage::JohnsonCookDamage)")
        self.strength_part = strength
        self.damage_part = damage
        n = len(strength.alpha)
        self.damage_init = np.zeros(n)
        self.dam = np.zeros(n)
        self.density = strength.density

    def __getattr__(self, name):
        if name in ("strength_part", "damage_part"):
            raise AttributeError(name)
        return getattr(self.strength_part, name)


class ElastoPlasticMaterial(MaterialType):
    """J2 plasticity with linear hardening, ElastoPlasticMaterial(E,nu,density,fy,k1,parCount),
    Material.jl:128-171.  State per particle: alpha, pstrain (2D Voigt) and pstrain_3D."""
    kind = _capi.MPM_MAT_J2

    def __init__(self, E, nu, density, fy, k1, parCount):
        self.E, self.nu, self.density = float(E), float(nu), float(density)
        self.lambda_, self.mu = _lame(self.E, self.nu)
        self.kappa = self.lambda_ + self.mu  # Material.jl:161 (kept as in the reference)
        self.fy, self.k1 = float(fy), float(k1)
        n = int(parCount)
        self.pstrain = np.zeros((n, 3))
        self.alpha = np.zeros(n)
        self.vmStr = np.zeros(n)
        self.pstrain_3D = matrix_array(n, 3)
