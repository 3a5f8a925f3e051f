"""Shared test helpers: rebuild a case from a golden fixture, run a context,
compare particle fields."""
from __future__ import annotations

import os

import numpy as np

from jump_gb300 import _capi
from jump_gb300.algorithm import USL, ConstantBodyForce2D, ConstantBodyForce3D
from jump_gb300.engine import Descriptors, colmajor, from_colmajor
from jump_gb300.grid import Grid2D, Grid3D
from jump_gb300.material import (ElasticMaterial, ElastoPlasticMaterial, JohnsonCookDamage, JohnsonCookMaterial,
                                 JohnsonCookMaterialWithDamage, NeoHookeanMaterial, VoceMaterial)
from jump_gb300.solid import Solid2D, Solid3D

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))

FIELDS = ("pos", "velocity", "volume", "F", "strain", "stress", "alpha", "pstrain", "vmstr", "alphadot",
          "damage_init", "damage", "temperature")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = int(z["meta_dim"])
    xmin, xmax, nodes = z["meta_xmin"], z["meta_xmax"], z["meta_nodes"]
    if d == 2:
        grid = Grid2D(xmin[0], xmax[0], xmin[1], xmax[1], nodes[0], nodes[1])
    else:
        grid = Grid3D(xmin[0], xmax[0], xmin[1], xmax[1], xmin[2], xmax[2], nodes[0], nodes[1], nodes[2])
    grid.fixedNodes[:, :] = z["meta_fixed"].T
    solids = []
    for b in range(int(z["meta_nbodies"])):
        typ, E, nu, rho, fy, k1 = z[f"b{b}_mat"]
        pos = z[f"b{b}_in_pos"]
        n = pos.shape[0]
        if int(typ) == _capi.MPM_MAT_ELASTIC:
            mat = ElasticMaterial(E, nu, rho, n)
        elif int(typ) == _capi.MPM_MAT_NEOHOOKEAN:
            mat = NeoHookeanMaterial(E, nu, rho, n)
        elif int(typ) == _capi.MPM_MAT_JOHNSON_COOK:
            A, Bh, Ch, nh, e0, cs = z[f"b{b}_matx"]
            mat = JohnsonCookMaterial(E, nu, rho, A, Bh, Ch, nh, e0, 0.0, 0.0, 0.0, cs, n)
        elif int(typ) == _capi.MPM_MAT_VOCE:
            A, Bh, Ch, nh, e0, cs = z[f"b{b}_matx"]
            mat = VoceMaterial(E, nu, rho, A, Bh, Ch, 0.0, 0.0, cs, n)
        elif int(typ) == _capi.MPM_MAT_JOHNSON_COOK_DAMAGE:
            A, Bh, Ch, nh, e0, cs = z[f"b{b}_matx"]
            m_, chi, Cp, d1, d2, d3, d4, d5, de0, Tr, Tm = z[f"b{b}_matd"]
            mat = JohnsonCookMaterialWithDamage(JohnsonCookMaterial(E, nu, rho, A, Bh, Ch, nh, e0, m_, chi, Cp, cs, n),
                                                JohnsonCookDamage(d1, d2, d3, d4, d5, de0, Tr, Tm, n))
            mat.damage_init[:] = z[f"b{b}_in_dinit"]
            mat.dam[:] = z[f"b{b}_in_dam"]
            mat.damage_part.temp[:] = z[f"b{b}_in_temp"]
        else:
            mat = ElastoPlasticMaterial(E, nu, rho, fy, k1, n)
        s = (Solid2D if d == 2 else Solid3D)(pos, mat)
        s.velocity[:] = z[f"b{b}_in_vel"]
        s.mass[:] = z[f"b{b}_in_mass"]
        s.volume[:] = z[f"b{b}_in_vol"]
        s.volumeInitial[:] = z[f"b{b}_in_vol0"]
        s.deformationGradient[:] = from_colmajor(z[f"b{b}_in_F"].ravel(), n, d)
        s.strain[:] = from_colmajor(z[f"b{b}_in_strain"].ravel(), n, d)
        s.stress[:] = from_colmajor(z[f"b{b}_in_stress"].ravel(), n, d)
        if isinstance(mat, (JohnsonCookMaterial, VoceMaterial, JohnsonCookMaterialWithDamage)):
            mat.alpha[:] = z[f"b{b}_in_alpha"]
            mat.alphadot[:] = z[f"b{b}_in_alphadot"]
        if isinstance(mat, ElastoPlasticMaterial):
            mat.alpha[:] = z[f"b{b}_in_alpha"]
            if d == 2:
                mat.pstrain[:] = z[f"b{b}_in_ep"]
            else:
                mat.pstrain_3D[:] = from_colmajor(z[f"b{b}_in_ep"].ravel(), n, 3)
        if f"b{b}_in_youngs" in z:
            s.youngs = z[f"b{b}_in_youngs"].copy()
        solids.append(s)
    g = z["meta_gravity"]
    bf = ConstantBodyForce2D(g[:2]) if d == 2 else ConstantBodyForce3D(g)
    return grid, solids, float(z["meta_tol"]), bf, float(z["meta_dt"]), int(z["meta_nsteps"]), z


def golden_kw(z):
    """Descriptor arguments of a fixture's update scheme and basis (USL and the
    linear basis when it names none)."""
    kw = {}
    if "meta_alg" in z and int(z["meta_alg"]) == 1:
        kw.update(algorithm="musl", alpha=float(z["meta_alpha"]))
    if "meta_basis" in z and int(z["meta_basis"]) != 0:
        kw["basis"] = ("linear", "quad", "cubic")[int(z["meta_basis"])]
    return kw


def golden_expected(z, b):
    """Expected outputs of body b in the download layout."""
    d = int(z["meta_dim"])
    out = {
        "pos": z[f"b{b}_out_pos"], "velocity": z[f"b{b}_out_vel"], "volume": z[f"b{b}_out_vol"],
        "F": z[f"b{b}_out_F"].ravel(), "strain": z[f"b{b}_out_strain"].ravel(),
        "stress": z[f"b{b}_out_stress"].ravel(), "alpha": z[f"b{b}_out_alpha"],
        "pstrain": z[f"b{b}_out_ep"].ravel(), "vmstr": z[f"b{b}_out_vm"],
    }
    if f"b{b}_out_alphadot" in z:
        out["alphadot"] = z[f"b{b}_out_alphadot"]
    if f"b{b}_out_dinit" in z:
        out["damage_init"] = z[f"b{b}_out_dinit"]
        out["damage"] = z[f"b{b}_out_dam"]
        out["temperature"] = z[f"b{b}_out_temp"]
    return out


def descriptors(grid, solids, tol, bf, dt, **kw):
    return Descriptors(grid, solids, tolerance=tol, body_force=bf, dt=dt, **kw)


def rel_err(a, b):
    """max |a - b| / max |b| over a field (0 when both are identically 0)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if b.size else 0.0
    if den == 0.0:
        return float(num)
    return float(num / den)


def field_errors(states_a, states_b, fields=FIELDS):
    errs = {}
    for s, (A, B) in enumerate(zip(states_a, states_b)):
        for f in fields:
            errs[(s, f)] = rel_err(getattr(A, f), getattr(B, f))
    return errs


# Per-particle metric: |a_p - b_p| / max(|b_p|, floor_f) per particle entry, with
# the absolute floor of field f a stated fraction of that field's scale (its
# largest magnitude, over the states compared or a given set of states).  Values
# smaller than the floor are compared at the floor's level: a particle whose
# component is zero by symmetry, or rounding noise of a rigidly moving body,
# would otherwise divide noise by noise.
PP_FLOOR = 1e-3


def field_scales(states, fields=FIELDS):
    return {f: max((float(np.max(np.abs(getattr(s, f)))) if getattr(s, f).size else 0.0) for s in states)
            for f in fields}


def particle_errors(states_a, states_b, fields=FIELDS, floor=PP_FLOOR, scales=None):
    """{field: max per-particle error} over all bodies, floor_f = floor * scale_f."""
    sc = scales or field_scales(states_b, fields)
    out = {}
    for f in fields:
        worst = 0.0
        fl = floor * sc[f]
        for A, B in zip(states_a, states_b):
            a = np.asarray(getattr(A, f), dtype=np.float64).ravel()
            b = np.asarray(getattr(B, f), dtype=np.float64).ravel()
            if b.size == 0:
                continue
            d = np.abs(a - b)
            den = np.maximum(np.abs(b), fl)
            with np.errstate(divide="ignore", invalid="ignore"):
                r = np.where(den > 0, d / den, np.where(d > 0, np.inf, 0.0))
            worst = max(worst, float(np.max(r)))
        out[f] = worst
    return out


def scaled_field_errors(states_a, states_b, fields=FIELDS, scales=None):
    """{field: max |a - b| / scale_f} over all bodies (the field-max metric with a
    shared scale, e.g. an ensemble's)."""
    sc = scales or field_scales(states_b, fields)
    out = {}
    for f in fields:
        num = max((float(np.max(np.abs(np.asarray(getattr(A, f)) - np.asarray(getattr(B, f)))))
                   if getattr(B, f).size else 0.0) for A, B in zip(states_a, states_b))
        out[f] = num / sc[f] if sc[f] > 0 else num
    return out

