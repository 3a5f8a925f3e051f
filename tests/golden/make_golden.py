"""Generate the golden fixtures of tests/golden/*.npz.

An independent pure-Python restatement of jump's USL step, written line by
line from the Julia source with Python floats (IEEE binary64, each operation
rounded, no fused multiply-add), run on small seeded cases.  The C++ oracle
must reproduce these outputs bit for bit; the CUDA path is then compared with
the oracle.  Neither restatement can be checked against the Julia reference
itself (no Julia toolchain exists where this project builds and runs).

Followed statements (paths relative to the reference repository):
  SolveExplicitSolidMechanics2D.jl:381-534   reset, P2G, grid update, G2P
  Basis.jl:63-78, 104-137, 219-251, 292-332  node lookup and hat functions
  Material.jl:68-81, 119-122, 174-275        update_stress!
  Grid.jl:104-154, 198-264                   node coordinates
3D uses the 2D USL statements with three components (the reference's 3D USL
reads undefined variables); J2 stress is computed as the math of
Material.jl:174-275 and returned.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))


def sign(x):
    return 1.0 if x > 0 else (-1.0 if x < 0 else 0.0)


def quad_bs(t, r):
    """Bsplines.jl:18-80: modified quadratic B-spline of type t, value and d/dr."""
    if t == 1:
        if r < -1.5 or r > 1.5:
            return 0.0, 0.0
        if -1.5 <= r <= -0.5:
            return 0.5 * r * r + 1.5 * r + 1.125, r + 1.5
        if r <= 0.0:
            return 1.0 + r, 1.0
        if r <= 0.5:
            return 1.0 - r, -1.0
        return 0.5 * r * r - 1.5 * r + 1.125, r - 1.5
    if t == 2:
        if r < -1.0 or r > 1.5:
            return 0.0, 0.0
        if -1.0 <= r <= -0.5:
            return 1.0 + r, 1.0
        if r <= 0.5:
            return -r * r + 0.75, -2 * r
        return 0.5 * r * r - 1.5 * r + 1.125, r - 1.5
    if t == 3:
        if r < -1.5 or r > 1.5:
            return 0.0, 0.0
        if -1.5 <= r <= -0.5:
            return 0.5 * r * r + 1.5 * r + 1.125, r + 1.5
        if r <= 0.5:
            return -r * r + 0.75, -2 * r
        return 0.5 * r * r - 1.5 * r + 1.125, r - 1.5
    if r < -1.5 or r > 1.0:
        return 0.0, 0.0
    if -1.5 <= r <= -0.5:
        return 0.5 * r * r + 1.5 * r + 1.125, r + 1.5
    if r <= 0.5:
        return -r * r + 0.75, -2 * r
    return 1.0 - r, -1.0


def cubic_bs(t, r):
    """Bsplines.jl:86-172: modified cubic B-spline of type t, value and d/dr."""
    r2 = r * r
    if t == 1:
        if r < -2.0 or r > 2.0:
            return 0.0, 0.0
        if -2.0 <= r <= -1.0:
            return 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333, 0.5 * r2 + 2 * r + 2.0
        if -1 <= r <= 0.0:
            return -0.16666666666666666 * r * r2 + r + 1, -0.5 * r2 + 1.0
        if 0 <= r <= 1.0:
            return 0.16666666666666666 * r * r2 - r + 1, 0.5 * r2 - 1.0
        return -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333, -0.5 * r2 + 2 * r - 2.0
    if t == 2:
        if r < -1.0 or r > 2.0:
            return 0.0, 0.0
        if -1.0 <= r <= 0.0:
            return -0.3333333333333333 * r * r2 - r2 + 0.6666666666666666, -r2 - 2 * r
        if 0.0 <= r <= 1.0:
            return 0.5 * r * r2 - r2 + 0.6666666666666666, 1.5 * r2 - 2 * r
        if 1 <= r <= 2.0:
            return -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333, -0.5 * r2 + 2 * r - 2
        return 0.0, 0.0
    if t == 3:
        if r < -2.0 or r > 2.0:
            return 0.0, 0.0
        if -2.0 <= r <= -1.0:
            return 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333, 0.5 * r2 + 2 * r + 2
        if -1.0 <= r <= 0.0:
            return -0.5 * r * r2 - r2 + 0.6666666666666666, -1.5 * r2 - 2 * r
        if 0 <= r <= 1.0:
            return 0.5 * r * r2 - r2 + 0.6666666666666666, 1.5 * r2 - 2 * r
        if 1.0 <= r <= 2.0:
            return -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333, -0.5 * r2 + 2 * r - 2
        return 0.0, 0.0
    if r < -2.0 or r > 1.0:
        return 0.0, 0.0
    if -2.0 <= r <= -1.0:
        return 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333, 0.5 * r2 + 2 * r + 2
    if -1.0 <= r <= 0.0:
        return -0.5 * r * r2 - r2 + 0.6666666666666666, -1.5 * r2 - 2 * r
    if 0 <= r <= 1.0:
        return 0.3333333333333333 * r * r2 - r2 + 0.6666666667, r2 - 2 * r
    return 0.0, 0.0


class PyGrid:
    def __init__(self, dim, xmin, xmax, nodes, basis=0):
        self.basis = basis  # 0 linear, 1 quadratic B-spline, 2 cubic B-spline
        self.dim = dim
        self.xmin = list(xmin)
        self.n = list(nodes)
        self.dx = [(xmax[a] - xmin[a]) / (float(nodes[a]) - 1.0) for a in range(dim)]
        self.dxI = [1.0 / self.dx[a] for a in range(dim)]
        self.nxy = nodes[0] * nodes[1]
        self.count = self.nxy * (nodes[2] if dim == 3 else 1)
        self.pos = []
        for k in range(nodes[2] if dim == 3 else 1):
            for j in range(nodes[1]):
                for i in range(nodes[0]):
                    x = float(i) * self.dx[0]
                    y = float(j) * self.dx[1]
                    if dim == 2:
                        self.pos.append((self.xmin[0] + x, self.xmin[1] + y))
                    else:
                        z = float(k) * self.dx[2]
                        self.pos.append((self.xmin[0] + x, self.xmin[1] + y, self.xmin[2] + z))

    def shape(self, xp):
        """getShapeAndGradient: (nearPoints 0-based, funcs, ders)."""
        if self.basis:
            return self.bspline_shape(xp)
        idx = []
        for a in range(self.dim):
            idx.append(math.floor((xp[a] - self.xmin[a]) * self.dxI[a] + 1.0))
        if self.dim == 2:
            I = self.n[0] * (idx[1] - 1) + idx[0]
            near = [I, I + 1, I + self.n[0], I + 1 + self.n[0]]
        else:
            I = self.nxy * (idx[2] - 1) + self.n[0] * (idx[1] - 1) + idx[0]
            nx, nxy = self.n[0], self.nxy
            near = [I, I + 1, I + nx, I + nx + 1, I + nxy, I + 1 + nxy, I + nx + nxy, I + nx + 1 + nxy]
        near = [q - 1 for q in near]
        funcs, ders = [], []
        for q in near:
            xi = self.pos[q]
            if self.dim == 2:
                xip = xp[0] - xi[0]
                yip = xp[1] - xi[1]
                Nx = 1.0 - abs(xip) * self.dxI[0]
                Ny = 1.0 - abs(yip) * self.dxI[1]
                funcs.append(Nx * Ny)
                ders.append((-Ny * sign(xip) * self.dxI[0], -Nx * sign(yip) * self.dxI[1]))
            else:
                xip = xp[0] - xi[0]
                yip = xp[1] - xi[1]
                zip_ = xp[2] - xi[2]
                Nx = 1.0 - abs(xip) * self.dxI[0]
                Ny = 1.0 - abs(yip) * self.dxI[1]
                Nz = 1.0 - abs(zip_) * self.dxI[2]
                funcs.append(Nx * Ny * Nz)
                ders.append((-Ny * Nz * sign(xip) * self.dxI[0],
                             -Nx * Nz * sign(yip) * self.dxI[1],
                             -Nx * Ny * sign(zip_) * self.dxI[2]))
        return near, funcs, ders

    def bspline_shape(self, xp):
        """Basis.jl:374-820: near nodes per axis (1-based ids), boundary-typed 1D
        B-splines, tensor product in the reference's i, j(, k) loop order.  The
        3D quadratic basis measures x from the origin; y and z are measured
        from (id-1)*dy and (id-1)*dz for both bases."""
        d, K = self.dim, (3 if self.basis == 1 else 4)
        fn = quad_bs if K == 3 else cubic_bs
        per_axis = []
        for a in range(d):
            n = self.n[a]
            num = xp[a] * self.dxI[a] if (K == 3 and d == 3) else (xp[a] - self.xmin[a]) * self.dxI[a]
            rem = num - math.floor(num)
            ib = math.floor(num + 1.0)
            if K == 3:
                if ib == 1:
                    ids = [ib, ib + 1, ib + 2]
                elif ib == n - 1:
                    ids = [ib - 1, ib, ib + 1]
                elif rem < 0.5:
                    ids = [ib - 1, ib, ib + 1]
                else:
                    ids = [ib, ib + 1, ib + 2]
            else:
                if ib == 1:
                    ids = [1, 2, 3, 4]
                elif ib == n - 1:
                    ids = [ib - 2, ib - 1, ib, ib + 1]
                else:
                    ids = [ib - 1, ib, ib + 1, ib + 2]
            vals = []
            for i in ids:
                if a == 0:
                    r = (xp[0] - self.pos[i - 1][0]) * self.dxI[0]
                else:
                    r = (xp[a] - (i - 1) * self.dx[a]) * self.dxI[a]
                t = 1 if (i == 1 or i == n) else (2 if i == 2 else (4 if i == n - 1 else 3))
                vals.append(fn(t, r))
            per_axis.append((ids, vals))
        near, funcs, ders = [], [], []
        (ix, vx), (iy, vy) = per_axis[0], per_axis[1]
        for i in range(K):
            Nx, dNx = vx[i]
            for j in range(K):
                Ny, dNy = vy[j]
                if d == 2:
                    near.append(self.n[0] * (iy[j] - 1) + ix[i] - 1)
                    funcs.append(Nx * Ny)
                    ders.append((dNx * self.dxI[0] * Ny, dNy * self.dxI[1] * Nx))
                else:
                    iz, vz = per_axis[2]
                    for k in range(K):
                        Nz, dNz = vz[k]
                        near.append(self.nxy * (iz[k] - 1) + self.n[0] * (iy[j] - 1) + ix[i] - 1)
                        funcs.append(Nx * Ny * Nz)
                        ders.append((dNx * self.dxI[0] * Ny * Nz, dNy * self.dxI[1] * Nx * Nz,
                                     dNz * self.dxI[2] * Nx * Ny))
        return near, funcs, ders


def mat_get(M, i, j, d):
    return M[i + d * j]  # column-major, 0-based


def matmul(A, B, d):
    C = [0.0] * (d * d)
    for j in range(d):
        for i in range(d):
            s = A[i] * B[d * j]
            for k in range(1, d):
                s = s + A[i + d * k] * B[k + d * j]
            C[i + d * j] = s
    return C


def det(A, d):
    if d == 2:
        return A[0] * A[3] - A[2] * A[1]
    x0, x1, x2 = A[0:3], A[3:6], A[6:9]
    cr = (x1[1] * x2[2] - x1[2] * x2[1], x1[2] * x2[0] - x1[0] * x2[2], x1[0] * x2[1] - x1[1] * x2[0])
    return x0[0] * cr[0] + x0[1] * cr[1] + x0[2] * cr[2]


def jc_failure(mat, damage_init, damage, pH, Sdev, epsdot, dp, T):
    """compute_damage, Material.jl:511-549: (damage_init, damage) after a plastic
    strain increment dp."""
    vm = 1.224744871 * math.sqrt(Sdev[0] * Sdev[0] + Sdev[4] * Sdev[4] + Sdev[8] * Sdev[8] +
                                 2 * (Sdev[3] * Sdev[3] + Sdev[6] * Sdev[6] + Sdev[7] * Sdev[7]))
    triax = 0.0
    if pH != 0.0 and vm != 0.0:
        triax = -pH / (vm + 0.01 * abs(pH))
    if triax > 3.0:
        triax = 3.0
    fs = mat["d1"] + mat["d2"] * math.exp(mat["d3"] * triax)
    if mat["d4"] > 0.0 and epsdot > mat["depsdot0"]:
        fs *= (1.0 + mat["d4"] * math.log(epsdot / mat["depsdot0"]))
    if mat["d5"] > 0.0 and T >= mat["Tr"]:
        fs *= 1. + mat["d5"] * (T - mat["Tr"]) / (mat["Tm"] - mat["Tr"])
    damage_init += dp / fs
    if damage_init >= 1.0:
        damage = min((damage_init - 1.0) * 10, 1.0)
    return damage_init, damage


def jc_damage_stress(mat, sig, eps, state):
    """update_stress! of JohnsonCookMaterialWithDamage, Material.jl:566-646, on the
    fields the method means (damage_part, strength_part), returning the stress."""
    lam, mu, kappa = mat["lambda"], mat["mu"], mat["kappa"]
    damage = state["dam"]
    if damage >= 1.0:
        pH = kappa * (eps[0] + eps[4] + eps[8])
        return [pH, 0.0, 0.0, 0.0, pH, 0.0, 0.0, 0.0, pH]
    ep = state["alpha"]
    ratio = max(state["alphadot"] / mat["epsdot0"], 1.0)
    T = state["temp"]
    if ep < 1.0e-10:
        ys = mat["A"]
    elif T < mat["Tm"]:
        if mat["C"] != 0:
            ys = (mat["A"] + mat["B"] * ep ** mat["n"]) * (1.0 + ratio) ** mat["C"]
        else:
            ys = mat["A"] + mat["B"] * ep ** mat["n"]
        if mat["m"] != 0 and T >= mat["Tr"]:
            ys *= 1.0 - ((T - mat["Tr"]) / (mat["Tm"] - mat["Tr"])) ** mat["m"]
    else:
        ys = 0.
    Gd = mu
    if damage > 0:
        Gd *= (1 - damage)
        ys *= (1 - damage)
    trial = [sig[k] + 2.0 * Gd * state["deps"][k] for k in range(9)]
    third = 0.333333333 * (trial[0] + trial[4] + trial[8])
    dev = list(trial)
    for k in (0, 4, 8):
        dev[k] = trial[k] - third
    J2 = 1.224744871391589 * math.sqrt(dev[0] * dev[0] + dev[4] * dev[4] + dev[8] * dev[8] +
                                       2 * (dev[3] * dev[3] + dev[6] * dev[6] + dev[7] * dev[7]))
    if J2 < ys:
        dp = 0.0
    else:
        dp = (J2 - ys) / (3.0 * Gd)
        dev = [x * (ys / J2) for x in dev]
    state["alpha"] = ep + dp
    pH = kappa * (eps[0] + eps[4] + eps[8])
    out = list(dev)
    for k in (0, 4, 8):
        out[k] = dev[k] + pH
    tav = 1000 * mat["cellsize"] / math.sqrt((lam + 2 * mu) / mat["density"])
    ad = state["alphadot"]
    ad -= ad * state["dt"] / tav
    ad += dp / tav
    state["alphadot"] = max(0.0, ad)
    flow = 1.224744871391589 * math.sqrt(dev[0] * dev[0] + dev[4] * dev[4] + dev[8] * dev[8] +
                                         2 * (dev[3] * dev[3] + dev[6] * dev[6] + dev[7] * dev[7]))
    state["vm"] = flow
    state["dinit"], state["dam"] = jc_failure(mat, state["dinit"], state["dam"], pH, dev, state["alphadot"], dp, T)
    T += mat["chi"] / (mat["density"] * mat["Cp"]) * flow * dp
    state["temp"] = T
    return out


def stress_update(mat, d, sig, eps, F, J, state):
    """update_stress! for one particle; returns the new stress (column-major).
    state carries alpha, ep, vm and, for Johnson-Cook/Voce, alphadot, the strain
    increment deps = dt D and dt."""
    typ, lam, mu = mat["type"], mat["lambda"], mat["mu"]
    if typ == 5:  # JohnsonCookMaterialWithDamage (3D)
        return jc_damage_stress(mat, sig, eps, state)
    if typ in (3, 4):  # JohnsonCookMaterial / VoceMaterial, Material.jl:386-493 (3D)
        ep = state["alpha"]
        if ep < 1.0e-10:
            yieldStress = mat["A"]
        elif typ == 3:
            ratio = max(state["alphadot"] / mat["epsdot0"], 1.0)
            if mat["C"] != 0:
                yieldStress = (mat["A"] + mat["B"] * ep ** mat["n"]) * (1.0 + ratio) ** mat["C"]
            else:
                yieldStress = mat["A"] + mat["B"] * ep ** mat["n"]
        else:
            yieldStress = mat["A"] - mat["B"] * math.exp(-mat["C"] * ep)
        Gd = mu
        trial = [sig[k] + 2.0 * Gd * state["deps"][k] for k in range(9)]
        third = 0.333333333 * (trial[0] + trial[4] + trial[8])
        dev = list(trial)
        for k in (0, 4, 8):
            dev[k] = trial[k] - third
        J2 = 1.224744871391589 * math.sqrt(dev[0] * dev[0] + dev[4] * dev[4] + dev[8] * dev[8] +
                                           2 * (dev[3] * dev[3] + dev[6] * dev[6] + dev[7] * dev[7]))
        dp = 0.0
        if not (J2 < yieldStress):
            dp = (J2 - yieldStress) / (3.0 * Gd)
            dev = [x * (yieldStress / J2) for x in dev]
        state["alpha"] = ep + dp
        tav = 1000 * mat["cellsize"] / math.sqrt((lam + 2 * mu) / mat["density"])
        ad = state["alphadot"]
        ad -= ad * state["dt"] / tav
        ad += dp / tav
        state["alphadot"] = max(0.0, ad)
        state["vm"] = math.sqrt(dev[0] * dev[0] + dev[4] * dev[4] + dev[8] * dev[8] +
                                2 * (dev[3] * dev[3] + dev[6] * dev[6] + dev[7] * dev[7]))
        p = mat["kappa"] * (eps[0] + eps[4] + eps[8])
        out = list(dev)
        for k in (0, 4, 8):
            out[k] = dev[k] + p
        return out
    if typ == 0:  # ElasticMaterial
        if d == 3:
            s = sig
            state["vm"] = math.sqrt(s[0] * s[0] + s[4] * s[4] + s[8] * s[8] + 2 * (s[3] * s[3] + s[6] * s[6] + s[7] * s[7]))
            tr = eps[0] + eps[4] + eps[8]
        else:
            tr = eps[0] + eps[3]
        out = []
        for j in range(d):
            for i in range(d):
                v = 2.0 * mu * eps[i + d * j]
                if i == j:
                    v = lam * tr * 1.0 + v
                out.append(v)
        return [out[i] for i in range(d * d)]
    if typ == 1:  # NeoHookeanMaterial
        FFt = [0.0] * (d * d)
        for j in range(d):
            for i in range(d):
                s = F[i] * F[j]
                for k in range(1, d):
                    s = s + F[i + d * k] * F[j + d * k]
                FFt[i + d * j] = s
        out = [0.0] * (d * d)
        ll = lam * math.log(J) * 1.0
        for j in range(d):
            for i in range(d):
                a = FFt[i + d * j] - (1.0 if i == j else 0.0) if i == j else FFt[i + d * j]
                v = mu * a
                if i == j:
                    v = v + ll
                out[i + d * j] = (1.0 / J) * v
        return out
    # ElastoPlasticMaterial
    k1, fy, kappa = mat["k1"], mat["fy"], mat["kappa"]
    if d == 3:
        ep = state["ep"]  # 9, column-major
        a0 = state["alpha"]
        t3 = 0.333333333 * (eps[0] + eps[4] + eps[8])
        ed = list(eps)
        for c in (0, 4, 8):
            ed[c] = ed[c] - t3
        s = [2 * mu * (ed[c] - ep[c]) for c in range(9)]
        ns = math.sqrt(s[0] * s[0] + s[4] * s[4] + s[8] * s[8] + 2.0 * (s[3] * s[3] + s[7] * s[7] + s[6] * s[6]))
        kt = kappa * (eps[0] + eps[4] + eps[8]) * 1.0
        st = list(s)
        for c in (0, 4, 8):
            st[c] = kt + st[c]
        f_trial = ns - (k1 * a0 + fy)
        if f_trial <= 0.0:
            sg = st
        else:
            nrm = [(1.0 / ns) * s[c] for c in range(9)]
            lamp = (ns - k1 * a0 - fy) / (2 * mu + k1)
            a0 += lamp
            ep = [ep[c] + lamp * nrm[c] for c in range(9)]
            sg = [st[c] - 2 * mu * lamp * nrm[c] for c in range(9)]
        state["alpha"], state["ep"] = a0, ep
        t3 = 0.333333333 * (sg[0] + sg[4] + sg[8])
        dv = list(sg)
        for c in (0, 4, 8):
            dv[c] = dv[c] - t3
        state["vm"] = math.sqrt(dv[0] * dv[0] + dv[4] * dv[4] + dv[8] * dv[8] + 2 * (dv[3] * dv[3] + dv[6] * dv[6] + dv[7] * dv[7]))
        return sg
    # 2D J2, Voigt
    Idev = [[0.5, -0.5, 0.0], [-0.5, 0.5, 0.0], [0.0, 0.0, 1.0]]
    Im = [[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 0.5]]
    Iinv = [[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 2.0]]
    ep = state["ep"]  # 3
    a0 = state["alpha"]
    e = [mat_get(eps, 0, 0, 2), mat_get(eps, 1, 1, 2), 2 * mat_get(eps, 0, 1, 2)]
    edv = [Idev[i][0] * e[0] + Idev[i][1] * e[1] + Idev[i][2] * e[2] for i in range(3)]
    a = [2 * mu * (edv[i] - ep[i]) for i in range(3)]
    s = [Im[i][0] * a[0] + Im[i][1] * a[1] + Im[i][2] * a[2] for i in range(3)]
    ns = math.sqrt(s[0] * s[0] + s[1] * s[1] + 2 * s[2] * s[2])
    eye2 = [1.0, 1.0, 0.0]
    kt = kappa * (e[0] + e[1])
    f_trial = ns - (k1 * a0 + fy)
    if f_trial <= 0.0:
        sg = [kt * eye2[i] + s[i] for i in range(3)]
    else:
        nrm = [(1.0 / ns) * s[i] for i in range(3)]
        lamp = (ns - k1 * a0 - fy) / (2 * mu + k1)
        a0 += lamp
        q = [Iinv[i][0] * nrm[0] + Iinv[i][1] * nrm[1] + Iinv[i][2] * nrm[2] for i in range(3)]
        ep = [ep[i] + lamp * q[i] for i in range(3)]
        sg = [kt * eye2[i] + s[i] - 2 * mu * lamp * nrm[i] for i in range(3)]
    state["alpha"], state["ep"] = a0, ep
    dv = [Idev[i][0] * sg[0] + Idev[i][1] * sg[1] + Idev[i][2] * sg[2] for i in range(3)]
    state["vm"] = math.sqrt(dv[0] * dv[0] + dv[1] * dv[1] + 2 * dv[2] * dv[2])
    return [sg[0], sg[2], sg[2], sg[1]]


def usl_steps(case, nsteps):
    """Run nsteps of the USL loop on a case dict (lists of floats); mutates it."""
    d = case["dim"]
    G = PyGrid(d, case["xmin"], case["xmax"], case["nodes"], case.get("basis", 0))
    fixed = case["fixed"]  # list of d-tuples per node
    dt, tol, body = case["dt"], case["tol"], case["gravity"][:d]
    for _ in range(nsteps):
        mass = [0.0] * G.count
        mom0 = [[0.0] * d for _ in range(G.count)]
        force = [[0.0] * d for _ in range(G.count)]
        for B in case["bodies"]:
            for ip in range(B["n"]):
                near, funcs, ders = G.shape(B["pos"][ip])
                fVolume, fMass, vp, sigma = B["vol"][ip], B["mass"][ip], B["vel"][ip], B["stress"][ip]
                for i in range(len(near)):
                    q, Ni, dNi = near[i], funcs[i], ders[i]
                    Nim = Ni * fMass
                    mass[q] += Nim
                    for a in range(d):
                        mom0[q][a] += Nim * vp[a]
                    for a in range(d):
                        s = sigma[a] * dNi[0] + sigma[a + d] * dNi[1]
                        if d == 3:
                            s = s + sigma[a + 2 * d] * dNi[2]
                        force[q][a] += -fVolume * s + fMass * body[a] * Ni
        mom = [[0.0] * d for _ in range(G.count)]
        for i in range(G.count):
            for a in range(d):
                mom[i][a] = mom0[i][a] + force[i][a] * dt
            for a in range(d):
                if fixed[i][a] == 1:
                    mom0[i][a] = 0.0
                    mom[i][a] = 0.0
        for B in case["bodies"]:
            mat = B["mat"]
            for ip in range(B["n"]):
                near, funcs, ders = G.shape(B["pos"][ip])
                L = [0.0] * (d * d)
                vvp = list(B["vel"][ip])
                xxp = list(B["pos"][ip])
                for i in range(len(near)):
                    q, Ni, dNi = near[i], funcs[i], ders[i]
                    mI = mass[q]
                    if mI > tol:
                        invM = 1.0 / mI
                        vI = [mom[q][a] * invM for a in range(d)]
                        for a in range(d):
                            vvp[a] += Ni * (mom[q][a] - mom0[q][a]) * invM
                        for a in range(d):
                            xxp[a] += Ni * vI[a] * dt
                        for j in range(d):
                            for a in range(d):
                                L[a + d * j] += dNi[j] * vI[a]
                B["vel"][ip] = vvp
                B["pos"][ip] = xxp
                D_ = [0.5 * (L[i + d * j] + L[j + d * i]) for j in range(d) for i in range(d)]
                B["strain"][ip] = [B["strain"][ip][c] + dt * D_[c] for c in range(d * d)]
                A = [L[c] * dt for c in range(d * d)]
                for a in range(d):
                    A[a * (d + 1)] = A[a * (d + 1)] + 1.0
                F = matmul(B["F"][ip], A, d)
                B["F"][ip] = F
                J = det(F, d)
                B["vol"][ip] = J * B["vol0"][ip]
                lam, mu = mat["lambda"], mat["mu"]
                m2 = dict(mat)
                if B.get("youngs") is not None:
                    E, nu = B["youngs"][ip], mat["nu"]
                    m2["lambda"] = E * nu / (1 + nu) / (1 - 2 * nu)
                    m2["mu"] = E / 2 / (1 + nu)
                    m2["kappa"] = m2["lambda"] + m2["mu"]
                state = {"alpha": B["alpha"][ip], "ep": B["ep"][ip], "vm": B["vm"][ip],
                         "alphadot": B["alphadot"][ip], "deps": [dt * x for x in D_], "dt": dt,
                         "dinit": B["dinit"][ip], "dam": B["dam"][ip], "temp": B["temp"][ip]}
                B["stress"][ip] = stress_update(m2, d, B["stress"][ip], B["strain"][ip], F, J, state)
                B["alpha"][ip], B["ep"][ip], B["vm"][ip] = state["alpha"], state["ep"], state["vm"]
                B["alphadot"][ip] = state["alphadot"]
                B["dinit"][ip], B["dam"][ip], B["temp"][ip] = state["dinit"], state["dam"], state["temp"]
    case["grid_out"] = (mass, mom0, mom, force)
    return case


def _kinematics(B, ip, L, d, dt):
    """strain += dt D, F *= (I + L dt), J, V, update_stress! (shared by the USL and MUSL loops)."""
    mat = B["mat"]
    D_ = [0.5 * (L[i + d * j] + L[j + d * i]) for j in range(d) for i in range(d)]
    B["strain"][ip] = [B["strain"][ip][c] + dt * D_[c] for c in range(d * d)]
    A = [L[c] * dt for c in range(d * d)]
    for a in range(d):
        A[a * (d + 1)] = A[a * (d + 1)] + 1.0
    F = matmul(B["F"][ip], A, d)
    B["F"][ip] = F
    J = det(F, d)
    B["vol"][ip] = J * B["vol0"][ip]
    m2 = dict(mat)
    if B.get("youngs") is not None:
        E, nu = B["youngs"][ip], mat["nu"]
        m2["lambda"] = E * nu / (1 + nu) / (1 - 2 * nu)
        m2["mu"] = E / 2 / (1 + nu)
        m2["kappa"] = m2["lambda"] + m2["mu"]
    state = {"alpha": B["alpha"][ip], "ep": B["ep"][ip], "vm": B["vm"][ip],
             "alphadot": B["alphadot"][ip], "deps": [dt * x for x in D_], "dt": dt,
             "dinit": B["dinit"][ip], "dam": B["dam"][ip], "temp": B["temp"][ip]}
    B["stress"][ip] = stress_update(m2, d, B["stress"][ip], B["strain"][ip], F, J, state)
    B["alpha"][ip], B["ep"][ip], B["vm"][ip] = state["alpha"], state["ep"], state["vm"]
    B["alphadot"][ip] = state["alphadot"]
    B["dinit"][ip], B["dam"][ip], B["temp"][ip] = state["dinit"], state["dam"], state["temp"]


def _cholesky_solve_band(A, n, w, rhs):
    """Solve A x = rhs for the symmetric positive definite A given by its lower
    band A[i][k] = A_{i,i-k}, k = 0..w: Cholesky A = L L^T (columns in ascending
    order, so the entries outside the band, all zero, never enter a sum), then
    forward and backward substitution."""
    Lb = [row[:] for row in A]
    for i in range(n):
        for j in range(max(0, i - w), i + 1):
            acc = Lb[i][i - j]
            for k in range(max(0, i - w, j - w), j):
                acc -= Lb[i][i - k] * Lb[j][j - k]
            if i == j:
                Lb[i][0] = math.sqrt(acc)
            else:
                Lb[i][i - j] = acc / Lb[j][0]
    out = []
    for b in rhs:
        y = [0.0] * n
        for i in range(n):
            acc = b[i]
            for k in range(max(0, i - w), i):
                acc -= Lb[i][i - k] * y[k]
            y[i] = acc / Lb[i][0]
        x = [0.0] * n
        for i in range(n - 1, -1, -1):
            acc = y[i]
            for k in range(i + 1, min(n - 1, i + w) + 1):
                acc -= Lb[k][k - i] * x[k]
            x[i] = acc / Lb[i][0]
        out.append(x)
    return out


def musl_steps(case, nsteps):
    """Run nsteps of the MUSL loop: 2D with the blended consistent mass matrix
    (SolveExplicitSolidMechanics2D.jl:24-329, bmassMat = 0.1 Diagonal(m) + 0.9 M,
    massless rows 1 on the diagonal; solved here by banded Cholesky), 3D with
    lumped mass and no body force (SolveExplicitSolidMechanics3D.jl:14-223)."""
    d = case["dim"]
    G = PyGrid(d, case["xmin"], case["xmax"], case["nodes"], case.get("basis", 0))
    fixed = case["fixed"]
    dt, alpha, body = case["dt"], case["alpha"], case["gravity"][:d]
    n = G.count
    for _ in range(nsteps):
        mass = [0.0] * n
        mom0 = [[0.0] * d for _ in range(n)]
        force = [[0.0] * d for _ in range(n)]
        w = (2 + case.get("basis", 0) - 1) * (case["nodes"][0] + 1)  # (K - 1)(nx + 1)
        band = [[0.0] * (w + 1) for _ in range(n)] if d == 2 else None
        for B in case["bodies"]:
            for ip in range(B["n"]):
                near, funcs, ders = G.shape(B["pos"][ip])
                fVolume, fMass, vp, sigma = B["vol"][ip], B["mass"][ip], B["vel"][ip], B["stress"][ip]
                for i in range(len(near)):
                    q, Ni, dNi = near[i], funcs[i], ders[i]
                    Nim = Ni * fMass
                    mass[q] += Nim
                    if d == 2:
                        for j in range(len(near)):
                            if near[j] <= q:
                                band[q][q - near[j]] += Nim * funcs[j]
                    for a in range(d):
                        mom0[q][a] += Nim * vp[a]
                    for a in range(d):
                        s = sigma[a] * dNi[0] + sigma[a + d] * dNi[1]
                        if d == 3:
                            s = s + sigma[a + 2 * d] * dNi[2]
                        if d == 2:
                            force[q][a] += -fVolume * s + fMass * body[a] * Ni
                        else:
                            force[q][a] += -fVolume * s  # no body force in the 3D MUSL
        if d == 2:
            for i in range(n):
                for k in range(w + 1):
                    band[i][k] *= (1 - 0.1)
                band[i][0] += 0.1 * mass[i]
                if mass[i] == 0.0:
                    band[i][0] = 1.0
            v0x, v0y, dvx, dvy = _cholesky_solve_band(
                band, n, w, [[mom0[i][0] for i in range(n)], [mom0[i][1] for i in range(n)],
                             [dt * force[i][0] for i in range(n)], [dt * force[i][1] for i in range(n)]])
            v0 = [[v0x[i], v0y[i]] for i in range(n)]
            gv = [[v0x[i] + dvx[i], v0y[i] + dvy[i]] for i in range(n)]
        mom = [[0.0] * d for _ in range(n)]
        for i in range(n):
            for a in range(d):
                mom[i][a] = mom0[i][a] + force[i][a] * dt
            for a in range(d):
                if fixed[i][a] == 1:
                    mom0[i][a] = 0.0
                    mom[i][a] = 0.0
        mom2 = [[0.0] * d for _ in range(n)]
        for B in case["bodies"]:
            for ip in range(B["n"]):
                near, funcs, ders = G.shape(B["pos"][ip])
                acc = [0.0] * d
                for i in range(len(near)):
                    q, Ni = near[i], funcs[i]
                    if mass[q] > 0:
                        if d == 2:
                            for a in range(d):
                                acc[a] += Ni * (gv[q][a] - alpha * v0[q][a])
                        else:
                            mii = (1 / mass[q]) * Ni
                            for a in range(d):
                                acc[a] += (mom[q][a] - alpha * mom0[q][a]) * mii
                B["vel"][ip] = [alpha * B["vel"][ip][a] + acc[a] for a in range(d)]
                if d == 3:
                    for i in range(len(near)):
                        for a in range(d):
                            mom2[near[i]][a] += funcs[i] * B["mass"][ip] * B["vel"][ip][a]
        for B in case["bodies"]:
            for ip in range(B["n"]):
                near, funcs, ders = G.shape(B["pos"][ip])
                L = [0.0] * (d * d)
                xxp = list(B["pos"][ip])
                for i in range(len(near)):
                    q, Ni, dNi = near[i], funcs[i], ders[i]
                    if mass[q] > 0.0:
                        if d == 2:
                            vI = gv[q]
                            for a in range(d):
                                xxp[a] += (Ni * vI[a]) * dt
                            for j in range(d):
                                for a in range(d):
                                    L[a + d * j] += dNi[j] * vI[a]
                        else:
                            mii = 1 / mass[q]
                            vI = [mii * mom2[q][a] for a in range(d)]
                            for a in range(d):
                                xxp[a] += Ni * mii * dt * mom[q][a]
                            for j in range(d):  # L_rj = dN_r vI_j, as the 3D solver builds it
                                for r in range(d):
                                    L[r + d * j] += dNi[r] * vI[j]
                B["pos"][ip] = xxp
                _kinematics(B, ip, L, d, dt)
    case["grid_out"] = (mass, mom0, mom, force)
    return case


# ---------------------------------------------------------------------------
def case_from_objects(grid, solids, alg, data, nsteps, basis=0):
    from jump_gb300.engine import colmajor
    from jump_gb300.material import ElastoPlasticMaterial
    d = grid.dim
    xmin = [grid.xmin, grid.ymin] + ([grid.zmin] if d == 3 else [])
    xmax = [grid.xmax, grid.ymax] + ([grid.zmax] if d == 3 else [])
    nodes = [grid.nodeCountX, grid.nodeCountY] + ([grid.nodeCountZ] if d == 3 else [])
    fixed = [tuple(int(v) for v in grid.fixedNodes[:, i]) for i in range(grid.nodeCount)]
    g = np.zeros(3)
    if data.get("bodyforce") is not None:
        g[:d] = data["bodyforce"].g
    bodies = []
    for s in solids:
        m = s.mat
        mat = {"type": m.kind, "E": m.E, "nu": m.nu, "density": m.density, "lambda": m.lambda_, "mu": m.mu,
               "kappa": m.lambda_ + m.mu, "fy": getattr(m, "fy", 0.0), "k1": getattr(m, "k1", 0.0)}
        for k in ("A", "B", "C", "n", "epsdot0", "cellsize"):
            mat[k] = float(getattr(m, k, 0.0))
        n = s.parCount
        dinit, dam, temp = np.zeros(n), np.zeros(n), np.zeros(n)
        dp_ = getattr(m, "damage_part", None)
        if dp_ is not None:
            mat.update(m=m.m, chi=m.chi, Cp=m.Cp, d1=dp_.d1, d2=dp_.d2, d3=dp_.d3, d4=dp_.d4, d5=dp_.d5,
                       depsdot0=dp_.epsdot0, Tr=dp_.Tr, Tm=dp_.Tm)
            dinit, dam, temp = m.damage_init[:n].copy(), m.dam[:n].copy(), dp_.temp[:n].copy()
        ps = 3 if d == 2 else 9
        ep = np.zeros((n, ps))
        alpha = np.zeros(n)
        alphadot = np.zeros(n)
        if isinstance(m, ElastoPlasticMaterial):
            alpha = m.alpha[:n].copy()
            ep = m.pstrain[:n].copy() if d == 2 else colmajor(m.pstrain_3D[:n]).reshape(n, 9)
        elif getattr(m, "alphadot", None) is not None:
            alpha = m.alpha[:n].copy()
            alphadot = m.alphadot[:n].copy()
        bodies.append({
            "n": n, "mat": mat,
            "pos": [list(map(float, r)) for r in s.pos], "vel": [list(map(float, r)) for r in s.velocity],
            "mass": list(map(float, s.mass)), "vol": list(map(float, s.volume)),
            "vol0": list(map(float, s.volumeInitial)),
            "F": [list(map(float, r)) for r in colmajor(s.deformationGradient).reshape(n, d * d)],
            "strain": [list(map(float, r)) for r in colmajor(s.strain).reshape(n, d * d)],
            "stress": [list(map(float, r)) for r in colmajor(s.stress).reshape(n, d * d)],
            "alpha": list(map(float, alpha)), "ep": [list(map(float, r)) for r in ep],
            "vm": [0.0] * n, "alphadot": list(map(float, alphadot)),
            "dinit": list(map(float, dinit)), "dam": list(map(float, dam)), "temp": list(map(float, temp)),
            "youngs": None if s.youngs is None else list(map(float, s.youngs)),
        })
    musl = hasattr(alg, "alpha")
    return {"dim": d, "xmin": xmin, "xmax": xmax, "nodes": nodes, "fixed": fixed, "dt": float(data["dt"]),
            "tol": 0.0 if musl else float(alg.tolerance), "gravity": list(map(float, g)), "bodies": bodies,
            "nsteps": nsteps, "alg": 1 if musl else 0, "alpha": float(alg.alpha) if musl else 1.0,
            "basis": basis}


def save_case(name, case_in, case_out):
    arrs = {}
    d = case_in["dim"]
    arrs["meta_dim"] = np.array(d)
    arrs["meta_xmin"] = np.array(case_in["xmin"])
    arrs["meta_xmax"] = np.array(case_in["xmax"])
    arrs["meta_nodes"] = np.array(case_in["nodes"])
    arrs["meta_fixed"] = np.array(case_in["fixed"], dtype=np.int64)
    arrs["meta_dt"] = np.array(case_in["dt"])
    arrs["meta_tol"] = np.array(case_in["tol"])
    arrs["meta_gravity"] = np.array(case_in["gravity"])
    arrs["meta_nsteps"] = np.array(case_in["nsteps"])
    arrs["meta_nbodies"] = np.array(len(case_in["bodies"]))
    arrs["meta_alg"] = np.array(case_in["alg"])
    arrs["meta_basis"] = np.array(case_in.get("basis", 0))
    arrs["meta_alpha"] = np.array(case_in["alpha"])
    for b, (Bi, Bo) in enumerate(zip(case_in["bodies"], case_out["bodies"])):
        m = Bi["mat"]
        arrs[f"b{b}_mat"] = np.array([m["type"], m["E"], m["nu"], m["density"], m["fy"], m["k1"]])
        arrs[f"b{b}_matx"] = np.array([m["A"], m["B"], m["C"], m["n"], m["epsdot0"], m["cellsize"]])
        for k in ("pos", "vel", "mass", "vol", "vol0", "F", "strain", "stress", "alpha", "ep", "alphadot"):
            arrs[f"b{b}_in_{k}"] = np.array(Bi[k], dtype=np.float64)
        if Bi["youngs"] is not None:
            arrs[f"b{b}_in_youngs"] = np.array(Bi["youngs"], dtype=np.float64)
        for k in ("pos", "vel", "vol", "F", "strain", "stress", "alpha", "ep", "vm", "alphadot"):
            arrs[f"b{b}_out_{k}"] = np.array(Bo[k], dtype=np.float64)
        if m["type"] == 5:  # Johnson-Cook with damage: its constants and state
            arrs[f"b{b}_matd"] = np.array([m[k] for k in ("m", "chi", "Cp", "d1", "d2", "d3", "d4", "d5",
                                                          "depsdot0", "Tr", "Tm")])
            for k in ("dinit", "dam", "temp"):
                arrs[f"b{b}_in_{k}"] = np.array(Bi[k], dtype=np.float64)
                arrs[f"b{b}_out_{k}"] = np.array(Bo[k], dtype=np.float64)
    mass, mom0, mom, force = case_out["grid_out"]
    arrs["grid_mass"] = np.array(mass)
    arrs["grid_momentum0"] = np.array(mom0)
    arrs["grid_momentum"] = np.array(mom)
    arrs["grid_force"] = np.array(force)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)


def main(only=None):
    import copy
    from jump_gb300 import scenarios
    from jump_gb300.algorithm import ConstantBodyForce2D, ConstantBodyForce3D, USL
    from jump_gb300.grid import Grid2D, Grid3D
    from jump_gb300.material import ElasticMaterial, ElastoPlasticMaterial, NeoHookeanMaterial
    from jump_gb300.solid import (Solid2D, Solid3D, assign_velocity, buildParticleForCircle,
                                  buildParticleForCylinder, buildParticleForRectangle,
                                  buildParticleForSphere)

    cases = {}
    # 1. the two-disk collision (416 particles, all faces fixed), 20 steps
    g, s, alg, data = scenarios.two_disks()
    scenarios.apply_dirichlet(g, data)
    cases["two_disks_elastic_20"] = (case_from_objects(g, s, alg, data, 20))
    # 2. 2D neo-Hookean beam under gravity with per-particle E, clamped left face
    g = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    off = g.dx / 2
    c = buildParticleForRectangle([0.3, 0.5], 0.6, 0.2, off)
    m = NeoHookeanMaterial(1e4, 0.3, 1000.0, len(c))
    so = Solid2D(c, m)
    so.mass *= off * off
    so.volume[:] = off * off
    so.volumeInitial[:] = off * off
    so.youngs = np.random.default_rng(1).uniform(0.5e4, 2e4, len(c))
    data = {"dt": 1e-3, "bodyforce": ConstantBodyForce2D([0.0, -10.0]), "dirichlet_grid": [("left", (1, 1))]}
    scenarios.apply_dirichlet(g, data)
    cases["beam_nh_gravity_15"] = case_from_objects(g, [so], USL(1e-9), data, 15)
    # 3. 2D J2 disks (yielding)
    g, s, alg, data = scenarios.two_disks(nodes=11, speed=0.5, material="j2", E=1e4)
    scenarios.apply_dirichlet(g, data)
    cases["two_disks_j2_25"] = case_from_objects(g, s, alg, data, 25)
    # 4. 3D J2 mini Taylor bar, fast impact so that particles yield
    g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3,
                                           gap=0.0, speed=300.0)
    scenarios.apply_dirichlet(g, data)
    cases["taylor_mini_j2_6"] = case_from_objects(g, s, alg, data, 6)
    # 5. 3D elastic and 3D neo-Hookean spheres hitting each other
    for kind in ("elastic", "neohookean"):
        g = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 7, 7, 7)
        off = g.dx / 2
        c1 = buildParticleForSphere([0.35, 0.35, 0.4], 0.17, off)
        c2 = buildParticleForSphere([0.65, 0.65, 0.6], 0.17, off)
        mk = (lambda n: ElasticMaterial(1e3, 0.3, 1000.0, n)) if kind == "elastic" else \
            (lambda n: NeoHookeanMaterial(1e3, 0.3, 1000.0, n))
        s1, s2 = Solid3D(c1, mk(len(c1))), Solid3D(c2, mk(len(c2)))
        for so in (s1, s2):
            so.mass *= off ** 3
            so.volume[:] = off ** 3
            so.volumeInitial[:] = off ** 3
        assign_velocity(s1, [0.3, 0.3, 0.2])
        assign_velocity(s2, [-0.3, -0.3, -0.2])
        data = {"dt": 2e-3, "bodyforce": ConstantBodyForce3D([0.0, 0.0, -1.0]),
                "dirichlet_grid": [("front", (0, 0, 1)), ("left", (1, 0, 0))]}
        scenarios.apply_dirichlet(g, data)
        cases[f"spheres_{kind}_12"] = case_from_objects(g, [s1, s2], USL(1e-9), data, 12)

    # 6. MUSL: 2D touching elastic disks (consistent mass, alpha 0.99); 3D
    #    neo-Hookean spheres colliding in one velocity field (lumped mass,
    #    alpha 1); 3D J2 mini Taylor bar (alpha 0.99: with alpha 1 the 3D
    #    solver's FLIP increment (p - p0)/m vanishes at the fixed wall nodes and
    #    the bar passes the wall undeformed)
    from jump_gb300.algorithm import MUSL
    touch = ((0.3, 0.3), (0.3 + 0.4 / math.sqrt(2.0), 0.3 + 0.4 / math.sqrt(2.0)))
    g, s, alg, data = scenarios.two_disks(nodes=11, centers=touch, speed=0.5)
    scenarios.apply_dirichlet(g, data)
    cases["two_disks_musl_15"] = case_from_objects(g, s, MUSL(0.99), data, 15)
    g = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 7, 7, 7)
    off = g.dx / 2
    c1 = buildParticleForSphere([0.4, 0.4, 0.45], 0.17, off)
    c2 = buildParticleForSphere([0.6, 0.6, 0.55], 0.17, off)
    s1, s2 = Solid3D(c1, NeoHookeanMaterial(1e3, 0.3, 1000.0, len(c1))), \
        Solid3D(c2, NeoHookeanMaterial(1e3, 0.3, 1000.0, len(c2)))
    for so in (s1, s2):
        so.mass *= off ** 3
        so.volume[:] = off ** 3
        so.volumeInitial[:] = off ** 3
    assign_velocity(s1, [0.3, 0.3, 0.2])
    assign_velocity(s2, [-0.3, -0.3, -0.2])
    data = {"dt": 2e-3, "bodyforce": ConstantBodyForce3D([0.0, 0.0, -1.0]),
            "dirichlet_grid": [("front", (0, 0, 1)), ("left", (1, 0, 0))]}
    scenarios.apply_dirichlet(g, data)
    cases["spheres_nh_musl_12"] = case_from_objects(g, [s1, s2], MUSL(1.0), data, 12)
    g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3,
                                           gap=0.0, speed=300.0)
    scenarios.apply_dirichlet(g, data)
    cases["taylor_mini_musl_j2_10"] = case_from_objects(g, s, MUSL(0.99), data, 10)

    # 7. Johnson-Cook (USL) and Voce (MUSL 0.99) mini Taylor bars: the copper of the
    #    reference's Taylor-bar driver in SI units, cellsize one grid cell
    from jump_gb300.material import JohnsonCookMaterial, VoceMaterial
    for kind in ("jc", "voce"):
        g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3,
                                               gap=0.0, speed=300.0)
        n = s[0].parCount
        if kind == "jc":
            s[0].mat = JohnsonCookMaterial(115e9, 0.31, 8940.0, 65e6, 356e6, 0.013, 0.37, 1e-3, 0.0, 0.0, 0.0,
                                           1e-3, n)
        else:
            s[0].mat = VoceMaterial(115e9, 0.31, 8940.0, 200e6, 120e6, 20.0, 0.0, 0.0, 1e-3, n)
        scenarios.apply_dirichlet(g, data)
        algo = USL(1e-3 * float(s[0].mass[0])) if kind == "jc" else MUSL(0.99)
        cases[f"taylor_mini_{kind}_10"] = case_from_objects(g, s, algo, data, 10)

    # 9. Johnson-Cook with damage (USL and MUSL 0.99): copper strength with a
    #    small failure strain and a melting point just above Tr, so that within
    #    a few steps particles initiate damage, fail completely, soften thermally
    #    and pass Tm
    from jump_gb300.material import JohnsonCookDamage, JohnsonCookMaterialWithDamage
    for scheme, steps, d1, d2, Tm in (("usl", 12, 0.002, 0.004, 294.0), ("musl", 10, 0.0002, 0.0004, 293.02)):
        g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3,
                                               gap=0.0, speed=300.0)
        n = s[0].parCount
        st = JohnsonCookMaterial(115e9, 0.31, 8940.0, 65e6, 356e6, 0.013, 0.37, 1e-3, 1.09, 0.9, 383.0, 1e-3, n)
        s[0].mat = JohnsonCookMaterialWithDamage(st, JohnsonCookDamage(d1, d2, -0.54, 0.015, 0.2, 1e-3,
                                                                       293.0, Tm, n))
        # seeded starting states: every 5th particle above Tm, every 7th with damage
        # initiated (damage_init 0.5), every 11th partly damaged (damage 0.3)
        m = s[0].mat
        m.damage_part.temp[::5] = Tm + 1.0
        m.damage_init[::7] = 0.5
        m.damage_init[::11] = 1.03
        m.dam[::11] = 0.3
        scenarios.apply_dirichlet(g, data)
        algo = USL(1e-3 * float(s[0].mass[0])) if scheme == "usl" else MUSL(0.99)
        cases[f"taylor_mini_jcdamage_{scheme}_{steps}"] = case_from_objects(g, s, algo, data, steps)

    # 8. B-spline bases: the two-disk collision with quadratic B-splines and USL
    #    (Main_TwoDisks.jl:53, 116); 3D neo-Hookean spheres with cubic B-splines
    #    and USL; a 2D neo-Hookean beam under gravity with cubic B-splines and
    #    MUSL (consistent mass, Main_VibratingBeam.jl:103); the J2 mini Taylor
    #    bar with quadratic B-splines and MUSL 0.99 (3D lumped)
    g, s, alg, data = scenarios.two_disks(nodes=21, centers=touch, speed=0.3)
    scenarios.apply_dirichlet(g, data)
    cases["two_disks_quad_12"] = case_from_objects(g, s, alg, data, 12, basis=1)
    g = Grid3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 9, 9, 9)
    off = g.dx / 2
    c1 = buildParticleForSphere([0.4, 0.4, 0.42], 0.14, off)
    c2 = buildParticleForSphere([0.6, 0.6, 0.58], 0.14, off)
    s1, s2 = Solid3D(c1, NeoHookeanMaterial(1e3, 0.3, 1000.0, len(c1))), \
        Solid3D(c2, NeoHookeanMaterial(1e3, 0.3, 1000.0, len(c2)))
    for so in (s1, s2):
        so.mass *= off ** 3
        so.volume[:] = off ** 3
        so.volumeInitial[:] = off ** 3
    assign_velocity(s1, [0.3, 0.3, 0.2])
    assign_velocity(s2, [-0.3, -0.3, -0.2])
    data = {"dt": 2e-3, "bodyforce": ConstantBodyForce3D([0.0, 0.0, -1.0]),
            "dirichlet_grid": [("front", (0, 0, 1))]}
    scenarios.apply_dirichlet(g, data)
    cases["spheres_nh_cubic_8"] = case_from_objects(g, [s1, s2], USL(1e-9), data, 8, basis=2)
    g = Grid2D(0.0, 1.0, 0.0, 1.0, 11, 11)
    off = g.dx / 2
    c = buildParticleForRectangle([0.4, 0.5], 0.6, 0.2, off)
    so = Solid2D(c, NeoHookeanMaterial(1e4, 0.3, 1000.0, len(c)))
    so.mass *= off * off
    so.volume[:] = off * off
    so.volumeInitial[:] = off * off
    so.velocity[:, 1] = 2.0 * (so.pos[:, 0] - 0.4)  # rotating: the 2D MUSL ignores the clamp
    data = {"dt": 1e-3, "bodyforce": ConstantBodyForce2D([0.0, -10.0]), "dirichlet_grid": [("left", (1, 1))]}
    scenarios.apply_dirichlet(g, data)
    cases["beam_nh_cubic_musl_10"] = case_from_objects(g, [so], MUSL(1.0), data, 10, basis=2)
    g, s, alg, data = scenarios.taylor_bar(h=1e-3, radius=2e-3, length=6e-3, width=8e-3, height=10e-3,
                                           gap=0.0, speed=300.0)
    scenarios.apply_dirichlet(g, data)
    cases["taylor_mini_quad_musl_8"] = case_from_objects(g, s, MUSL(0.99), data, 8, basis=1)

    for name, cin in cases.items():
        if only and name not in only:
            continue
        run = musl_steps if cin["alg"] == 1 else usl_steps
        cout = run(copy.deepcopy(cin), cin["nsteps"])
        save_case(name, cin, cout)
        print("wrote", name, [b["n"] for b in cin["bodies"]])


if __name__ == "__main__":
    # optional case names: regenerate only those fixtures
    main(sys.argv[1:])
