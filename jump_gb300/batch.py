"""Batched ensembles: many independent problems advanced together.

    ens = Ensemble([scenarios.ensemble_member(i) for i in range(512)], precision="f64")
    ens.tune()                 # strategy and launch shape, timed (cached per workload signature)
    ens.step(1000)             # every problem advances 1000 steps
    ens.download(i)            # BodyState list of problem i

Each problem is the (grid, solids, alg, data) a solve_explicit_dynamics_2D/3D
call would take; ``data["contact"]`` / ``data["friction"]`` select contact
mode per problem.  Strategies: "persistent" (one launch for all problems and
steps; one material model type, no contact) and "wide" (one launch per stage
for all problems; any mix).  The C entry points are mpm_batch_* in
include/jump_mpm.h.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os

import numpy as np

from . import _capi
from .dirichlet import fix_Dirichlet_grid
from .engine import BodyState, Descriptors, PRECISIONS


def _cache_path():
    base = os.environ.get("JUMP_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "jump_gb300"))
    return os.path.join(base, "autotune.json")


class Ensemble:
    def __init__(self, problems, precision="f64"):
        self.L = _capi.lib()
        self._descs = []
        insts = (_capi.InstanceDesc * len(problems))()
        self.counts = []
        self.dim = None
        for i, (grid, solids, alg, data) in enumerate(problems):
            fix_Dirichlet_grid(grid, data, ghostcell="ghostcell" in data)
            d = Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"),
                            dt=data["dt"], precision=precision)
            self._descs.append(d)
            insts[i].grid = d.grid
            insts[i].bodies = C.cast(d.bodies, C.POINTER(_capi.BodyDesc))
            insts[i].nbodies = d.nbodies
            insts[i].dt = d.params.dt
            insts[i].tolerance = d.params.tolerance
            for a in range(3):
                insts[i].body_force[a] = d.params.body_force[a]
            insts[i].contact = 1 if data.get("contact") else 0
            insts[i].friction = float(data.get("friction", 0.0))
            self.counts.append([d.bodies[s].count for s in range(d.nbodies)])
            self.dim = d.dim
        self._insts = insts
        self.precision = precision
        h = C.c_void_p()
        _capi.check(self.L.mpm_batch_create(C.cast(insts, C.c_void_p), len(problems),
                                            PRECISIONS[precision], C.byref(h)), self.L)
        self.h = h
        self.n = len(problems)
        self.particles = int(sum(sum(c) for c in self.counts))

    def signature(self) -> str:
        """Workload key of the autotune cache: dimension, precision, sizes."""
        sizes = ",".join(str(sum(c)) for c in self.counts)
        kinds = ",".join(f"{int(i.contact)}" for i in self._insts)
        return (f"d{self.dim}-{self.precision}-n{self.n}-"
                + hashlib.sha1((sizes + "|" + kinds).encode()).hexdigest()[:12])

    def tune(self, probe_steps: int = 20, use_cache: bool = True):
        """Pick threads per CTA and CTAs per SM by timing them; remembered per workload."""
        path = _cache_path()
        key = self.signature()
        cache = {}
        if use_cache and os.path.exists(path):
            try:
                cache = json.load(open(path))
            except (OSError, ValueError):
                cache = {}
        if use_cache and key in cache and "strategy" in cache[key]:
            th, cps = cache[key]["threads"], cache[key]["ctas_per_sm"]
            _capi.check(self.L.mpm_batch_set_launch(self.h, th, cps), self.L)
            self.set_strategy(cache[key]["strategy"])
            return dict(cache[key], cached=True)
        th, cps, ms = C.c_int32(), C.c_int32(), C.c_double()
        _capi.check(self.L.mpm_batch_tune(self.h, int(probe_steps), C.byref(th), C.byref(cps), C.byref(ms)), self.L)
        res = {"threads": th.value, "ctas_per_sm": cps.value, "ms_per_step": ms.value,
               "strategy": self.strategy}
        if use_cache:
            cache[key] = res
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                json.dump(cache, open(path, "w"), indent=1)
            except OSError:
                pass
        return dict(res, cached=False)

    STRATEGIES = {"persistent": _capi.MPM_BATCH_PERSISTENT, "wide": _capi.MPM_BATCH_WIDE}

    @property
    def strategy(self) -> str:
        v = C.c_int32()
        _capi.check(self.L.mpm_batch_strategy(self.h, C.byref(v)), self.L)
        return {k: n for n, k in self.STRATEGIES.items()}[v.value]

    def set_strategy(self, name: str):
        """'persistent' (one launch for all problems and steps) or 'wide' (one launch per stage)."""
        _capi.check(self.L.mpm_batch_set_strategy(self.h, self.STRATEGIES[name]), self.L)

    def set_launch(self, threads: int, ctas_per_sm: int = 0):
        _capi.check(self.L.mpm_batch_set_launch(self.h, int(threads), int(ctas_per_sm)), self.L)

    def step(self, nsteps: int, check: bool = True):
        rc = self.L.mpm_batch_step(self.h, int(nsteps))
        if check:
            _capi.check(rc, self.L)
        return rc

    def jvp(self, nsteps: int, dE) -> list:
        """Advance nsteps steps (as step) and return, per problem, dx/ds of its
        particles (bodies in order, (n, dim)), where s is one scalar per problem
        and dE[i][k] = dE_k/ds is the change of body k's Young's modulus.
        Forward-mode derivative through mpm_batch_jvp (FP64 batches, elastic
        and neo-Hookean bodies, frictionless contact)."""
        seeds = np.zeros((self.n, _capi.MPM_BATCH_MAX_BODIES))
        for i, row in enumerate(dE):
            seeds[i, :len(row)] = row
        xd = np.zeros(self.particles * self.dim)
        _capi.check(self.L.mpm_batch_jvp(self.h, int(nsteps), _capi.dptr(seeds.ravel()), _capi.dptr(xd)), self.L)
        out, off = [], 0
        for c in self.counts:
            k = sum(c)
            out.append(xd[off * self.dim:(off + k) * self.dim].reshape(k, self.dim))
            off += k
        return out

    def status(self):
        st = (C.c_int32 * self.n)()
        _capi.check(self.L.mpm_batch_status(self.h, st), self.L)
        return list(st)

    def last_ms(self) -> float:
        ms = C.c_double()
        _capi.check(self.L.mpm_batch_last_ms(self.h, C.byref(ms)), self.L)
        return ms.value

    def download(self, i: int):
        out = []
        for b, n in enumerate(self.counts[i]):
            st = BodyState(n, self.dim)
            v = st.view()
            _capi.check(self.L.mpm_batch_download(self.h, int(i), int(b), C.byref(v)), self.L)
            out.append(st)
        return out

    def energies(self) -> np.ndarray:
        out = np.zeros(self.n * (2 + self.dim))
        _capi.check(self.L.mpm_batch_energies(self.h, _capi.dptr(out)), self.L)
        return out.reshape(self.n, 2 + self.dim)

    def close(self):
        if getattr(self, "h", None):
            self.L.mpm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
