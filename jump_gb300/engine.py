"""Context objects over the C ABI (include/jump_mpm.h).

``build_descriptors`` turns the host mirror of jump's types (Grid2D/3D,
Solid2D/3D, materials, USL, a constant body force) into the ABI's
descriptors; ``MPMContext`` owns one device context of the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .algorithm import USL, ConstantBodyForce2D, ConstantBodyForce3D
from .material import ElastoPlasticMaterial, RigidMaterial

PRECISIONS = {"f64": _capi.MPM_PREC_F64, "f32": _capi.MPM_PREC_F32, "dw": _capi.MPM_PREC_DW}


def colmajor(a: np.ndarray) -> np.ndarray:
    """(n, d, d) with a[p, i, j] = A_ij  ->  flat column-major per particle."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose(0, 2, 1))


def from_colmajor(flat: np.ndarray, n: int, d: int) -> np.ndarray:
    return flat.reshape(n, d, d).transpose(0, 2, 1)


class Descriptors:
    """Descriptors plus the numpy arrays they point into (kept alive here).
    precision: "f64", "f32" (FP32 particles, FP64 nodes) or "dw" (FP64 fields
    and nodes, P2G and G2P arithmetic in double-word FP32; 3D USL)."""

    def __init__(self, grid, solids, tolerance=0.0, body_force=None, dt=0.0, precision="f64",
                 contact=False, friction=0.0, sort_interval=0, algorithm="usl", alpha=1.0, basis="linear"):
        d = grid.dim
        self.dim = d
        self._keep = []
        g = _capi.GridDesc()
        g.dim = d
        g.xmin[0], g.xmin[1] = grid.xmin, grid.ymin
        g.xmax[0], g.xmax[1] = grid.xmax, grid.ymax
        g.nodes[0], g.nodes[1] = grid.nodeCountX, grid.nodeCountY
        if d == 3:
            g.xmin[2], g.xmax[2], g.nodes[2] = grid.zmin, grid.zmax, grid.nodeCountZ
        else:
            g.nodes[2] = 1
        fixed = np.ascontiguousarray(np.asarray(grid.fixedNodes, dtype=np.int64).T)  # (Nn, d)
        self._keep.append(fixed)
        g.fixed_nodes = _capi.iptr(fixed)
        self.grid = g
        bodies = (_capi.BodyDesc * max(1, len(solids)))()
        for s, sol in enumerate(solids):
            b = bodies[s]
            b.count = sol.parCount
            m = sol.mat
            b.mat.type = m.kind
            if isinstance(m, RigidMaterial):
                b.mat.v_rigid[0], b.mat.v_rigid[1], b.mat.v_rigid[2] = m.vx, m.vy, m.vz
                b.mat.fixed = 1 if m.fixed else 0
            b.mat.E, b.mat.nu, b.mat.density = m.E, m.nu, m.density
            b.mat.fy, b.mat.k1 = getattr(m, "fy", 0.0), getattr(m, "k1", 0.0)
            for k in ("A", "B", "C", "n", "epsdot0", "cellsize"):
                setattr(b.mat, k, float(getattr(m, k, 0.0)))
            dmg = getattr(m, "damage_part", None)
            if dmg is not None:  # JohnsonCookMaterialWithDamage
                b.mat.m, b.mat.chi, b.mat.Cp = m.m, m.chi, m.Cp
                for k in ("d1", "d2", "d3", "d4", "d5", "Tr", "Tm"):
                    setattr(b.mat, k, getattr(dmg, k))
                b.mat.depsdot0 = dmg.epsdot0
            arrs = {
                "pos": np.ascontiguousarray(sol.pos, dtype=np.float64),
                "velocity": np.ascontiguousarray(sol.velocity, dtype=np.float64),
                "mass": np.ascontiguousarray(sol.mass, dtype=np.float64),
                "volume": np.ascontiguousarray(sol.volume, dtype=np.float64),
                "volume_initial": np.ascontiguousarray(sol.volumeInitial, dtype=np.float64),
                "F": colmajor(sol.deformationGradient),
                "strain": colmajor(sol.strain),
                "stress": colmajor(sol.stress),
            }
            if isinstance(m, ElastoPlasticMaterial):
                arrs["alpha"] = np.ascontiguousarray(m.alpha[: sol.parCount], dtype=np.float64)
                if d == 2:
                    arrs["pstrain"] = np.ascontiguousarray(m.pstrain[: sol.parCount], dtype=np.float64)
                else:
                    arrs["pstrain"] = colmajor(m.pstrain_3D[: sol.parCount])
            if getattr(sol, "youngs", None) is not None:
                arrs["youngs"] = np.ascontiguousarray(sol.youngs, dtype=np.float64)
            if getattr(m, "alphadot", None) is not None:  # Johnson-Cook / Voce state
                arrs["alpha"] = np.ascontiguousarray(m.alpha[: sol.parCount], dtype=np.float64)
                arrs["alphadot"] = np.ascontiguousarray(m.alphadot[: sol.parCount], dtype=np.float64)
            if getattr(m, "vmStr", None) is not None:
                arrs["vmstr"] = np.ascontiguousarray(m.vmStr[: sol.parCount], dtype=np.float64)
            if dmg is not None:
                arrs["damage_init"] = np.ascontiguousarray(m.damage_init[: sol.parCount], dtype=np.float64)
                arrs["damage"] = np.ascontiguousarray(m.dam[: sol.parCount], dtype=np.float64)
                arrs["temperature"] = np.ascontiguousarray(dmg.temp[: sol.parCount], dtype=np.float64)
            for k, v in arrs.items():
                self._keep.append(v)
                setattr(b, k, _capi.dptr(v))
        self.bodies = bodies
        self.nbodies = len(solids)
        p = _capi.Params()
        p.dt = float(dt)
        p.tolerance = float(tolerance)
        bf = np.zeros(3)
        if body_force is not None:
            g_ = np.asarray(getattr(body_force, "g", body_force), dtype=np.float64).ravel()
            bf[: g_.size] = g_
        p.body_force[0], p.body_force[1], p.body_force[2] = bf
        p.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        p.contact = 1 if contact else 0
        p.friction = float(friction)
        p.sort_interval = int(sort_interval)
        p.flags = 0
        p.algorithm = {"usl": _capi.MPM_ALG_USL, "musl": _capi.MPM_ALG_MUSL}[algorithm]
        p.alpha = float(alpha)
        p.basis = {"linear": _capi.MPM_BASIS_LINEAR, "quad": _capi.MPM_BASIS_QUAD_BSPLINE,
                   "cubic": _capi.MPM_BASIS_CUBIC_BSPLINE}[basis]
        self.params = p


class BodyState:
    """Host arrays one body downloads into (the reference layouts)."""

    def __init__(self, n: int, d: int):
        self.n, self.d = n, d
        self.pos = np.zeros((n, d))
        self.velocity = np.zeros((n, d))
        self.volume = np.zeros(n)
        self.F = np.zeros(n * d * d)
        self.strain = np.zeros(n * d * d)
        self.stress = np.zeros(n * d * d)
        self.alpha = np.zeros(n)
        self.pstrain = np.zeros(n * (3 if d == 2 else 9))
        self.vmstr = np.zeros(n)
        self.alphadot = np.zeros(n)
        self.damage_init = np.zeros(n)
        self.damage = np.zeros(n)
        self.temperature = np.zeros(n)

    FIELDS = ("pos", "velocity", "volume", "F", "strain", "stress", "alpha", "pstrain", "vmstr", "alphadot",
              "damage_init", "damage", "temperature")

    def view(self) -> _capi.BodyView:
        v = _capi.BodyView()
        for k in self.FIELDS:
            setattr(v, k, _capi.dptr(getattr(self, k)))
        return v

    def matrices(self):
        n, d = self.n, self.d
        return (from_colmajor(self.F, n, d), from_colmajor(self.strain, n, d),
                from_colmajor(self.stress, n, d))


class _ContextBase:
    """Shared driver logic for the CUDA context and the CPU oracle."""

    def __init__(self, desc: Descriptors):
        self.desc = desc
        self.dim = desc.dim
        self.counts = [desc.bodies[s].count for s in range(desc.nbodies)]

    def download_body(self, s: int, into: BodyState | None = None) -> BodyState:
        """Body s's state, into `into` (reused host arrays) or new arrays."""
        st = BodyState(self.counts[s], self.dim) if into is None else into
        if st.n != self.counts[s] or st.d != self.dim:
            raise ValueError("download_body: state arrays of the wrong size")
        self._download(s, st.view())
        return st

    def download_all(self, into: list | None = None):
        """Every body's state; pass the list a previous call returned to reuse its arrays."""
        if into is None:
            return [self.download_body(s) for s in range(len(self.counts))]
        return [self.download_body(s, st) for s, st in enumerate(into)]


class MPMContext(_ContextBase):
    """One device context of libjumpmpm.so."""

    def __init__(self, desc: Descriptors):
        super().__init__(desc)
        self.L = _capi.lib()
        h = C.c_void_p()
        _capi.check(self.L.mpm_create(C.byref(desc.grid), desc.bodies, desc.nbodies,
                                      C.byref(desc.params), C.byref(h)), self.L)
        self.h = h

    def step(self, nsteps: int, t: float | None = None, check: bool = True):
        tt = C.c_double(0.0 if t is None else t)
        rc = self.L.mpm_step(self.h, int(nsteps), C.byref(tt))
        if check:
            _capi.check(rc, self.L)
        return tt.value if t is not None else rc

    def step_energies(self, nsteps: int, every: int = 1, first: int = 0, t: float | None = None,
                      check: bool = True):
        """nsteps steps with the EnergiesFix sums after local steps first, first + every, ...;
        returns (records, t or status): records is (n, 2 + dim) = [KE, SE, momentum...]."""
        nrec = (nsteps - 1 - first) // every + 1 if nsteps > first else 0
        out = np.zeros((max(nrec, 0), 2 + self.dim))
        tt = C.c_double(0.0 if t is None else t)
        rc = self.L.mpm_step_energies(self.h, int(nsteps), int(every), int(first), C.byref(tt),
                                      _capi.dptr(out) if nrec > 0 else None)
        if check:
            _capi.check(rc, self.L)
        return out, (tt.value if t is not None else rc)

    P2G_STRATEGIES = {"atomic": _capi.MPM_P2G_ATOMIC, "warp": _capi.MPM_P2G_WARP, "tile": _capi.MPM_P2G_TILE,
                      "tile_warp": _capi.MPM_P2G_TILE_WARP, "fused": _capi.MPM_P2G_FUSED}

    def set_launch(self, p2g: str | None = None, threads: int | None = None, sort_interval: int | None = None):
        """P2G strategy ("atomic", "warp", "tile", "tile_warp"; "fused": every stage of every step in
        one cooperative launch, for small problems), CTA size of P2G and G2P, cell-sort interval;
        None keeps a setting."""
        s = -1 if p2g is None else self.P2G_STRATEGIES[p2g]
        _capi.check(self.L.mpm_set_launch(self.h, s, -1 if threads is None else int(threads),
                                          -1 if sort_interval is None else int(sort_interval)), self.L)

    def launch(self) -> dict:
        s, t, i = C.c_int32(), C.c_int32(), C.c_int32()
        _capi.check(self.L.mpm_get_launch(self.h, C.byref(s), C.byref(t), C.byref(i)), self.L)
        names = {v: k for k, v in self.P2G_STRATEGIES.items()}
        return {"p2g": names[s.value], "threads": t.value, "sort_interval": i.value}

    def tune(self, probe_steps: int = 5) -> dict:
        """Time every P2G strategy x CTA size x sort interval from the current state, keep the
        fastest; the simulation does not advance.  ``probes`` maps "p2g/threads/sort" to ms per step."""
        s, t, i, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        allms = np.zeros(_capi.MPM_TUNE_CANDIDATES)
        _capi.check(self.L.mpm_tune(self.h, int(probe_steps), C.byref(s), C.byref(t), C.byref(i), C.byref(ms),
                                    _capi.dptr(allms)), self.L)
        probes = {}
        for q, v in enumerate(allms[:48]):
            p2g, th, si = ("atomic", "warp", "tile", "tile_warp")[q // 12], (64, 128, 256)[(q // 4) % 3], \
                (0, 1, 4, 16)[q % 4]
            if v >= 0:
                probes[f"{p2g}/{th}/{si}"] = float(v)
        if allms[48] >= 0:
            probes["fused"] = float(allms[48])
        return dict(self.launch(), ms_per_step=ms.value, probes=probes)

    def _download(self, s, view):
        _capi.check(self.L.mpm_download(self.h, int(s), C.byref(view)), self.L)

    def download_grid(self, nn: int):
        d = self.dim
        m, p0, p, f = np.zeros(nn), np.zeros((nn, d)), np.zeros((nn, d)), np.zeros((nn, d))
        _capi.check(self.L.mpm_download_grid(self.h, _capi.dptr(m), _capi.dptr(p0), _capi.dptr(p),
                                             _capi.dptr(f)), self.L)
        return m, p0, p, f

    def energies(self):
        ke, se = C.c_double(), C.c_double()
        mom = np.zeros(3)
        _capi.check(self.L.mpm_energies(self.h, C.byref(ke), C.byref(se), _capi.dptr(mom)), self.L)
        return ke.value, se.value, mom[: self.dim]

    def save(self) -> bytes:
        n = C.c_size_t(0)
        _capi.check(self.L.mpm_save(self.h, None, C.byref(n)), self.L)
        buf = C.create_string_buffer(n.value)
        _capi.check(self.L.mpm_save(self.h, buf, C.byref(n)), self.L)
        return buf.raw

    def load(self, data: bytes):
        _capi.check(self.L.mpm_load(self.h, data, len(data)), self.L)

    def last_step_ms(self) -> float:
        ms = C.c_double()
        _capi.check(self.L.mpm_last_step_ms(self.h, C.byref(ms)), self.L)
        return ms.value

    def fwd_checkpointed(self, nsteps: int, every: int):
        """nsteps steps keeping a snapshot every `every` steps (reverse mode)."""
        _capi.check(self.L.mpm_fwd_checkpointed(self.h, int(nsteps), int(every)), self.L)

    def bwd(self, x_bar: np.ndarray, v_bar: np.ndarray | None = None) -> dict:
        """Reverse sweep of the last fwd_checkpointed run.  x_bar/v_bar: dL/dx, dL/dv
        at the final step, (total particles, dim).  Returns dL/dE per particle and
        dL/dv, dL/dx at the initial step."""
        n = sum(self.counts)
        xb = np.ascontiguousarray(x_bar, dtype=np.float64).reshape(n, self.dim)
        vb = None if v_bar is None else np.ascontiguousarray(v_bar, dtype=np.float64).reshape(n, self.dim)
        E = np.zeros(n)
        v0 = np.zeros((n, self.dim))
        x0 = np.zeros((n, self.dim))
        _capi.check(self.L.mpm_bwd(self.h, _capi.dptr(xb), _capi.dptr(vb), _capi.dptr(E), _capi.dptr(v0),
                                   _capi.dptr(x0)), self.L)
        return {"E": E, "v0": v0, "x0": x0}

    def profile_stages(self, nsteps: int) -> dict:
        """Device ms per stage summed over nsteps steps (individual launches, CUDA events)."""
        out = np.zeros(len(_capi.STAGES))
        _capi.check(self.L.mpm_profile_stages(self.h, int(nsteps), _capi.dptr(out)), self.L)
        return dict(zip(_capi.STAGES, out.tolist()))

    def close(self):
        if getattr(self, "h", None):
            self.L.mpm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
