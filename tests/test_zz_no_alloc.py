"""mpm_energies_static -- the entry point for callers that cannot allocate
device memory (code inside a CUDA stream capture, or programs whose device
memory belongs to another allocator) -- gives the same sums as mpm_energies.

It is called through the C ABI on particle arrays in device memory that the
test owns (allocated here with torch; the entry point itself allocates
nothing), twice in a row: all particles, then a prefix (fewer blocks), so a
partial sum left in its shared static scratch by the first call would corrupt
the second.  Each call is checked against mpm_energies of a context holding
the same particles.  This file is collected last on purpose; it passes alone
in a fresh process and after the other tests.
"""
import copy
import ctypes as C
import os
import re

import numpy as np
import pytest

from jump_gb300 import _capi, scenarios
from jump_gb300.engine import Descriptors, MPMContext

pytestmark = pytest.mark.gpu

TOL = 1e-10  # the FP64 tolerance of the parity tests


def _sym(m, d):
    """(n, d, d) -> (S, n) symmetric components in the ABI order."""
    idx = [(0, 0), (1, 1), (0, 1)] if d == 2 else [(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]
    return np.stack([m[:, i, j] for i, j in idx])


def _prefix_solids(solids, states, n):
    """Solid objects holding the downloaded state of the first n particles."""
    out, left = [], n
    for sol, st in zip(solids, states):
        if left <= 0:
            break
        k = min(left, st.n)
        s = copy.deepcopy(sol)
        F, eps, sig = st.matrices()
        s.parCount = k
        s.pos, s.velocity = st.pos[:k].copy(), st.velocity[:k].copy()
        s.mass, s.volume, s.volumeInitial = sol.mass[:k].copy(), st.volume[:k].copy(), sol.volumeInitial[:k].copy()
        s.deformationGradient, s.strain, s.stress = F[:k].copy(), eps[:k].copy(), sig[:k].copy()
        if hasattr(s.mat, "alpha"):
            s.mat.alpha = st.alpha[:k].copy()
            s.mat.pstrain = np.zeros((k, 3))
            s.mat.pstrain_3D = np.zeros((k, 3, 3))
        out.append(s)
        left -= k
    return out


def _context_energies(grid, solids, alg, data):
    ctx = MPMContext(Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"),
                                 dt=data["dt"]))
    try:
        return ctx.energies()
    finally:
        ctx.close()


def _static(L, torch, d, n, arrs):
    mass, vel, vol, sig, eps = (torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in arrs)
    out = torch.full((2 + d,), float("nan"), dtype=torch.float64, device="cuda")
    rc = L.mpm_energies_static(d, n, mass.data_ptr(), vel.data_ptr(), vol.data_ptr(), sig.data_ptr(),
                               eps.data_ptr(), out.data_ptr(), None)
    assert rc == _capi.MPM_OK, L.mpm_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(got, ref, d, arrs):
    ke, se, mom = ref
    assert abs(got[0] - ke) <= TOL * abs(ke), (got, ref)
    assert abs(got[1] - se) <= TOL * abs(se), (got, ref)
    # total momentum can cancel to rounding noise (two disks moving head-on):
    # compare against the sum of |m v_a|, the scale its rounding error lives on
    mass, vel = arrs[0], arrs[1]
    for a in range(d):
        scale = float(np.sum(np.abs(mass * vel[a])))
        assert abs(got[2 + a] - mom[a]) <= TOL * scale, (got, ref)


@pytest.mark.parametrize("dim", [2, 3])
def test_static_energies_match_context_energies(dim):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _capi.lib()
    if dim == 2:
        grid, solids, alg, data = scenarios.two_disks()
    else:
        grid, solids, alg, data = scenarios.taylor_bar(h=5e-4)
    scenarios.apply_dirichlet(grid, data)
    ctx = MPMContext(Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"),
                                 dt=data["dt"]))
    ctx.step(25)  # non-zero strain and stress everywhere
    states = ctx.download_all()
    ref_all = ctx.energies()
    ctx.close()
    assert ref_all[1] != 0.0

    def arrays(n):
        sols = _prefix_solids(solids, states, n)
        vel = np.concatenate([s.velocity for s in sols]).T
        sig = _sym(np.concatenate([s.stress for s in sols]), dim)
        eps = _sym(np.concatenate([s.strain for s in sols]), dim)
        mass = np.concatenate([s.mass for s in sols])
        vol = np.concatenate([s.volume for s in sols])
        return sols, (mass, vel, vol, sig, eps)

    n_all = sum(st.n for st in states)
    _, arrs = arrays(n_all)
    _check(_static(L, torch, dim, n_all, arrs), ref_all, dim, arrs)  # call 1

    n_pre = n_all // 3
    sols, arrs = arrays(n_pre)
    ref_pre = _context_energies(grid, sols, alg, data)
    _check(_static(L, torch, dim, n_pre, arrs), ref_pre, dim, arrs)  # call 2, fewer blocks


def test_static_energies_rejects_oversize():
    L = _capi.lib()
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "jump_mpm.h")).read()
    limit = int(re.search(r"#define MPM_STATIC_MAX_PARTICLES (\d+)", hdr).group(1))
    out = C.c_double(0.0)
    rc = L.mpm_energies_static(3, limit + 1, None, None, None, None, None, C.addressof(out), None)
    assert rc == _capi.MPM_ERR_ARG
    assert b"MPM_STATIC_MAX_PARTICLES" in L.mpm_last_error()
