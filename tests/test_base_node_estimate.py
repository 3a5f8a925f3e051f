"""The FP32 estimate of the hat's base node (base_node_estimate in
jump_gb300/csrc/mpm_common.cuh), modelled in numpy on the CPU: wherever the
estimate decides (farther from an integer than its error bound), its floor is
the floor of the FP64 expression t = RN(RN(RN(x - xmin) dxI) + 1) that the
reference's getAdjacentGridPoints evaluates (Basis.jl:63-78) -- over random
positions on grids of every scale the step meets and adversarial positions
within a few units in the last place of node lines, where the estimate must
give way to the FP64 expression."""
import numpy as np
import pytest

F32 = np.float32


def f32_trunc(x):
    """FP64 -> float by truncation of the fraction (the kernel's f32_trunc):
    NaN outside [2^-126, 2^128), zero included"""
    b = np.atleast_1d(np.asarray(x, dtype=np.float64)).view(np.uint64)
    ex = (b >> np.uint64(52)) & np.uint64(0x7FF)
    out = (b & np.uint64(0xFFFFFFFFE0000000)).view(np.float64)
    out = np.where((ex < 897) | (ex > 1150), np.nan, out)
    return out.astype(np.float32)


def fma32(a, b, c):
    """RN32(a b + c): the product of two floats is exact in FP64, and the sum's
    rounding to FP64 then to float differs from one rounding only at exact
    FP64 ties, which the bound's factor of two absorbs"""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def estimate(x, xmin, dxI):
    """(decided, i1) of base_node_estimate"""
    xminf, dxIf = F32(xmin), F32(dxI)
    xf = f32_trunc(x)
    t32 = fma32((xf - xminf).astype(F32), dxIf, F32(1.0))
    bound = F32(2.0 ** -21) * fma32((np.abs(xf) + np.abs(xminf)).astype(F32), dxIf, (np.abs(t32) + F32(1.0)).astype(F32))
    fl = np.floor(t32)
    decided = (t32 - fl > bound) & (fl + F32(1.0) - t32 > bound) & (np.abs(fl) < F32(1e9))
    return decided, np.where(decided, fl, F32(0.0)).astype(np.int64)


def reference_floor(x, xmin, dxI):
    return np.floor((x - xmin) * dxI + 1.0).astype(np.int64)


GRIDS = [  # (xmin, xmax, nodes): the Taylor bar's axes, unit and offset grids, coarse and fine
    (-8e-3, 8e-3, 65), (0.0, 40e-3, 161), (0.0, 1.0, 21), (0.0, 1.0, 81), (-1.0, 3.0, 401),
    (1000.0, 1001.0, 257), (-0.02, 0.02, 4097), (0.0, 4.0, 65)]


@pytest.mark.parametrize("xmin, xmax, nodes", GRIDS)
def test_estimate_agrees_with_the_fp64_floor(xmin, xmax, nodes):
    dx = (xmax - xmin) / (nodes - 1.0)
    dxI = 1.0 / dx
    rng = np.random.default_rng(nodes)
    # random positions over the grid and a cell beyond it
    x = rng.uniform(xmin - dx, xmax + dx, 200_000)
    # positions a few FP64 units from node lines, on both sides, and on them
    k = rng.integers(0, nodes, 100_000)
    xn = xmin + k * dx
    near = xn + rng.integers(-64, 65, k.size) * np.spacing(np.abs(xn) + 1e-300)
    x = np.concatenate([x, xn, near])
    decided, i1 = estimate(x, xmin, dxI)
    ref = reference_floor(x, xmin, dxI)
    assert np.all(i1[decided] == ref[decided])
    # it never decides on a node line; elsewhere it falls back only within its
    # bound of an integer, 2^-21 ((|x| + |xmin|) dxI + t + 1)
    assert not decided[200_000:200_000 + k.size].any()
    B = 2.0 ** -21 * ((max(abs(xmin), abs(xmax)) + dx + abs(xmin)) * dxI + nodes + 2)
    assert decided[:200_000].mean() >= 1.0 - 3.0 * B, (decided[:200_000].mean(), B)


def test_out_of_float_range_and_zero_fall_back():
    decided, _ = estimate(np.array([0.0, 1e-300, 1e300, np.nan, np.inf]), 0.0, 10.0)
    assert not decided.any()
