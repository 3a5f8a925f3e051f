"""Print the throughput of the operations the step kernels are bound by on the
current GPU (mpm_probe_rates): FP64 fused multiply-adds, FP64 divisions and
FP64 atomic additions executed in L2.  dw_op runs the double-word operations
of the MPM_PREC_DW G2P on given operands (mpm_probe_dw), for their tests.

  python -m jump_gb300.probe [--repeat 3]
"""
from __future__ import annotations

import argparse
import ctypes as C

from . import _capi


def rates() -> dict:
    L = _capi.lib()
    fma, div, atom = C.c_double(), C.c_double(), C.c_double()
    _capi.check(L.mpm_probe_rates(C.byref(fma), C.byref(div), C.byref(atom)), L)
    return {"fp64_fma_per_s": fma.value, "fp64_div_per_s": div.value, "fp64_atomics_per_s": atom.value}


def dw_op(op: int, a, b=None, c=None):
    """mpm_probe_dw: double-word operation op (_capi.MPM_DW_OP_*) on the FP64
    operand arrays a, b, c (each converted to double-word first); returns the
    results' (hi, lo) float parts as two float64 arrays."""
    import numpy as np

    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(np.zeros_like(a) if b is None else b, dtype=np.float64)
    c = np.ascontiguousarray(np.zeros_like(a) if c is None else c, dtype=np.float64)
    assert a.shape == b.shape == c.shape and a.ndim == 1
    out = np.empty(2 * a.size, dtype=np.float64)
    dp = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    L = _capi.lib()
    _capi.check(L.mpm_probe_dw(int(op), a.size, dp(a), dp(b), dp(c), dp(out)), L)
    return out[0::2].copy(), out[1::2].copy()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args()
    for _ in range(a.repeat):
        r = rates()
        print(f"FP64 FMA {r['fp64_fma_per_s'] / 1e9:.1f} G/s   FP64 division {r['fp64_div_per_s'] / 1e9:.1f} G/s   "
              f"FP64 atomics (L2) {r['fp64_atomics_per_s'] / 1e9:.1f} G/s")


if __name__ == "__main__":
    main()
