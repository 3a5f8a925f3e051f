"""Print the throughput of the operations the step kernels are bound by on the
current GPU (mpm_probe_rates): FP64 fused multiply-adds, FP64 divisions and
FP64 atomic additions executed in L2.

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
