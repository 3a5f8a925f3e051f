"""Run a workload for a few steps, for profiling the step kernels.

  python -m jump_gb300.profile_step [--workload taylor_bar] [--precision f64]
                                    [--warmup 2] [--steps 2] [--h 2.5e-4]
                                    [--algorithm usl|musl] [--alpha 0.99]
                                    [--basis linear|quad|cubic] [--material j2|jc|jcdamage]
                                    [--sort-interval 0] [--energies]
                                    [--p2g atomic|warp|tile|tile_warp] [--threads N]
                                    [--sweep] [--stages]

--sweep: instead of the timed steps, the device ms per stage (reset, P2G,
grid, G2P; individual launches timed with CUDA events, mean of 10 steps) for
every P2G strategy x CTA size {128, 256} x sort interval {0, 4}, one JSON
line each.  --stages: after the timed steps, the same per-stage ms of the
configuration as given.

Launch order per step: p2g_kernel, grid_kernel, g2p_kernel (one each per body),
after the aos_to_soa upload launches of context creation.
"""
from __future__ import annotations

import argparse
import json
import time

from . import scenarios
from .engine import Descriptors, MPMContext


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="taylor_bar", choices=["taylor_bar", "two_disks", "cantilever"])
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "dw"])
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--h", type=float, default=2.5e-4)
    ap.add_argument("--algorithm", default="usl", choices=["usl", "musl"])
    ap.add_argument("--alpha", type=float, default=0.99)
    ap.add_argument("--basis", default="linear", choices=["linear", "quad", "cubic"])
    ap.add_argument("--material", default="j2", choices=list(scenarios.TAYLOR_MATERIALS))
    ap.add_argument("--sort-interval", type=int, default=0)
    ap.add_argument("--energies", action="store_true", help="take the EnergiesFix sums after every step")
    ap.add_argument("--p2g", default=None, choices=list(MPMContext.P2G_STRATEGIES), help="P2G strategy")
    ap.add_argument("--threads", type=int, default=None, help="CTA size of P2G and G2P")
    ap.add_argument("--sweep", action="store_true", help="stage times of every P2G strategy / CTA size / sort")
    ap.add_argument("--stages", action="store_true", help="then the device ms per stage (mean of 10 steps)")
    a = ap.parse_args()
    if a.workload == "taylor_bar":
        g, s, alg, data = scenarios.taylor_bar(h=a.h)
        scenarios.taylor_material(s[0], a.material, a.h)
    elif a.workload == "two_disks":
        g, s, alg, data = scenarios.two_disks()
    else:
        g, s, alg, data = scenarios.cantilever()
    scenarios.apply_dirichlet(g, data)
    musl = a.algorithm == "musl"
    ctx = MPMContext(Descriptors(g, s, tolerance=alg.tolerance, body_force=data.get("bodyforce"),
                                 dt=data["dt"], precision=a.precision, algorithm=a.algorithm,
                                 alpha=a.alpha if musl else 1.0, basis=a.basis, sort_interval=a.sort_interval))
    if a.p2g is not None or a.threads is not None:
        ctx.set_launch(p2g=a.p2g, threads=a.threads)
    ctx.step(a.warmup)
    if a.sweep:
        for p2g in MPMContext.P2G_STRATEGIES:
            for th in (128, 256):
                for si in (0, 4):
                    ctx.set_launch(p2g=p2g, threads=th, sort_interval=si)
                    ctx.step(2)
                    st = ctx.profile_stages(10)
                    print(json.dumps({"precision": a.precision, "p2g": p2g, "threads": th, "sort_interval": si,
                                      "stage_ms": {k: round(v / 10, 4) for k, v in st.items()}}), flush=True)
        ctx.close()
        return
    t0 = time.perf_counter()
    if a.energies:
        ctx.step_energies(a.steps, 1, 0)
    else:
        ctx.step(a.steps)
    dt = time.perf_counter() - t0
    n = sum(x.parCount for x in s)
    print(f"{a.workload} {a.precision} {a.algorithm} {a.basis} {a.material} {ctx.launch()}: {n} particles, {a.steps} steps, {1e3 * dt / max(a.steps, 1):.3f} ms/step, "
          f"device {ctx.last_step_ms() / max(a.steps, 1):.3f} ms/step")
    if a.stages:
        st = ctx.profile_stages(10)
        print(json.dumps({"stage_ms": {k: round(v / 10, 4) for k, v in st.items()}}))
    ctx.close()


if __name__ == "__main__":
    main()
