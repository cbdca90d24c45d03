"""Time every node-block SpMV form on this GPU for jittered LSpace cantilevers.

    python -m oofem_gb300.spmv_sweep [--sizes 100x20x20,200x40x40,290x58x58]

For each mesh and precision it runs one LinearStatic solve to 1e-8 per form
(OGB_OPT_SPMV_VARIANT 1..6, 0 = the library's own choice of the full-copy form,
and 8 = the half-stored FP32 operator of mixed solves) after a warm-up
solve, with kernel timing on, and prints one JSON line per run: the step time,
the PCG iterations and the mean device time and bandwidth of the sampled SpMV
launches. This is how the split rule and the autotuner's candidate forms in
csrc/solver.cu were chosen; rerun it on other hardware to check them."""
from __future__ import annotations

import argparse
import json
import time

from . import meshgen as mg
from . import native

FORMS = {1: "plain loop", 2: "prefetch 1", 3: "prefetch 4", 4: "TMA-staged", 5: "2 warps per slice",
         6: "4 warps per slice", 0: "library choice", 8: "half-stored (mixed only)"}


def sweep(sizes, device=0):
    for dims in sizes:
        mesh = mg.hex_cantilever(*dims, h=0.05, jitter=0.2, seed=0)
        ctx = native.Context(device)
        model = native.GpuModel(ctx, mesh)
        A = native.GpuCsrMtrx(ctx)
        model.build_matrix(A)
        for prec in (native.PREC_MIXED, native.PREC_FP64):
            for v in (1, 2, 3, 4, 5, 6, 0, 8):
                if v == 8 and prec != native.PREC_MIXED:
                    continue
                # 8: the half-stored FP32 operator (OGB_OPT_SPMV_HALF 2); the others the full copy
                ctx.set_option(native.OPT_SPMV_VARIANT, 0 if v == 8 else v)
                ctx.set_option(native.OPT_SPMV_HALF, 2 if v == 8 else 0)
                model.linear_static(A, rtol=1e-8, maxit=200000, precision=prec)
                ctx.profile(True)
                ctx.profile_read()
                t0 = time.perf_counter()
                _, _, info = model.linear_static(A, rtol=1e-8, maxit=200000, precision=prec)
                dt = time.perf_counter() - t0
                ms, n, by = ctx.profile_read()
                ctx.profile(False)
                yield dict(mesh="x".join(map(str, dims)), precision="mixed" if prec else "fp64", form=FORMS[v],
                           variant=v, step_ms=round(dt * 1e3, 3), iterations=info.iterations,
                           spmv_us=round(1e3 * ms / max(n, 1), 2),
                           spmv_gbs=round((by / n) / (ms / n * 1e-3) / 1e9, 1) if n else None)
        A.close()
        model.close()
        ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="100x20x20,200x40x40,290x58x58")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    sizes = [tuple(int(v) for v in s.split("x")) for s in args.sizes.split(",")]
    for row in sweep(sizes, args.device):
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
