"""Benchmark: linear-static solve of the large jittered LSpace cantilever.

Workload (one step): the 290x58x58 LSpace hex cantilever (h = 0.05 m, interior
nodes jittered +-0.2h, seed 0; E = 210e9, nu = 0.3; x = 0 face fixed; 1e5 N in
-z over the x = L face), 3,028,470 free DOFs. A step is the LinearStatic
sequence on the GPU: element stiffness + deterministic assembly, load vector
(f_ext - f_int of the prescribed field), mixed-precision PCG (half-stored FP32
operator, FP32 block Jacobi) with FP64 residual replacements to
||f - K u||/||f|| <= 1e-8 (FP64 residual), solution scatter and reactions; the
FP64 drop-in solve is timed beside it. value = free DOFs / step time (DOF/s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs independent replicas, one per GPU (the path has no exchange step).

  python bench.py --workload rve_batch

measures the batched solve instead: 256 PlaneStress2d RVEs (sides uniform in
32..256 from seed 0, inclusions E = 300e9 at area fraction 0.3 in a matrix
E = 30e9), three prescribed-strain load cases each, one batched mixed-precision
PCG to 1e-8 for all 768 (RVE, load case) pairs (the batched FP64 PCG beside it);
value = free DOFs x load cases / step. `--workload mises_block` (J2 plasticity,
10 NonLinearStatic increments), `--workload idm1_batch` (IDM1 damage on tets, a
batch of seeds), `--workload solvers` (every linear solver of the reference on
smaller cantilevers) and `--workload spmv_forms` (every SpMV loop form) are
described in their functions.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF/s to 1e-8 rel residual, mixed-prec+IR vs FP64 GPU; assembly+SpMV HBM GB/s"
SPMV_FORMS = {1: "plain loop", 2: "columns prefetched 1 ahead", 3: "columns prefetched 4 ahead", 4: "TMA-staged",
              8: "half-stored: upper blocks streamed, lower blocks applied as transposes"}
HALF_FORMS = {1: "groups of 8 blocks, registers for 4 blocks per SM (64)",
              2: "groups of 8 blocks, registers for 3 blocks per SM (80)",
              3: "groups of 8 blocks, registers for 2 blocks per SM (128)",
              4: "values of 4 blocks loaded before their products, 3 blocks per SM (80)",
              5: "values of 3 blocks loaded before their products, 4 blocks per SM (64)",
              6: "values of 2 blocks loaded before their products, 5 blocks per SM (48)"}
WORKLOAD = dict(nx=290, ny=58, nz=58, h=0.05, jitter=0.2, seed=0)
RTOL = 1e-8


def dist_env():
    from oofem_gb300 import replicas
    return replicas.env()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


ARGS = None


def apply_options(ctx):
    """Library options given on the command line (defaults: the library's)."""
    from oofem_gb300 import native
    if ARGS is not None and ARGS.mixed_x64 >= 0:
        ctx.set_option(native.OPT_MIXED_X64, ARGS.mixed_x64)
    if ARGS is not None and ARGS.block_jacobi >= 0:
        ctx.set_option(native.OPT_MIXED_BLOCK_JACOBI, ARGS.block_jacobi)
    if ARGS is not None and ARGS.tangent_tc >= 0:
        ctx.set_option(native.OPT_TANGENT_TC, ARGS.tangent_tc)
    if ARGS is not None and ARGS.half_form >= 0:
        ctx.set_option(native.OPT_HALF_FORM, ARGS.half_form)
    if ARGS is not None and ARGS.update_blocks >= 0:
        ctx.set_option(native.OPT_UPDATE_BLOCKS, ARGS.update_blocks)
    if ARGS is not None and ARGS.fused_update >= 0:
        ctx.set_option(native.OPT_FUSED_UPDATE, ARGS.fused_update)
    if ARGS is not None and ARGS.batch_x64 >= 0:
        ctx.set_option(native.OPT_BATCH_X64, ARGS.batch_x64)


def profile_traffic(form: int):
    """DRAM bytes per SpMV launch of this form from the committed ncu summary (if any)."""
    p = os.path.join(ROOT, "profiles", "spmv_half_traffic.json" if form % 10 == 8 else "spmv_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except ValueError:
            return None
    return None


# ----------------------------------------------------------------------------- CPU side
class CpuFull:
    """The oracle (a C restatement of the reference path: equation numbering,
    location arrays, CompCol-style pattern, element stiffness + scatter assembly,
    IML CG with the diagonal preconditioner) on the full workload mesh: the
    pattern and the assembly are timed once, CG iterations on the full matrix are
    timed per sample, and the time to 1e-8 is the assembly plus the FP64
    iteration count of the workload times the time per iteration (the only
    scaling: running the ~3,000 iterations would take half an hour)."""

    def __init__(self):
        from oofem_gb300 import meshgen as mg
        from oracle import oracle as O
        self.O = O
        sm = mg.hex_cantilever(WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["nz"], h=WORKLOAD["h"],
                               jitter=WORKLOAD["jitter"], seed=WORKLOAD["seed"])
        md = O.mesh_dict(sm)
        t0 = time.perf_counter()
        neq, _, eq = O.number_equations(sm.bc_mask)
        loc = O.location_arrays(sm.conn, eq)
        self.rp, self.ci = O.build_pattern(neq, loc)
        t1 = time.perf_counter()
        self.val = O.assemble_tangent(md, loc, neq, self.rp, self.ci)
        t2 = time.perf_counter()
        self.t_pattern, self.t_assembly = t1 - t0, t2 - t1
        self.b = np.zeros(neq)
        free = eq > 0
        self.b[eq[free] - 1] = sm.nodal_load[free]
        self.neq, self.nelem, self.nnz = neq, sm.nelem, int(self.ci.size)
        self.threads = O.threads()

    def cg_seconds_per_iteration(self, n_it: int) -> float:
        t0 = time.perf_counter()
        self.O.pcg(self.rp, self.ci, self.val, self.b, rtol=1e-30, maxit=n_it)
        return (time.perf_counter() - t0) / n_it

    def baseline(self, t_it: float, iters_full: int, iters_src: str, n_it: int) -> dict:
        t_full = self.t_pattern + self.t_assembly + iters_full * t_it
        return {"value": self.neq / t_full, "unit": "DOF/s", "cores": self.threads, "kind": "port",
                "sample": (f"oracle (C restatement of the reference path) on the full workload mesh "
                           f"({self.neq} DOFs, {self.nelem} elements, nnz {self.nnz}): pattern {self.t_pattern:.1f} s "
                           f"(serial) and assembly {self.t_assembly:.1f} s (element matrices on {self.threads} OpenMP "
                           f"threads as the reference's element loop, added in element order), "
                           f"CG {t_it:.3f} s per iteration single-threaded (as the "
                           f"reference's IML CG) timed over {n_it} iterations on the full matrix, times the "
                           f"{iters_full} FP64 Jacobi-PCG iterations the workload needs to 1e-8 ({iters_src})"),
                "seconds_to_solution": t_full}


def cpu_sample(iters_full: int, n_it: int = 2) -> dict:
    """cpu_baseline of the GPU arm: one CpuFull measurement."""
    cf = CpuFull()
    t_it = cf.cg_seconds_per_iteration(n_it)
    out = cf.baseline(t_it, iters_full, "measured by this run's FP64 solve", n_it)
    del cf
    return out


def fp64_iterations():
    """FP64 Jacobi-PCG iterations to 1e-8 on the full workload, as measured on a
    GB300 by this bench (same algorithm as the reference's IML CG)."""
    p = os.path.join(ROOT, "profiles", "bench_workload.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return int(d["fp64_iterations"]), "measured"
    return 6000, "assumed"


def run_reference(args):
    """The reference arm: the oracle port of the reference's CPU path on the full
    workload (see CpuFull); each step times CG iterations on the full matrix."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    iters, src = fp64_iterations()
    cf = CpuFull()
    n_it = 2
    secs = []
    for k in range(args.warmup + args.steps):
        t_it = cf.cg_seconds_per_iteration(n_it)
        if k >= args.warmup:
            secs.append(t_it)
    t_it = statistics.median(secs)
    cb = cf.baseline(t_it, iters, src, n_it)
    v = cb["value"]
    t_full = cb.pop("seconds_to_solution")
    out = {"metric": METRIC, "value": v, "unit": "DOF/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t_full, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": "hex_cantilever_%dx%dx%d_jitter0.2_seed0" % (WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["nz"]),
                      "free_dofs": cf.neq, "elements": cf.nelem, "nnz": cf.nnz, "rtol": RTOL},
           "step": f"{n_it} CG iterations on the full matrix per step; ms_per_step = the time to 1e-8 it implies",
           "cpu_baseline": cb,
           "e2e": {"value": v, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ----------------------------------------------------------------------------- GPU side
def run_gpu(args):
    import torch
    from oofem_gb300 import meshgen as mg, native

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from oofem_gb300 import replicas
    barrier = replicas.barrier

    if args.nx:
        WORKLOAD.update(nx=args.nx, ny=args.ny, nz=args.nz)
    mesh = mg.hex_cantilever(WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["nz"], h=WORKLOAD["h"],
                             jitter=WORKLOAD["jitter"], seed=WORKLOAD["seed"] + rank)
    nfree = mesh.nfree
    ctx = native.Context(local)
    apply_options(ctx)
    if args.spmv_variant:
        ctx.set_option(native.OPT_SPMV_VARIANT, args.spmv_variant)
    ctx.set_option(native.OPT_SPMV_HALF, args.spmv_half)
    model = native.GpuModel(ctx, mesh)
    A = native.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    nnz = A.nnz
    bcv = torch.from_numpy(mesh.bc_value.ravel()).to(dev)
    load = torch.from_numpy(mesh.nodal_load.ravel()).to(dev)
    u = torch.zeros_like(bcv)
    reac = torch.zeros_like(bcv)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    lib = ctx.lib
    import ctypes as C

    def step(prec):
        info = native.SolveInfo()
        code = lib.ogb_linear_static_dev(model.h, A.h, C.c_void_p(bcv.data_ptr()), C.c_void_p(load.data_ptr()),
                                         RTOL, 200000, prec, C.c_void_p(u.data_ptr()),
                                         C.c_void_p(reac.data_ptr()), C.byref(info))
        if code != 0:
            raise native.OgbError(code, lib.ogb_last_error().decode())
        return info

    def timed(prec, k, w, profile=False):
        for _ in range(w):
            step(prec)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        if profile:
            ctx.profile(True)
            ctx.profile_read()
        l0 = ctx.kernel_launches()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        infos = []
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for _ in range(k):
                infos.append(step(prec))
            ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / k
        launches = (ctx.kernel_launches() - l0) / k
        prof = ctx.profile_read() if profile else None
        if profile:
            ctx.profile(False)
        return ms, infos, launches, prof

    clocks = ClockSampler(local)
    clocks.start()
    ms, infos, launches, prof = timed(native.PREC_MIXED, args.steps, args.warmup, profile=True)
    clk = clocks.stop()

    def fields():
        """Node displacements, reactions and GP stresses of the last step (host copies)."""
        fn = torch.zeros_like(bcv)
        lib.ogb_model_internal_forces_dev(model.h, C.c_void_p(u.data_ptr()), C.c_void_p(fn.data_ptr()))
        sig, _ = model.gp_stress()
        return u.cpu().numpy().copy(), reac.cpu().numpy().copy(), sig
    u_m, r_m, s_m = fields()
    # FP64 drop-in path: iteration count and DOF/s for the mixed/FP64 ratio
    ms64, infos64, _, _ = timed(native.PREC_FP64, 1, 1)
    u_6, r_6, s_6 = fields()

    def relerr(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
    accuracy = {"u_rel": relerr(u_m, u_6), "reactions_rel": relerr(r_m, r_6), "gp_stress_rel": relerr(s_m, s_6),
                "measure": "max |mixed - FP64| / max |FP64| over all nodes (u, reactions) and Gauss points "
                           "(stress); both solves to ||f - K u|| / ||f|| <= 1e-8 (FP64 residual)"}
    del s_m, s_6

    # element evaluations: stiffness (K1) + deterministic gather assembly (K4),
    # and internal forces (K2 + node gather), CUDA events on the library stream
    def stream_ms(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    fnode = torch.zeros_like(bcv)
    ms_k = stream_ms(lambda: lib.ogb_model_assemble_stiffness(model.h, A.h))
    ms_f = stream_ms(lambda: lib.ogb_model_internal_forces_dev(model.h, C.c_void_p(u.data_ptr()),
                                                               C.c_void_p(fnode.data_ptr())))
    nnpe, nd = mesh.nnpe, mesh.ndofpn
    ke_bytes = mesh.nelem * (nnpe * nd) ** 2 * 8
    # K1 writes every element matrix once, K4 reads it once and writes the CSR
    # values and both node-block copies (FP64 + FP32) once
    asm_bytes = 2 * ke_bytes + nnz * (8 + 8 + 4)
    elements = {"stiffness_assembly_ms": ms_k, "element_stiffness_per_s": mesh.nelem / (ms_k * 1e-3),
                "stiffness_assembly_gbs": asm_bytes / (ms_k * 1e-3) / 1e9,
                "internal_forces_ms": ms_f, "element_force_evals_per_s": mesh.nelem / (ms_f * 1e-3)}
    # replicas: total free DOFs of all ranks over the slowest rank's step time
    value = replicas.job_throughput(nfree, ms * 1e-3)
    ms = replicas.max_over_ranks(ms)

    # end to end through the host API: mesh upload, pattern, assembly, solve, copy back;
    # the inputs and the result buffers live in page-locked host memory
    keep = []

    def pinned(a):
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        keep.append(t)
        v = t.numpy()
        v[...] = a
        return v
    mesh_h = dataclasses.replace(mesh, coords=pinned(mesh.coords), conn=pinned(mesh.conn),
                                 elem_mat=pinned(mesh.elem_mat), bc_mask=pinned(mesh.bc_mask),
                                 bc_value=pinned(mesh.bc_value), nodal_load=pinned(mesh.nodal_load))
    out_h = (pinned(np.zeros_like(mesh.bc_value)), pinned(np.zeros_like(mesh.bc_value)))

    def e2e_once():
        c2 = native.Context(local)
        m2 = native.GpuModel(c2, mesh_h)
        A2 = native.GpuCsrMtrx(c2)
        uh, rh, info = m2.linear_static(A2, rtol=RTOL, maxit=200000, precision=native.PREC_MIXED, out=out_h)
        A2.close()
        m2.close()
        c2.close()
        return info
    e2e_s = float("nan")
    if not args.no_e2e:
        e2e_once()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n_e2e = 2
        for _ in range(n_e2e):
            e2e_once()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / n_e2e
    if not args.no_e2e:
        e2e_s = replicas.max_over_ranks(e2e_s)
    # where the end-to-end time goes: one more call, outside the timed runs, with the host
    # clock read after each phase (every phase below returns with its work finished)
    phases = None
    if not args.no_e2e:
        t = [time.perf_counter()]
        c2 = native.Context(local)
        t.append(time.perf_counter())
        m2 = native.GpuModel(c2, mesh_h)
        A2 = native.GpuCsrMtrx(c2)
        c2.synchronize()
        t.append(time.perf_counter())
        m2.linear_static(A2, rtol=RTOL, maxit=200000, precision=native.PREC_MIXED, out=out_h)
        t.append(time.perf_counter())
        A2.close()
        m2.close()
        c2.close()
        t.append(time.perf_counter())
        phases = {k: (t[i + 1] - t[i]) * 1e3 for i, k in enumerate(
            ("context", "mesh_upload", "assemble_solve_copy_back", "release"))}
    h2d = (mesh.coords.nbytes + mesh.conn.nbytes + mesh.elem_mat.nbytes + mesh.material_table().nbytes
           + mesh.bc_mask.nbytes + mesh.bc_value.nbytes + mesh.nodal_load.nbytes)
    d2h = 2 * mesh.bc_value.nbytes

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    sp_ms, sp_n, sp_bytes = prof
    achieved = (sp_bytes / sp_n) / (sp_ms / sp_n * 1e-3) / 1e9 if sp_n else None
    f32_form = A.spmv_forms()[1]
    traffic = profile_traffic(f32_form)
    nblocks = nnz / (mesh.ndofpn ** 2)
    full_bytes = nnz * 4 + nblocks * 4 + 2 * 4 * nfree
    info = infos[-1]
    cb = None
    if ws == 1 and not args.no_cpu:
        cb = cpu_sample(infos64[-1].iterations)
        cb.pop("seconds_to_solution", None)
    out = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": "hex_cantilever_%dx%dx%d_jitter0.2_seed0" % (WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["nz"]),
                   "free_dofs": nfree,
                   "elements": mesh.nelem, "nnz": nnz, "rtol": RTOL, "precision": "mixed FP32 PCG + FP64 IR",
                   "l2": "inputs larger than L2 (FP32 node-block matrix %.2f GB, FP64 %.2f GB)" % (
                       nnz * 4.44 / 1e9, nnz * 8.44 / 1e9),
                   "parallelism": f"replicas x{ws}"},
        "solve": {"inner_iterations": info.iterations, "outer": info.outer, "achieved": info.achieved},
        "fp64": {"value": nfree / (ms64 * 1e-3), "ms_per_step": ms64, "iterations": infos64[-1].iterations,
                 "achieved": infos64[-1].achieved},
        "mixed_over_fp64": ms64 / ms,
        "mixed_vs_fp64_accuracy": accuracy,
        "preconditioner": "block Jacobi (FP32 3x3 node blocks)" if A.last_block_jacobi() else "Jacobi (diagonal)",
        "roofline": {"bound": "hbm", "kernel": ("k_half_spmv" if f32_form % 10 == 8 else "k_sell_spmv") +
                     " (node-block SELL-32, FP32 values, difference form, fused p.q; form %s)" %
                     (SPMV_FORMS[8] + ", " + HALF_FORMS.get(f32_form // 10, "?") if f32_form % 10 == 8
                      else SPMV_FORMS.get(f32_form, "?")),
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_kind": peak_kind,
                     "traffic": traffic.get("dram_bytes_per_launch") if traffic else None,
                     "spmv_launches_per_step": sp_n / args.steps if sp_n else 0,
                     "spmv_ms_per_step": sp_ms / args.steps if sp_n else 0,
                     # the same operator applied from the full FP32 node-block copy moves every stored
                     # block once: values + block columns + x + y (what a plain SpMV of K needs)
                     "full_copy_bytes": full_bytes,
                     "effective_frac": (full_bytes / (sp_ms / sp_n * 1e-3) / 1e9 / peak) if sp_n else None,
                     "effective_frac_note": "bytes of the full-copy SpMV of the same operator / measured time / "
                                            "peak: the half-stored form applies K at this fraction of the "
                                            "copy-bound time of a full-copy SpMV; frac counts its own bytes"},
        "elements": elements,
        "clocks": clk,
        "gpu_launches": int(launches),
        "e2e": {"value": ws * nfree / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds": e2e_s, "phases_ms": phases},
        "cpu_baseline": cb,
    }
    print(json.dumps(out))


def spmv_sample_roofline(ctx, work, f32_form):
    """Roofline of the mixed solves' FP32 SpMV from the library's kernel timing
    (CUDA events on its stream around sampled launches, with the algorithmic
    bytes of each) over one more run of `work`, outside the timed region.
    f32_form: the matrix's reported SpMV form, or a callable giving it after
    `work` (None: the batched SpMV)."""
    ctx.profile(True)
    ctx.profile_read()
    work()
    sp_ms, sp_n, sp_bytes = ctx.profile_read()
    ctx.profile(False)
    peak, peak_kind = measured_peaks()
    gbs = (sp_bytes / sp_n) / (sp_ms / sp_n * 1e-3) / 1e9 if sp_n else None
    if callable(f32_form):
        f32_form = f32_form()
    if f32_form is None:
        kernel = "k_bspmv (node-block SELL-32, FP32 values, difference form, right-hand sides interleaved, fused p.q)"
    elif f32_form % 10 == 8:
        kernel = "k_half_spmv (half-stored node-block SELL-32, FP32 values, difference form, fused p.q; form %s)" % (
            HALF_FORMS.get(f32_form // 10, "?"))
    else:
        kernel = "k_sell_spmv (node-block SELL-32, FP32 values; form %s)" % SPMV_FORMS.get(f32_form, "?")
    return {"bound": "hbm", "kernel": kernel, "achieved": gbs, "peak": peak, "unit": "GB/s",
            "frac": gbs / peak if gbs else None, "peak_kind": peak_kind, "traffic": None,
            "bytes_per_launch": sp_bytes / sp_n if sp_n else None,
            "ms_per_launch": sp_ms / sp_n if sp_n else None, "sampled_launches": sp_n}


def run_gpu_batch(args):
    """256-RVE sweep with three load cases per RVE through the batched solve."""
    import ctypes as C
    import torch
    from oofem_gb300 import meshgen as mg, native

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nrve, nrhs = args.rve_count, 3
    meshes = mg.rve_batch(nrve, seed=rank)
    big, ns = mg.concat_meshes(meshes)
    nfree = big.nfree
    bcv_h = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(nrhs)])
    ctx = native.Context(local)
    apply_options(ctx)
    model = native.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    lib = ctx.lib
    bcv = torch.from_numpy(bcv_h.ravel()).to(dev)
    u = torch.zeros_like(bcv)
    reac = torch.zeros_like(bcv)
    its = np.zeros(nrve * nrhs, np.int32)
    ach = np.zeros(nrve * nrhs)
    st = np.zeros(nrve * nrhs, np.int32)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def step(prec):
        code = lib.ogb_batch_linear_static_dev(model.h, A.h, nrhs, C.c_void_p(bcv.data_ptr()), None, RTOL, 200000,
                                               prec, C.c_void_p(u.data_ptr()), C.c_void_p(reac.data_ptr()),
                                               its.ctypes.data_as(C.c_void_p), ach.ctypes.data_as(C.c_void_p),
                                               st.ctypes.data_as(C.c_void_p))
        if code != 0:
            raise native.OgbError(code, lib.ogb_last_error().decode())

    def timed(prec, k, w):
        for _ in range(w):
            step(prec)
        torch.cuda.synchronize()
        l0 = ctx.kernel_launches()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for _ in range(k):
                step(prec)
            ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / k, (ctx.kernel_launches() - l0) / k, its.copy(), ach.copy(), st.copy()

    clocks = ClockSampler(local)
    clocks.start()
    ms, launches, its_m, ach_m, st_m = timed(native.PREC_MIXED, args.steps, args.warmup)
    clk = clocks.stop()
    ms64, _, its64, ach64, st64 = timed(native.PREC_FP64, 1, 1)
    value = nfree * nrhs / (ms * 1e-3)
    # the dominant kernel (batched FP32 SpMV) timed outside the timed steps: with
    # kernel timing on, each batched mixed solve times one launch of its chosen
    # form with every (RVE, load case) pair running
    roofline = spmv_sample_roofline(ctx, lambda: [step(native.PREC_MIXED) for _ in range(2)], None)
    roofline["sample"] = ("one launch per mixed solve with every pair running; launches late in a solve skip "
                          "the RVEs whose pairs have finished")
    # end to end through the host API (host arrays in and out, model upload included)
    e2e_s = float("nan")
    if not args.no_e2e:
        t0 = time.perf_counter()
        c2 = native.Context(local)
        m2 = native.GpuModel(c2, big)
        m2.set_instances(ns)
        A2 = native.GpuCsrMtrx(c2)
        m2.batch_linear_static(A2, bcv_h, rtol=RTOL, maxit=200000, precision=native.PREC_MIXED)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        A2.close()
        m2.close()
        c2.close()
    h2d = (big.coords.nbytes + big.conn.nbytes + big.elem_mat.nbytes + big.material_table().nbytes
           + big.bc_mask.nbytes + bcv_h.nbytes)
    d2h = 2 * bcv_h.nbytes
    cb = None
    if not args.no_cpu:
        from oracle import oracle as O
        t0 = time.perf_counter()
        done_dofs = 0
        k = 0
        while k < nrve and (time.perf_counter() - t0) < 15.0:
            md = O.mesh_dict(meshes[k])
            for lc in range(nrhs):
                md["bc_value"] = mg.rve_bc_values(meshes[k], lc)
                O.linear_static(md, rtol=RTOL)
            done_dofs += meshes[k].nfree * nrhs
            k += 1
        t_cpu = time.perf_counter() - t0
        cb = {"value": done_dofs / t_cpu, "unit": "DOF/s", "cores": 1, "kind": "port",
              "sample": f"oracle LinearStatic (serial C) on the first {k} RVEs of the batch x {nrhs} load cases"}
    out = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": f"rve_batch_{nrve}x{nrhs}rhs_sides32-256_seed{rank}", "rves": nrve,
                   "load_cases": nrhs, "free_dofs": nfree, "elements": big.nelem, "nnz": A.nnz, "rtol": RTOL,
                   "precision": "mixed FP32 batched PCG + FP64 residual replacement",
                   "l2": "inputs larger than L2 (FP32 matrix %.2f GB)" % (A.nnz * 4.5 / 1e9)},
        "solve": {"max_iterations": int(its_m.max()), "mean_iterations": float(its_m.mean()),
                  "all_converged": bool((st_m == 0).all()), "max_achieved": float(ach_m.max())},
        "fp64": {"value": nfree * nrhs / (ms64 * 1e-3), "ms_per_step": ms64, "max_iterations": int(its64.max()),
                 "mean_iterations": float(its64.mean()), "all_converged": bool((st64 == 0).all())},
        "mixed_over_fp64": ms64 / ms,
        "roofline": roofline,
        "clocks": clk, "gpu_launches": int(launches),
        "e2e": {"value": nfree * nrhs / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds": e2e_s},
        "cpu_baseline": cb,
    }
    print(json.dumps(out))


def run_gpu_newton(args):
    """J2 plasticity block: MisesMat (E 210e9, nu 0.3, yield 250e6, H 2e9), x = 0
    face fixed, x = L face pulled to 3 yield strains over 10 increments, each a
    NonLinearStatic step (initialguess 1) with full Newton (tangent every
    iteration) to rtolf 1e-8; linear systems by mixed-precision PCG to 1e-8.
    value = free DOFs x steps / time of the 10-step analysis."""
    import torch
    from oofem_gb300 import meshgen as mg, native

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    nx, ny, nz = args.nx or 185, args.ny or 37, args.nz or 37
    h, nsteps = 0.05, 10
    eps_y = 250e6 / 210e9
    mesh = mg.hex_block_pull(nx, ny, nz, h=h, end_disp=3.0 * eps_y * nx * h)
    nfree = mesh.nfree
    ctx = native.Context(local)
    apply_options(ctx)
    model = native.GpuModel(ctx, mesh)
    model.set_initial_guess(1)   # IG_Tangent, as for changing Dirichlet values
    A = native.GpuCsrMtrx(ctx)
    model.build_matrix(A)

    def analysis(prec):
        model.reset_state()
        nites = []
        for k in range(1, nsteps + 1):
            _, _, nite = model.nonlinear_step(A, mesh.bc_value * (k / nsteps), None, rtolf=1e-8, maxiter=50,
                                              lin_rtol=1e-8, precision=prec)
            nites.append(nite)
        return nites, model.solver_stats()

    analysis(native.PREC_MIXED)   # warm-up: autotuning, graph capture, allocations
    torch.cuda.synchronize()
    used_tc = model.tangent_kernel()[0]
    # element tangent kernels of this state, CUDA events on the library stream
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def tangent_ms(prec, reps=3):
        model.assemble_tangent(A, prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                model.assemble_tangent(A, prec)
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    ms64 = tangent_ms(native.PREC_FP64)
    ctx.set_option(native.OPT_TANGENT_TC, 1)
    ms_tc = tangent_ms(native.PREC_MIXED)
    ctx.set_option(native.OPT_TANGENT_TC, args.tangent_tc if args.tangent_tc >= 0 else 0)
    tangent = {"assembly_ms_fp64_kernel": ms64, "assembly_ms_tensor_core_kernel": ms_tc,
               "mixed_steps_used": "tensor cores (split-BF16 tcgen05)" if used_tc else "FP64 CUDA cores",
               "note": "tangent assembly of the converged state (element kernel + deterministic gather into the "
                       "CSR and node-block copies), CUDA events; the tensor-core kernel is FP32-accurate and off "
                       "by default in mixed steps (OGB_OPT_TANGENT_TC)"}
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.kernel_launches()
    t0 = time.perf_counter()
    nites, lin = analysis(native.PREC_MIXED)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    launches = ctx.kernel_launches() - l0
    clk = clocks.stop()
    t0 = time.perf_counter()
    nites64, lin64 = analysis(native.PREC_FP64)
    torch.cuda.synchronize()
    secs64 = time.perf_counter() - t0
    # the FP32 SpMV of the mixed solves timed in one more first increment, outside the timed analysis
    def first_increment():
        model.reset_state()
        model.nonlinear_step(A, mesh.bc_value * (1.0 / nsteps), None, rtolf=1e-8, maxiter=50, lin_rtol=1e-8,
                             precision=native.PREC_MIXED)
    roofline = spmv_sample_roofline(ctx, first_increment, lambda: A.spmv_forms()[1])
    cb = None
    if not args.no_cpu:
        from oracle import oracle as O
        sm = mg.hex_block_pull(20, 4, 4, h=h, end_disp=3.0 * eps_y * 20 * h)
        md = O.mesh_dict(sm)
        t0 = time.perf_counter()
        O.nonlinear_static(md, [float(k) for k in range(1, nsteps + 1)], float(nsteps), 1e-8, 50, initial_guess=1)
        tc = time.perf_counter() - t0
        cb = {"value": sm.nfree * nsteps / tc, "unit": "DOF/s", "cores": 1, "kind": "port",
              "sample": f"oracle NonLinearStatic/NRSolver (serial C + numpy) on the 20x4x4 block ({sm.nfree} DOFs), "
                        f"same material and ramp, {nsteps} steps"}
    out = {
        "metric": METRIC, "value": nfree * nsteps / secs, "unit": "DOF/s", "n_gpus": 1, "steps": nsteps,
        "warmup": 1, "ms_per_step": 1e3 * secs / nsteps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": f"mises_block_{nx}x{ny}x{nz}_10_increments", "free_dofs": nfree,
                   "elements": mesh.nelem, "rtolf": 1e-8, "lin_rtol": 1e-8,
                   "precision": "FP64 radial return and residual, mixed FP32 PCG + FP64 refinement"},
        "newton_iterations": nites, "linear_solves": lin[0], "pcg_iterations": lin[1],
        "fp64": {"value": nfree * nsteps / secs64, "seconds": secs64, "newton_iterations": nites64,
                 "linear_solves": lin64[0], "pcg_iterations": lin64[1]},
        "mixed_over_fp64": secs64 / secs, "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
        "tangent": tangent,
        "timing": "host wall clock around the 10-step analysis (device synchronized)",
        "cpu_baseline": cb,
    }
    print(json.dumps(out))


def run_gpu_idm1_batch(args):
    """Damage on tets, a batch of seeds: unit cube of n^3 cells x 6 LTRSpace tets
    per seed (nodes jittered +-0.15h, seed-dependent), IsotropicDamageMaterial1
    (E 30e9, nu 0.2, e0 1e-4, gf 100), z = 0 fixed, z = 1 pulled to 4 e0 over 20
    increments; the batch takes the first `--idm-steps` increments (the pre-peak
    part, before the softening steps that need hundreds of Newton iterations) as
    batched NonLinearStatic steps, each seed with its own NRSolver test (rtolf
    1e-6), linear systems by mixed-precision batched PCG to 1e-8.
    value = free DOFs of all seeds x steps / time."""
    import torch
    from oofem_gb300 import meshgen as mg, native

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    n, nseed, nsteps, run = args.cube_n, args.seeds, 20, args.idm_steps
    mat = mg.Material(mg.MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=100.0)
    meshes = [mg.tet_cube(n, jitter=0.15, seed=100 * rank + k, material=mat, end_disp=4e-4) for k in range(nseed)]
    big, ns = mg.concat_meshes(meshes)
    nfree = big.nfree
    ctx = native.Context(local)
    apply_options(ctx)
    model = native.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native.GpuCsrMtrx(ctx)
    model.build_matrix(A)

    def analysis():
        model.reset_state()
        its = []
        for k in range(1, run + 1):
            _, _, it = model.batch_nonlinear_step(A, big.bc_value * (k / nsteps), None, rtolf=1e-6, maxiter=400,
                                                  lin_rtol=1e-8, precision=native.PREC_MIXED)
            its.append(it.tolist())
        return its

    model.batch_nonlinear_step(A, big.bc_value * (1.0 / nsteps), None, rtolf=1e-6, maxiter=400, lin_rtol=1e-8,
                               precision=native.PREC_MIXED)   # warm-up
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.kernel_launches()
    t0 = time.perf_counter()
    its = analysis()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    clk = clocks.stop()
    launches = ctx.kernel_launches() - l0
    # the batched FP32 SpMV timed in one more increment (the first), outside the timed analysis
    def first_increment():
        model.reset_state()
        model.batch_nonlinear_step(A, big.bc_value * (1.0 / nsteps), None, rtolf=1e-6, maxiter=400, lin_rtol=1e-8,
                                   precision=native.PREC_MIXED)
    roofline = spmv_sample_roofline(ctx, first_increment, None)
    cb = None
    if not args.no_cpu:
        from oracle import oracle as O
        sm = mg.tet_cube(4, jitter=0.15, seed=1, material=mat, end_disp=4e-4)
        t0 = time.perf_counter()
        O.nonlinear_static(O.mesh_dict(sm), [float(k) for k in range(1, run + 1)], float(nsteps), 1e-6, 400)
        tc = time.perf_counter() - t0
        cb = {"value": sm.nfree * run / tc, "unit": "DOF/s", "cores": 1, "kind": "port",
              "sample": f"oracle NonLinearStatic/NRSolver (serial C + numpy, direct solves) on one 4^3-cell cube "
                        f"({sm.nfree} DOFs), same material and the same {run} increments"}
    out = {
        "metric": METRIC, "value": nfree * run / secs, "unit": "DOF/s", "n_gpus": 1, "steps": run,
        "warmup": 1, "ms_per_step": 1e3 * secs / run, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic",
        "config": {"workload": f"idm1_tet_cube_{n}_x{nseed}_seeds_first_{run}_of_{nsteps}_increments",
                   "free_dofs": nfree, "elements": big.nelem, "rtolf": 1e-6, "lin_rtol": 1e-8,
                   "precision": "FP64 damage update and residual, mixed FP32 batched PCG"},
        "newton_iterations_per_seed": its, "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
        "timing": "host wall clock around the analysis (device synchronized)", "cpu_baseline": cb,
    }
    print(json.dumps(out))


SWEEP_FORMS = {1: "plain loop", 2: "prefetch 1", 3: "prefetch 4", 4: "TMA-staged", 5: "2 warps per slice",
               6: "4 warps per slice", 0: "library choice", 8: "half-stored (mixed only)"}


def run_spmv_forms(args):
    """Every node-block SpMV form on this GPU (how the split rule and the
    autotuner's candidate forms were chosen): for each cantilever of
    --sweep-sizes and each precision, one warm-up LinearStatic solve to 1e-8 per
    form (OGB_OPT_SPMV_VARIANT 1..6, 0 = the library's choice of the full-copy
    form, 8 = the half-stored FP32 operator of mixed solves), then one timed solve
    with kernel timing on; one JSON line per run (step time, PCG iterations, mean
    device time and algorithmic bandwidth of the sampled SpMV launches)."""
    import time as _t
    from oofem_gb300 import meshgen as mg, native
    sizes = [tuple(int(v) for v in sz.split("x")) for sz in args.sweep_sizes.split(",")]
    for dims in sizes:
        mesh = mg.hex_cantilever(*dims, h=WORKLOAD["h"], jitter=WORKLOAD["jitter"], seed=WORKLOAD["seed"])
        ctx = native.Context(0)
        model = native.GpuModel(ctx, mesh)
        A = native.GpuCsrMtrx(ctx)
        model.build_matrix(A)
        for prec in (native.PREC_MIXED, native.PREC_FP64):
            for v in (1, 2, 3, 4, 5, 6, 0, 8):
                if v == 8 and prec != native.PREC_MIXED:
                    continue
                ctx.set_option(native.OPT_SPMV_VARIANT, 0 if v == 8 else v)
                ctx.set_option(native.OPT_SPMV_HALF, 2 if v == 8 else 0)
                model.linear_static(A, rtol=RTOL, maxit=200000, precision=prec)
                ctx.profile(True)
                ctx.profile_read()
                t0 = _t.perf_counter()
                _, _, info = model.linear_static(A, rtol=RTOL, maxit=200000, precision=prec)
                dt = _t.perf_counter() - t0
                ms, n, by = ctx.profile_read()
                ctx.profile(False)
                print(json.dumps(dict(mesh="x".join(map(str, dims)), precision="mixed" if prec else "fp64",
                                      form=SWEEP_FORMS[v], variant=v, step_ms=round(dt * 1e3, 3),
                                      iterations=info.iterations, spmv_us=round(1e3 * ms / max(n, 1), 2),
                                      spmv_gbs=round((by / n) / (ms / n * 1e-3) / 1e9, 1) if n else None)),
                      flush=True)
        A.close()
        model.close()
        ctx.close()


def run_solvers(args):
    """Linear solvers of the reference on one cantilever (--nx/--ny/--nz, default
    60x12x12), FP64: IML CG with lsprecond 1 (diagonal), 4 (incomplete Cholesky),
    2 (ILU by columns), 0 (none), each to 1e-8, the direct L D L^T (lstype 0) and
    the mixed-precision solve of this library.
    One warm-up solve, then one timed LinearStatic step per solver (host wall
    clock, device synchronized); one JSON line per solver."""
    from oofem_gb300 import meshgen as mg, native
    nx, ny, nz = args.nx or 60, args.ny or 12, args.nz or 12
    mesh = mg.hex_cantilever(nx, ny, nz, h=WORKLOAD["h"], jitter=WORKLOAD["jitter"], seed=WORKLOAD["seed"])
    for name, lstype, prec, pr in (("CG + diagonal (lsprecond 1)", 1, 1, native.PREC_FP64),
                                   ("CG + incomplete Cholesky (lsprecond 4)", 1, 4, native.PREC_FP64),
                                   ("CG + ILU by columns (lsprecond 2)", 1, 2, native.PREC_FP64),
                                   ("CG, no preconditioner (lsprecond 0)", 1, 0, native.PREC_FP64),
                                   ("direct L D L^T (lstype 0)", 0, 1, native.PREC_FP64),
                                   ("mixed: FP32 block-Jacobi PCG + FP64 residual replacement", 1, 1,
                                    native.PREC_MIXED)):
        ctx = native.Context(0)
        apply_options(ctx)
        model = native.GpuModel(ctx, mesh)
        A = native.GpuCsrMtrx(ctx)
        A.set_solver(native.LS_DIRECT if lstype == 0 else native.LS_IML)
        A.set_preconditioner(prec)
        model.linear_static(A, rtol=RTOL, maxit=1000000, precision=pr)
        ctx.synchronize()
        t0 = time.perf_counter()
        u, reac, info = model.linear_static(A, rtol=RTOL, maxit=1000000, precision=pr)
        ctx.synchronize()
        dt = time.perf_counter() - t0
        rec = {"mesh": f"{nx}x{ny}x{nz}", "free_dofs": mesh.nfree, "solver": name, "step_ms": 1e3 * dt,
               "iterations": info.iterations, "achieved": info.achieved, "status": info.status}
        if lstype == 1:
            # the same matrix again, its preconditioner kept (same version): the
            # iterations alone, per iteration
            neq = A.neq
            sol = native.GpuPcgSolver(lstol=RTOL, lsiter=1000000, precision=pr, lsprecond=prec)
            bb = np.ones(neq)
            xx = np.zeros(neq)
            ctx.synchronize()
            t0 = time.perf_counter()
            sol.solve(A, bb, xx)
            ctx.synchronize()
            ds = time.perf_counter() - t0
            if sol.last.iterations > 0:
                rec["ms_per_iteration_kept_preconditioner"] = 1e3 * ds / sol.last.iterations
        print(json.dumps(rec), flush=True)
        A.close()
        model.close()
        ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--nx", type=int, default=0, help="profiling only: smaller cantilever")
    ap.add_argument("--ny", type=int, default=0)
    ap.add_argument("--nz", type=int, default=0)
    ap.add_argument("--workload", default="cantilever",
                    choices=["cantilever", "rve_batch", "mises_block", "idm1_batch", "spmv_forms", "solvers"])
    ap.add_argument("--sweep-sizes", default="100x20x20,200x40x40,290x58x58",
                    help="spmv_forms: cantilevers to sweep")
    ap.add_argument("--cube-n", type=int, default=40)
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--idm-steps", type=int, default=16)
    ap.add_argument("--rve-count", type=int, default=256)
    ap.add_argument("--spmv-variant", type=int, default=0,
                    help="profiling only: force a node-block SpMV form (OGB_OPT_SPMV_VARIANT)")
    ap.add_argument("--mixed-x64", type=int, default=-1, choices=(-1, 0, 1, 2, 3),
                    help="single mixed solves: 1 accumulate the solution in FP64 every iteration (2: with the "
                         "update's dot-product terms summed per thread in FP32), 0 / 3 as an FP32 increment folded "
                         "after every batch of iterations (3: FP64 sums) (OGB_OPT_MIXED_X64; -1 = library default)")
    ap.add_argument("--block-jacobi", type=int, default=-1, choices=(-1, 0, 1),
                    help="mixed solves: 1 block-Jacobi, 0 scalar Jacobi preconditioner "
                         "(OGB_OPT_MIXED_BLOCK_JACOBI; -1 = library default)")
    ap.add_argument("--tangent-tc", type=int, default=-1, choices=(-1, 0, 1, 2),
                    help="mixed Newton tangents: 0 FP64 CUDA cores, 1 tensor cores, 2 the faster "
                         "(OGB_OPT_TANGENT_TC; -1 = library default)")
    ap.add_argument("--half-form", type=int, default=-1, choices=tuple(range(-1, 7)),
                    help="half-stored SpMV loop form (OGB_OPT_HALF_FORM; -1 = library default, timed)")
    ap.add_argument("--update-blocks", type=int, default=-1, help="OGB_OPT_UPDATE_BLOCKS (-1 = library default)")
    ap.add_argument("--batch-x64", type=int, default=-1, choices=(-1, 0, 1),
                    help="batched mixed solves: 1 FP64 solution every iteration, 0 FP32 increment folded after "
                         "every batch of iterations (OGB_OPT_BATCH_X64; -1 = library default)")
    ap.add_argument("--fused-update", type=int, default=-1, choices=(-1, 0, 1),
                    help="block-Jacobi update and p update in one cooperative launch "
                         "(OGB_OPT_FUSED_UPDATE; -1 = library default)")
    ap.add_argument("--spmv-half", type=int, default=1, choices=(0, 1, 2),
                    help="half-stored FP32 operator in mixed solves (OGB_OPT_SPMV_HALF; 1 = default rule)")
    args = ap.parse_args()
    global ARGS
    ARGS = args
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "rve_batch":
        run_gpu_batch(args)
    elif args.workload == "mises_block":
        run_gpu_newton(args)
    elif args.workload == "idm1_batch":
        run_gpu_idm1_batch(args)
    elif args.workload == "spmv_forms":
        run_spmv_forms(args)
    elif args.workload == "solvers":
        run_solvers(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
