"""Benchmark: RCS solves/s of the dense CFIE multi-incidence job on one GB300.

Workload (the configuration the headline metric is quoted on): PEC sphere of
radius 1 m at 300 MHz, icosahedron subdivided 4 times (5120 triangles, 7680
RWG unknowns), CFIE alpha = 0.5, 360 incidences (theta = 90, phi = 0..359,
theta-polarised) solved as one block of right-hand sides, monostatic RCS of
each.  One step = fill Z + excitation for all 360 incidences + multi-RHS solve
to 1e-6 + 360 monostatic RCS values: 360 solves.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl emfa|reference]

value         solves/s with the mesh resident on the device (CUDA events on
              the library's stream, max over ranks x ranks' solves)
e2e           the same job through the host-buffer C ABI call emfa_dense_rcs
              (mesh in from host memory, RCS out to host memory, all inside)
accuracy      the job's RCS and currents against the reference's own run at
              this size (tests/golden/c2_cfie_sphere_7680.npz: the reference's
              RCS of the exact solution of its FP64 matrix)
vs_plain_fp64 the same 360-incidence job on the plain FP64 GPU path (FP64
              fill, FP64 GMRES(30) with two Gram-Schmidt passes): its solves/s
              and the mixed path's RCS / current difference from it
c1, mlfma,    the other configurations, a few seconds each: C1 plain FP64 EFIE
batch, serve  (1,920 RWG, bistatic), C3 MLFMA (122,880 RWG), C4 batched (64
              uneven EFIE problems), C5 served stream (Poisson arrivals)
Multi-GPU: replicas only (independent jobs per GPU, no collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RCS solves/s + p50/p99 latency vs plain FP64 GPU path at <=0.1 dB RCS error"
WORKLOADS = {
    # name: (subdivisions, radius m, freq Hz, alpha, n_inc)
    "c2_cfie_sphere_7680x360": (4, 1.0, 3e8, 0.5, 360),
}
GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden(name):
    """A reference fixture (the reference's own run at a benchmark size)."""
    import ast
    p = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(p):
        return None
    d = dict(np.load(p, allow_pickle=False))
    d["meta"] = ast.literal_eval(str(d["meta"]))
    return d


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rank_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def incidences(n_inc):
    return np.array([[90.0, float(p), 0.0] for p in np.arange(n_inc) * (360.0 / n_inc)], dtype=np.float64)


def run_emfa(args, workload):
    import torch
    from emfa_gb300 import api, mesh

    rank, local, world = rank_env()
    torch.cuda.set_device(local)
    sub, radius, freq, alpha, n_inc = WORKLOADS[workload]
    m = mesh.icosphere(sub, radius)
    ctx = api.Context(local)
    geo = api.Geometry(ctx, m)
    n = geo.n
    ang = incidences(n_inc)
    dirs = api.monostatic_dirs(ang)
    fp = api.fill_params("cfie", "f32", freq, alpha)
    sp = api.solver_params("gmres", restart=30, max_iter=900, tol=1e-6, matvec=args.matvec, orth=args.orth,
                           inner_reduction=args.inner_reduction, basis=args.basis)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())
    Z = torch.empty((n, n), dtype=torch.complex64, device="cuda")
    V = torch.empty((n_inc, n), dtype=torch.complex64, device="cuda")
    stages = {"fill_z": [], "fill_v": [], "solve": [], "rcs": []}
    infos = []
    last = {}

    def step(record):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(stream)
        api.fill_z(geo, fp, out=Z)
        ev[1].record(stream)
        api.fill_v(geo, fp, ang, out=V)
        ev[2].record(stream)
        X, info = api.solve(ctx, Z, V, sp)
        ev[3].record(stream)
        r = api.rcs(geo, fp, X, dirs, per_rhs=True)
        ev[4].record(stream)
        if record:
            torch.cuda.synchronize()
            for i, k in enumerate(stages):
                stages[k].append(ev[i].elapsed_time(ev[i + 1]))
            infos.append((info.iterations, info.cycles, info.converged, info.max_rel_residual))
        last["X"], last["rcs"] = X, r
        return ev, r

    for _ in range(args.warmup):
        step(False)
    torch.cuda.synchronize()
    l0 = ctx.launches()
    ctx.kernel_timing(True)  # event pairs around the fill, the TF32 product and the residual
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    step_ms = []
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(args.steps):
            ev, r_last = step(True)
            step_ms.append(ev[0].elapsed_time(ev[4]))
        end.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    total_ms = start.elapsed_time(end)
    launches = ctx.launches() - l0  # every library kernel launched in the timed region
    kernels = {k: ctx.kernel_time(k) for k in ctx.KERNEL_TIMERS}
    ctx.kernel_timing(False)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n_inc * args.steps / (total_ms * 1e-3)

    # end to end through the host-buffer C ABI call
    e2e_ms = []
    for i in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out, info, _ = api.dense_rcs(ctx, m, fp, ang, sp, dirs, per_rhs=True)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = world * n_inc / (statistics.median(e2e_ms) * 1e-3)
    h2d = m.verts.nbytes + m.tris.nbytes + ang.nbytes + dirs.nbytes
    d2h = out.nbytes

    acc, plain = {}, {}
    if args.check and rank == 0:
        acc = accuracy_vs_reference(ang, last["X"], last["rcs"])
        plain = plain_fp64_job(ctx, geo, freq, alpha, ang, dirs, last["X"], last["rcs"])
    torch.cuda.synchronize()
    geo.close()  # geometry before its context, not left to the interpreter's shutdown
    ctx.close()
    p50 = statistics.median(step_ms)
    p99 = float(np.percentile(step_ms, 99))
    return {
        "value": value, "total_ms": total_ms, "step_ms": step_ms, "p50": p50, "p99": p99,
        "stages": {k: statistics.median(v) for k, v in stages.items()}, "infos": infos,
        "launches": launches, "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                                      "d2h_bytes_per_step": int(d2h), "ms": statistics.median(e2e_ms)},
        "clocks": clocks.summary(), "n": n, "n_inc": n_inc, "acc": acc, "plain": plain, "world": world,
        "rank": rank, "kernels": kernels, "n_tri": int(m.tris.shape[0]),
        "autotune": api.autotune_query(local, n, n_inc),
    }


def accuracy_vs_reference(ang, X, r):
    """The job's monostatic RCS and currents at the reference fixture's
    incidences (phi = 0 and 137 of the 360) against the reference's RCS of
    the exact solution I* of its FP64 matrix, and against I*."""
    g = golden("c2_cfie_sphere_7680")
    if g is None:
        return {"reference_fixture": "absent"}
    fix = np.array([[float(t), float(p), float(q)] for t, p, q in g["meta"]["incidences"]])
    idx = [int(np.nonzero(np.all(np.isclose(ang, a), axis=1))[0][0]) for a in fix]
    Xh = X[idx].cpu().numpy()
    errs = [rel(Xh[i], g["Istar"][i]) for i in range(len(idx))]
    return {"against": "reference run at this size: its RCS of I* = Z64^-1 V64 (tests/golden/c2_cfie_sphere_7680)",
            "incidences_phi_deg": [float(a[1]) for a in fix],
            "rcs_max_abs_err_db": float(np.abs(r[idx] - g["rcs_f64"]).max()),
            "current_max_rel_err": float(max(errs)), "bar_db": 0.1, "bar_current": 1e-4}


def plain_fp64_job(ctx, geo, freq, alpha, ang, dirs, X_mixed, r_mixed):
    """The same 360-incidence job on the plain FP64 GPU path: FP64 fill and
    excitation, FP64 GMRES(30) to 1e-6 with two Gram-Schmidt passes, FP64
    products on the CUDA cores, RCS.  Timed once end to end on the device
    (wall clock, device synchronised on both sides)."""
    import torch
    from emfa_gb300 import api
    fp64 = api.fill_params("cfie", "f64", freq, alpha)
    sp64 = api.solver_params("gmres", restart=30, max_iter=900, tol=1e-6)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Z = api.fill_z(geo, fp64)
    t1 = time.perf_counter()
    V = api.fill_v(geo, fp64, ang)
    X, info = api.solve(ctx, Z, V, sp64)
    r = api.rcs(geo, fp64, X, dirs, per_rhs=True)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    cur = (torch.linalg.vector_norm(X_mixed - X, dim=1) / torch.linalg.vector_norm(X, dim=1)).max().item()
    del Z, V, X
    torch.cuda.empty_cache()
    return {"solves_per_s": round(len(ang) / t, 3), "seconds": round(t, 3), "fill_s": round(t1 - t0, 3),
            "iterations": info.iterations, "converged": info.converged,
            "rcs_max_abs_err_db_mixed_vs_plain": float(np.abs(r_mixed - r).max()),
            "current_max_rel_err_mixed_vs_plain": float(cur),
            "work": "same job: %d incidences, tol 1e-6, one fill" % len(ang)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


_ARGS = {}


def args_matvec():
    return _ARGS.get("matvec", "auto")


def roofline(res):
    """Roofline of the dominant kernel of the step (the tensor-core inner
    product of the Krylov iterations: split-FP16 kind::f16, the bf16 rate),
    from the event-timed launches of the timed region."""
    from emfa_gb300 import roofline as RM
    peaks, src = measured_peaks()
    n_l, ms, flops = res["kernels"]["gemm"]
    if not n_l:
        return None
    achieved = flops / (ms * 1e-3) / 1e12
    peak = peaks["bf16_tflops_sustained"]
    f16 = args_matvec() in ("auto", "f16x")
    tall = 5 * ((res["n"] + 255) // 256) >= 137  # 256-row tiles fill the 152 SMs
    traffic = RM.INNER_TRAFFIC_7680x360 if f16 and (res["n"], res["n_inc"]) == (7680, 360) else None
    return {"kernel": ("th::k_hgemm<144,2>" if tall else "th::k_hgemm<144,1>") if f16 else "tc::k_gemm_tf32",
            "bound": "tensor", "achieved": round(achieved, 2), "peak": peak,
            "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "frac_of_burst": round(achieved / peaks["bf16_tflops"], 4),
            "traffic": traffic,
            "traffic_source": "ncu capture of this kernel at this size (DRAM read + write per launch)" if traffic
            else None,
            "algorithmic_bytes_per_launch": RM.split_fp16_inner_bytes(res["n"], res["n_inc"]),
            "peak_source": "%s bf16 dense, sustained (kernel timed inside a long step); frac_of_burst against "
                           "the burst figure" % src,
            "operand": "fp16 (hi plane of Z) x fp16, fp32 accumulate" if f16
            else "tf32 (nominal tf32 dense rate = 1/2 bf16)", "launches": n_l,
            "avg_launch_ms": round(ms / n_l, 5), "flops_per_launch": flops / n_l}


def fill_roofline(res):
    """The FP32 fill's model FLOP rate (regular pairs: 9 point pairs of 75
    FLOP per triangle pair) against the nominal FP32 rate of the clocks seen."""
    from emfa_gb300 import roofline as RM
    n_l, ms, entries = res["kernels"]["fill_z"]
    if not n_l:
        return None
    flops = RM.fill_flops(res["n_tri"], True) * n_l
    mhz = res["clocks"].get("sm_mhz") or 2070.0
    peak = RM.fp32_nominal_tflops(152, mhz)
    achieved = flops / (ms * 1e-3) / 1e12
    return {"kernel": "k_fill_tile_cfie_sym (CFIE)", "bound": "fp32/mufu issue", "avg_launch_ms": round(ms / n_l, 4),
            "achieved": round(achieved, 2), "unit": "TFLOP/s (model)", "peak": round(peak, 1),
            "frac": round(achieved / peak, 4),
            "peak_source": "nominal FP32 FMA rate at the median SM clock (no measured FP32 figure)"}


def kernel_table(res):
    out = {}
    for k, (n_l, ms, work) in res["kernels"].items():
        if n_l:
            unit = "Gentries/s" if k == "fill_z" else "TFLOP/s"
            rate = work / (ms * 1e-3) / (1e9 if k == "fill_z" else 1e12)
            out[k] = {"launches": n_l, "avg_ms": round(ms / n_l, 4), "rate": round(rate, 2), "unit": unit}
    return out


def run_c1(args):
    """C1: plain EFIE on the r = 0.5 m sphere (icosphere 3, 1,920 RWG) at
    300 MHz, incidence along -z, theta-polarised, bistatic RCS over the
    reference's 541 directions.  The plain FP64 GPU path (FP64 fill, FP64
    GMRES(30) to 1e-6) and the mixed path (FP32 fill with FP64 self terms,
    FP32 LU with FP64 refinement to 1e-6), each timed per job (fill +
    excitation + solve + RCS, device synchronised on both sides) and checked
    against the reference's run at this size and the Mie series."""
    import torch
    from emfa_gb300 import api, mesh
    from oracle import mie
    m = mesh.icosphere(3, 0.5)
    ctx = api.Context(0)
    geo = api.Geometry(ctx, m)
    ang = np.array([[0.0, 0.0, 0.0]])
    g = golden("c1_efie_sphere_1920")
    dirs = api.bistatic_dirs(0.0, 180.0, 1.0, 0.0, ring=True)
    out = {"workload": "c1_efie_sphere_1920", "n_rwg": geo.n, "directions": int(dirs.shape[0])}
    for name, prec, sp, disc in (
            ("plain_fp64", "f64", api.solver_params("gmres", restart=30, tol=1e-6, max_iter=20000), "reference"),
            ("mixed", "f32", api.solver_params("lu", tol=1e-6, max_iter=50), "reference"),
            # the discretisation the configuration states: 7-point rule,
            # extraction on self and edge-adjacent pairs (no reference run)
            ("plain_fp64_config_discretisation", "f64",
             api.solver_params("gmres", restart=30, tol=1e-6, max_iter=20000), "config"),
            ("mixed_config_discretisation", "f32", api.solver_params("lu", tol=1e-6, max_iter=50), "config")):
        fp = api.fill_params("efie", prec, 3e8, 1.0, discretisation=disc)
        times = []
        for i in range(max(1, args.warmup) + max(1, min(args.steps, 5))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Z = api.fill_z(geo, fp)
            V = api.fill_v(geo, fp, ang)
            X, info = api.solve(ctx, Z, V, sp)
            r = api.rcs(geo, fp, X, dirs)[0]
            torch.cuda.synchronize()
            if i >= max(1, args.warmup):
                times.append(time.perf_counter() - t0)
            del Z
        t = statistics.median(times)
        e = {"solves_per_s": round(1.0 / t, 2), "ms_per_job": round(1e3 * t, 3), "iterations": info.iterations,
             "converged": info.converged, "max_rel_residual": info.max_rel_residual}
        if g is not None:
            if disc == "reference":
                e["rcs_max_abs_err_db_vs_reference"] = float(np.abs(r - g["rcs_f64"][0]).max())
                e["current_rel_err_vs_istar"] = rel(X.cpu().numpy()[0], g["Istar"][0])
            inc = g["inc_f64"][0]
            exact = mie.pec_sphere_rcs_db(0.5, 3e8, inc[:3], inc[3:6], g["rcs_dirs_f64"].astype(np.float64))
            e["rcs_max_abs_err_db_vs_mie"] = float(np.abs(r - exact).max())
            e["reference_rcs_max_abs_err_db_vs_mie"] = float(np.abs(g["rcs_f64"][0] - exact).max())
        out[name] = e
    out["speedup_mixed_vs_plain_fp64"] = round(out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"], 2)
    geo.close()
    ctx.close()
    return out


def run_lu(args):
    """Dense LU solve (EMFA_LU) alone: a seeded random complex64 system of
    order --lu-n (diagonal weight 3 sqrt(n), so well conditioned) with 8
    right-hand sides, factor + solve + FP64 refinement to 1e-6, wall time
    with the device synchronised on both sides.  FLOPs counted as (8/3) n^3
    (complex LU) + 16 n^2 R (two triangular solves)."""
    import torch
    from emfa_gb300 import api
    n, r = args.lu_n, 8
    ctx = api.Context(0)
    g = torch.Generator(device="cuda").manual_seed(3)
    Z = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    Z += 3.0 * n ** 0.5 * torch.eye(n, dtype=torch.complex64, device="cuda")
    B = torch.randn((r, n), dtype=torch.complex64, device="cuda", generator=g)
    sp = api.solver_params("lu", tol=1e-6)
    times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, info = api.solve(ctx, Z, B, sp)
        torch.cuda.synchronize()
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    flops = 8.0 / 3.0 * n ** 3 + 16.0 * n * n * r
    print(json.dumps({"mode": "lu", "n": n, "n_rhs": r, "seconds": round(t, 5),
                      "tflops": round(flops / t / 1e12, 2), "refinement_passes": info.iterations,
                      "converged": info.converged, "max_rel_residual": info.max_rel_residual}))


def run_gemm_only(args):
    """Micro-benchmark of the multi-RHS products alone: the inner product of
    the solver and (split FP16) the refinement residual, Z (N x N complex64,
    random) times R vectors, kernel time from the context's event timers.
    Used to profile the tensor-core kernels in isolation."""
    import torch
    from emfa_gb300 import api
    n, r = args.gemm_n, args.gemm_r
    mv = args.matvec if args.matvec != "auto" else "f16x"
    ctx = api.Context(0)
    g = torch.Generator(device="cuda").manual_seed(1)
    Z = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    X = torch.randn((r, n), dtype=torch.complex64, device="cuda", generator=g)
    Xd = X.to(torch.complex128)
    resid = mv in ("f16x", "f32")
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            ctx.kernel_timing(True)
        api.matvec(ctx, Z, X, mv)
        if resid:
            api.residual(ctx, Z, Xd, X, mv)
    torch.cuda.synchronize()
    flops = 8.0 * n * n * r
    out = {"mode": "gemm", "matvec": mv, "n": n, "r": r}
    for k in ("gemm", "residual"):
        n_l, ms, _ = ctx.kernel_time(k)
        if n_l:
            out[k + "_ms"] = round(ms / n_l, 5)
            out[k + "_tflops"] = round(flops / (ms / n_l * 1e-3) / 1e12, 2)
    ctx.kernel_timing(False)
    print(json.dumps(out))


def run_mlfma(args):
    """C3: MLFMA CFIE on the 5-lambda sphere (81920 triangles, 122880 RWG),
    finest box 0.25 lambda, one plane wave along -z: operator set-up, the
    mat-vec alone (time and HBM bytes), GMRES(30) to 1e-3 and the bistatic
    RCS against the reference's MLFMA run at this size."""
    import torch
    from emfa_gb300 import api, mesh
    from emfa_gb300 import roofline as RM
    lam = 299792458.0 / 3e8
    m = mesh.icosphere(args.mlfma_subdiv, 5.0 * lam)
    ctx = api.Context(0)
    t0 = time.perf_counter()
    geo = api.Geometry(ctx, m)
    ml = api.Mlfma(geo, api.mlfma_params(3e8, 0.5, 0.25))
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    V = ml.fill_v(np.array([[0.0, 0.0, 0.0]]))
    x = V.clone()
    for _ in range(max(3, args.warmup)):
        ml.apply(x)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(1, args.steps)
    e0.record(stream)
    for _ in range(reps):
        ml.apply(x)
    e1.record(stream)
    torch.cuda.synchronize()
    mv_ms = e0.elapsed_time(e1) / reps
    sp = api.solver_params("gmres", restart=30, max_iter=300, tol=1e-3)
    t0 = time.perf_counter()
    X, info = ml.solve(V, sp)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    out = {"workload": "c3_mlfma_sphere_122880", "n_rwg": geo.n, "levels": ml.levels,
           "level_boxes": ml.level_boxes.tolist(), "poles": ml.poles.tolist(), "near_nnz": ml.nnz,
           "setup_s": round(t_setup, 3), "matvec_ms": round(mv_ms, 4), "solve_s": round(t_solve, 4),
           "iterations": info.iterations, "converged": info.converged, "rel_residual": info.max_rel_residual}
    g = golden("c3_mlfma_sphere_122880") if geo.n == 122880 else None
    if g is not None:
        r = api.rcs(geo, api.fill_params("cfie", "f32", 3e8, 0.5), ml.unpermute(X), g["rcs_dirs"].astype(np.float64))[0]
        keep = g["rcs"] > g["rcs"].max() - 20.0
        out["accuracy"] = {"against": "reference MLFMA run at this size (BiCGStab to 1e-3)",
                           "rcs_max_abs_err_db": float(np.abs(r - g["rcs"]).max()),
                           "rcs_max_abs_err_db_within_20db_of_peak": float(np.abs(r - g["rcs"])[keep].max()),
                           "reference_iterations": int(g["iters"][0])}
    if args.mlfma_sai:
        # the same solve with the SAI preconditioner (own batched QR per finest box)
        t0 = time.perf_counter()
        mlp = api.Mlfma(geo, api.mlfma_params(3e8, 0.5, 0.25, precond=True))
        torch.cuda.synchronize()
        t_setup_p = time.perf_counter() - t0
        t0 = time.perf_counter()
        Xp, infop = mlp.solve(V, sp)
        torch.cuda.synchronize()
        out["sai"] = {"setup_s": round(t_setup_p, 3), "solve_s": round(time.perf_counter() - t0, 4),
                      "iterations": infop.iterations, "converged": infop.converged,
                      "nnz": int(mlp.precond_csr()[0][-1]),
                      "current_vs_unpreconditioned": float(torch.linalg.norm(Xp - X) / torch.linalg.norm(X))}
        mlp.close()
    peaks, src = measured_peaks()
    b3 = RM.mlfma_matvec_bytes(geo.n, ml.nnz, ml.level_boxes.tolist(), ml.poles.tolist(), comps=3,
                               radrec_comps=2)
    b2 = RM.mlfma_matvec_bytes(geo.n, ml.nnz, ml.level_boxes.tolist(), ml.poles.tolist(), comps=2,
                               near_index_bytes=4)
    gbs = b3 / (mv_ms * 1e-3) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": round(gbs, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                       "frac": round(gbs / peaks["hbm_gbs"], 4), "peak_source": src,
                       "algorithmic_bytes": b3,
                       "model": "as stored: radiation/receive patterns theta, phi; level patterns x, y, z",
                       "model_bytes_2comp_theta_phi": b2,
                       "model_frac_2comp_theta_phi": round(b2 / (mv_ms * 1e-3) / 1e9 / peaks["hbm_gbs"], 4)}
    ml.close()
    geo.close()
    ctx.close()
    return out


def _pct(v, q):
    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def run_batch(args):
    """C4 batched engine: 64 uneven EFIE problems (ellipsoids and cubes at
    lambda/10, 500..8000 unknowns, 200..600 MHz), 8 incidences each with
    their monostatic RCS, all through emfa_serve at once.  The engine factors
    each EFIE problem (EMFA_LU); "iterations" are its refinement passes.
    The plain FP64 GPU path (FP64 fill and GMRES(250)) is timed on a
    stratified sample of the same problems (the smallest, the largest and
    evenly between, by unknowns), with fill and solve timed apart, and its
    solves/s over the whole set is composed from the sample's per-problem
    times scaled by N^2 (fill) and N^2 x iterations (solve)."""
    import torch
    from emfa_gb300 import api, workloads as W
    probs = W.batch_set(seed=0, count=64, n_inc=8)

    def requests():
        return [api.RcsRequest(m, f, ang, d, kind="efie", per_rhs=True) for (m, f, ang, d) in probs]

    for _ in range(max(1, min(args.warmup, 2))):
        api.serve(requests(), lanes=args.lanes)
    walls, res, reqs = [], None, None
    for _ in range(max(1, min(args.steps, 3))):
        reqs = requests()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = api.serve(reqs, lanes=args.lanes)
        walls.append(time.perf_counter() - t0)
    solves = sum(r.angles.shape[0] for r in reqs)
    wall = statistics.median(walls)
    svc = [r.t_done - r.t_start for r in res]
    ok = sum(1 for r in res if r.status == 0)
    order = np.argsort([r.n_rwg for r in res])
    sample = [int(order[i]) for i in np.linspace(0, len(order) - 1, args.batch_plain_sample).astype(int)]
    ctx = api.Context(0)
    err_db, rows = 0.0, []
    for i in sample:
        m, f, ang, d = probs[i]
        geo = api.Geometry(ctx, m)
        fp = api.fill_params("efie", "f64", f, 1.0)
        fp.edm_mode = 2
        sp = api.solver_params("gmres", restart=250, tol=1e-5, max_iter=5000)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Z = api.fill_z(geo, fp)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        V = api.fill_v(geo, fp, ang)
        X, info = api.solve(ctx, Z, V, sp)
        r = api.rcs(geo, fp, X, d, per_rhs=True)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        rows.append((geo.n, t1 - t0, t2 - t1, info.iterations))
        err_db = max(err_db, float(np.abs(reqs[i].rcs - r).max()))
        del Z, V, X
        geo.close()
    ctx.close()
    # compose the plain path over all 64 problems from the sample: fill ~ N^2,
    # solve ~ N^2 x iterations (iterations interpolated in log N)
    ns = np.array([x[0] for x in rows], dtype=np.float64)
    fill_c = np.array([x[1] / x[0] ** 2 for x in rows])
    its = np.array([max(1, x[3]) for x in rows], dtype=np.float64)
    solve_c = np.array([x[2] / (x[0] ** 2 * max(1, x[3])) for x in rows])
    t_plain = 0.0
    for r in res:
        n = float(r.n_rwg)
        it = float(np.interp(np.log(n), np.log(ns), its))
        t_plain += n * n * (float(np.interp(np.log(n), np.log(ns), fill_c)) +
                            it * float(np.interp(np.log(n), np.log(ns), solve_c)))
    plain_sample_solves_per_s = sum(probs[i][2].shape[0] for i in sample) / sum(x[1] + x[2] for x in rows)
    return {
        "workload": "c4_batch_64_efie", "value": round(solves / wall, 3), "unit": "solves/s", "problems": len(reqs),
        "ok": ok, "solves": solves, "wall_s": round(wall, 4), "lanes": args.lanes or 6,
        "unknowns": {"min": min(r.n_rwg for r in res), "max": max(r.n_rwg for r in res),
                     "mean": round(statistics.mean(r.n_rwg for r in res), 1)},
        "iterations": {"p50": _pct([r.iterations for r in res], 50), "max": max(r.iterations for r in res)},
        "service_ms": {"p50": round(1e3 * _pct(svc, 50), 2), "p99": round(1e3 * _pct(svc, 99), 2)},
        "plain_fp64": {"sample_problems": len(sample),
                       "sample": [{"n": int(a), "fill_s": round(b, 4), "solve_s": round(c, 4), "iterations": int(it)}
                                  for a, b, c, it in rows],
                       "sample_solves_per_s": round(plain_sample_solves_per_s, 3),
                       "composed_all_64_seconds": round(t_plain, 3),
                       "composed_all_64_solves_per_s": round(solves / t_plain, 3)},
        "speedup_vs_plain_fp64": round(solves / wall / (solves / t_plain), 2),
        "rcs_max_abs_err_db_vs_fp64": err_db,
        # every problem is factored (EMFA_LU): (8/3) N^3 complex-LU FLOPs in all
        "lu": {"tflop": round(sum(8.0 / 3.0 * r.n_rwg ** 3 for r in res) / 1e12, 2),
               "aggregate_tflops": round(sum(8.0 / 3.0 * r.n_rwg ** 3 for r in res) / wall / 1e12, 2)},
        "data": "synthetic, seeded (seed 0)"}


def _serve_stream(args, rate, count):
    import torch
    from emfa_gb300 import api, workloads as W
    stream = W.served_stream(seed=0, count=count, rate=rate, n_inc=4)
    reqs = [api.RcsRequest(m, f, ang, d, kind="cfie", alpha=0.5, per_rhs=True, arrival_s=t)
            for (t, m, f, ang, d) in stream]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = api.serve(reqs, lanes=args.lanes, realtime=True)
    wall = time.perf_counter() - t0
    lat = [r.t_done - r.t_arrive for r in res]
    solves = sum(r.angles.shape[0] for r in reqs)
    mk = max(r.t_done for r in res)
    span = stream[-1][0]
    dense = [r for r in res if r.method == 1]
    ml = [r for r in res if r.method == 2]
    return {
        "offered_req_per_s": rate, "requests": len(reqs), "ok": sum(1 for r in res if r.status == 0),
        "solves": solves, "value": round(solves / mk, 3), "unit": "solves/s", "wall_s": round(wall, 3),
        "arrival_span_s": round(span, 3), "offered_rate_measured": round(len(reqs) / span, 1),
        "served_req_per_s": round(len(reqs) / mk, 1),
        "latency_ms": {"p50": round(1e3 * _pct(lat, 50), 1), "p99": round(1e3 * _pct(lat, 99), 1)},
        "dense": {"requests": len(dense),
                  "latency_p50_ms": round(1e3 * _pct([r.t_done - r.t_arrive for r in dense], 50), 1) if dense else None},
        "mlfma": {"requests": len(ml),
                  "latency_p50_ms": round(1e3 * _pct([r.t_done - r.t_arrive for r in ml], 50), 1) if ml else None,
                  "max_unknowns": max((r.n_rwg for r in ml), default=0)}}


def run_serve(args):
    """C5 served stream: Poisson arrivals of monostatic RCS requests (4
    incidences each), 1k..120k unknowns log-uniform on spheres, ellipsoids
    and cubes at lambda/10, CFIE alpha 0.5; dense below 10k unknowns, MLFMA
    above; 150 GB admission budget.  Latency = completion - arrival on the
    host clock.  Two streams: the configured mean of 200 requests/s, which
    arrives faster than one GPU serves it (its latency is mostly queueing),
    and a steady stream at --serve-steady-rate, below the served rate, whose
    latency is the engine's own."""
    from emfa_gb300 import api, workloads as W
    warm = W.served_stream(seed=1, count=6, rate=200.0, n_inc=4)
    api.serve([api.RcsRequest(m, f, ang, d, kind="cfie", per_rhs=True) for (t, m, f, ang, d) in warm],
              lanes=args.lanes)
    return {"workload": "c5_served_stream", "lanes": args.lanes or 6, "hbm_budget_gb": 150,
            "configured": _serve_stream(args, 200.0, args.requests),
            "steady": _serve_stream(args, args.serve_steady_rate, args.requests),
            "data": "synthetic, seeded (seed 0)"}


def _secondary(name, fn, args):
    """One of the other configurations for the default line; a failure is
    recorded there, it does not lose the headline."""
    t0 = time.perf_counter()
    try:
        out = fn(args)
    except Exception as e:  # noqa: BLE001 -- reported in the line
        out = {"error": "%s: %s" % (type(e).__name__, e)}
    out["bench_seconds"] = round(time.perf_counter() - t0, 2)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="emfa", choices=["emfa", "reference"])
    ap.add_argument("--workload", default="c2_cfie_sphere_7680x360", choices=list(WORKLOADS))
    ap.add_argument("--matvec", default="auto", choices=["auto", "f32", "tf32", "f16x"])
    ap.add_argument("--check", type=int, default=1)
    ap.add_argument("--orth", default="auto", choices=["auto", "cgs1", "cgs2", "cgs1_split", "cgs1_fused"])
    ap.add_argument("--basis", default="auto", choices=["auto", "f32", "f16"],
                    help="GMRES basis storage of the FP32 inner solve")
    ap.add_argument("--inner-reduction", type=float, default=0.0,
                    help="GMRES refinement: per-cycle inner reduction (0 = the solver's default, <0 = none)")
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--secondary", type=int, default=1,
                    help="add the C1, C3, C4 and C5 blocks to the default line")
    ap.add_argument("--mode", default="job", choices=["job", "c1", "gemm", "mlfma", "batch", "serve", "lu"])
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--serve-steady-rate", type=float, default=30.0)
    ap.add_argument("--batch-plain-sample", type=int, default=4)
    ap.add_argument("--mlfma-subdiv", type=int, default=6)
    ap.add_argument("--mlfma-sai", type=int, default=0)
    ap.add_argument("--gemm-n", type=int, default=7680)
    ap.add_argument("--gemm-r", type=int, default=360)
    ap.add_argument("--lu-n", type=int, default=7938)
    args = ap.parse_args()
    if args.impl == "emfa":
        from emfa_gb300 import build
        build.build()
    single = {"lu": run_lu, "gemm": run_gemm_only}
    if args.mode in single:
        single[args.mode](args)
        return
    blocks = {"c1": run_c1, "mlfma": run_mlfma, "batch": run_batch, "serve": run_serve}
    if args.mode in blocks:
        print(json.dumps(dict(mode=args.mode, **blocks[args.mode](args))))
        return
    rank, local, world = rank_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        if rank == 0:
            from oracle import cpu_baseline
            print(json.dumps(cpu_baseline.reference_arm(args, WORKLOADS[args.workload], args.workload)))
        return
    _ARGS["matvec"] = args.matvec
    res = run_emfa(args, args.workload)
    if rank != 0:
        return
    plain = res["plain"]
    line = {
        "metric": METRIC, "value": round(res["value"], 3), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(res["total_ms"] / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64/f32 (+f64 Krylov)",
        "data": "synthetic (seeded icosphere mesh, analytic plane waves)",
        "config": {"workload": args.workload, "n_rwg": res["n"], "n_rhs": res["n_inc"], "formulation": "CFIE a=0.5",
                   "solver": "GMRES(30)+refinement tol 1e-6", "parallelism": "replicas",
                   "l2": "inputs > L2 (Z = %.0f MB)" % (res["n"] ** 2 * 8 / 1e6)},
        "latency_ms": {"p50": round(res["p50"], 3), "p99": round(res["p99"], 3)},
        "stages_ms": {k: round(v, 3) for k, v in res["stages"].items()},
        "solver": {"iterations": res["infos"][-1][0], "cycles": res["infos"][-1][1],
                   "converged": res["infos"][-1][2], "max_rel_residual": res["infos"][-1][3],
                   "orth": args.orth, "basis": args.basis},
        "e2e": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in res["e2e"].items()},
        "gpu_launches": res["launches"],
        "gpu_launches_per_step": res["launches"] // max(1, args.steps),
        "clocks": res["clocks"],
        "accuracy": res["acc"],
        "vs_plain_fp64": dict(plain, speedup=round(res["value"] / plain["solves_per_s"], 2)) if plain else None,
        "roofline": roofline(res),
        "fill_roofline": fill_roofline(res),
        "kernels": kernel_table(res),
        # the inner product's tile shape (columns x rows) the autotuner chose in
        # the warm-up, with each candidate's best time (ms)
        "autotune": {"shape": res["autotune"][0],
                     "candidates_ms": {k: round(v, 4) for k, v in res["autotune"][1].items()}},
    }
    if world == 1 and args.secondary:
        for name, fn in (("c1", run_c1), ("mlfma", run_mlfma), ("batch", run_batch), ("serve", run_serve)):
            line[name] = _secondary(name, fn, args)
    if world == 1 and args.cpu_baseline:
        # the reference's own CPU path on this host's cores, bounded sample (oracle/cpu_baseline.py)
        from oracle import cpu_baseline
        vals, det = cpu_baseline.measure(WORKLOADS[args.workload], args.workload, rows=1024, steps=1)
        line["cpu_baseline"] = {"value": round(vals[0], 6), "unit": "solves/s", "cores": det["cores"],
                                "kind": det["kind"], "sample": det["sample"]}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
