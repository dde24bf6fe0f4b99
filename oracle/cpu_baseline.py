"""CPU baseline -- TEST INFRASTRUCTURE, run only by bench.py's reference arm
and its cpu_baseline field.

Times the reference's own CFIE path (xiangwei0909/EMFA compiled from its
sources, oracle/_ref) on this machine's host cores, on a bounded sample of
the dense CFIE job, and scales the stage times to the full job:

  one reference process = fill Z once + per incidence (fillV + BiCGStab to
  1e-2 + one monostatic RCS direction); the reference's CFIE is single-
  threaded and solves one incidence per run, so all host cores are used as a
  farm of processes that each fill Z and solve their share of incidences.

Measured per step (all processes at once, so memory bandwidth is shared as in
a real farm): the leading rows x rows block of the fill, fillV, one Armadillo
complex GEMV of the full order (BiCGStab runs two per iteration,
EMIterative/iml.cpp:22,29) and one getBiRCS direction.

When the reference cannot be built here, the same stages are timed with the
oracle restatement (oracle/emfa_oracle.c) and the result says kind "port".
"""
from __future__ import annotations

import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# BiCGStab iterations of the reference on this job (CFIE alpha 0.5, 7680-RWG
# sphere, theta = 90 incidence, tolerance 1e-2): measured with the reference
# binary itself (oracle/_ref, `time` mode with solve=1) on the same mesh.
REF_BICGSTAB_ITERS = {"c2_cfie_sphere_7680x360": 10, "c1_cfie_sphere_1920x360": 8}


def ensure_reference() -> str | None:
    exe = O.ref_binary(32)
    if exe:
        return exe
    try:
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--staged"], check=True, timeout=900,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    except Exception:
        return None
    return O.ref_binary(32)


def _job_files(wl):
    from emfa_gb300 import mesh as M
    sub, radius, freq, alpha, n_inc = wl
    d = tempfile.mkdtemp(prefix="emfa_cpu_")
    m = M.icosphere(sub, radius)
    nas = os.path.join(d, "job.nas")
    M.write_nas(m, nas)
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver="CFIE", mesh_path=nas, frequency=repr(freq), alpha=repr(alpha), theta="90",
                   phi="0", pole="0")
    return d, cfg, m


def _stages_parallel(exe, cfg, rows, procs, reps=2, timeout=900):
    cmds = []
    for p in range(procs):
        cwd = tempfile.mkdtemp(prefix="emfa_cpu_p%d_" % p)
        cmds.append(subprocess.Popen([exe, "stages", cfg, str(rows), str(reps)], cwd=cwd, stdin=subprocess.DEVNULL,
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True))
    out = []
    for c in cmds:
        so, _ = c.communicate(timeout=timeout)
        # the reference's progress bar leaves no newline before the record
        line = [l[l.index('{"n"'):] for l in so.splitlines() if '{"n"' in l]
        if c.returncode != 0 or not line:
            raise RuntimeError("reference stages run failed")
        out.append(json.loads(line[-1]))
    return out


def _stages_port(cfg_mesh, wl, rows):
    """Same stages with the oracle restatement (single process)."""
    import numpy as np
    from emfa_gb300 import api
    sub, radius, freq, alpha, n_inc = wl
    m = cfg_mesh
    t0 = time.perf_counter()
    rwg = O.build_rwg(m.tris)
    t_init = time.perf_counter() - t0
    g = O.Geometry(m.verts.astype(np.float32), m.tris, rwg, 32)
    k = O.wavenumber(freq, 32)
    sub_idx = np.arange(min(rows, g.n))
    gs = O.Geometry(g.verts, g.tris, g.rwg[sub_idx], 32)
    t0 = time.perf_counter()
    O.fill_z_cfie(gs, k, alpha)
    t_block = time.perf_counter() - t0
    inc = O.incidence(90, 0, 0, 32)
    t0 = time.perf_counter()
    O.fill_v(g, k, inc, cfie=True, alpha=alpha)
    t_fillv = time.perf_counter() - t0
    Z = (np.random.default_rng(3).standard_normal((g.n, g.n)) + 0j).astype(np.complex64)
    x = np.ones(g.n, np.complex64)
    t0 = time.perf_counter()
    for _ in range(2):
        Z @ x
    t_gemv = (time.perf_counter() - t0) / 2
    t0 = time.perf_counter()
    O.rcs(g, k, x[None].astype(np.complex64), np.array([[1.0, 0.0, 0.0]], np.float32))
    t_rcs = time.perf_counter() - t0
    return [{"n": g.n, "rows": len(sub_idx), "init_s": t_init, "block_fill_s": t_block, "fillv_s": t_fillv,
             "gemv_s": t_gemv, "rcs_dir_s": t_rcs}]


def job_time(stage_rows, n_inc, iters, procs):
    """Seconds for the whole job on `procs` reference processes."""
    s = stage_rows
    n, rows = s[0]["n"], s[0]["rows"]
    block = statistics.mean(r["block_fill_s"] for r in s)
    fill = block * (n / rows) ** 2
    per_inc = statistics.mean(r["fillv_s"] + 2 * iters * r["gemv_s"] + r["rcs_dir_s"] for r in s)
    init = statistics.mean(r["init_s"] for r in s)
    return init + fill + math.ceil(n_inc / procs) * per_inc, {"fill_s": fill, "per_incidence_s": per_inc,
                                                             "init_s": init}


def measure(wl, name, rows=1024, procs=None, steps=1, warmup=0):
    """Returns (values, detail): RCS solves/s of the reference's CPU path per
    timed step, and what was measured."""
    procs = procs or (os.cpu_count() or 1)
    d, cfg, m = _job_files(wl)
    n_inc = wl[4]
    iters = REF_BICGSTAB_ITERS.get(name, 10)
    exe = ensure_reference()
    kind = "reference" if exe else "port"
    vals, detail = [], {}
    for i in range(warmup + steps):
        r = rows if i >= warmup else max(64, rows // 4)
        st = _stages_parallel(exe, cfg, r, procs) if exe else _stages_port(m, wl, r)
        p = procs if exe else 1
        t, detail = job_time(st, n_inc, iters, p)
        if i >= warmup:
            vals.append(n_inc / t)
    detail.update({"kind": kind, "cores": procs if exe else 1, "rows": rows, "iters": iters,
                   "sample": ("leading %dx%d block of the CFIE fill, fillV, %d-order complex GEMV and one RCS "
                              "direction per process on %d concurrent reference processes, scaled to the full "
                              "job: fill once per process + ceil(%d/%d) incidences x (fillV + %d BiCGStab "
                              "iterations x 2 GEMV + 1 RCS)" % (rows, rows, m.n_rwg_closed(), procs if exe else 1,
                                                                n_inc, procs if exe else 1, iters))})
    return vals, detail


def reference_arm(args, wl, name):
    """bench.py --impl reference: the JSON line of the reference's CPU path."""
    vals, det = measure(wl, name, rows=1024, steps=args.steps, warmup=args.warmup)
    v = statistics.median(vals)
    return {"metric": "RCS solves/s + p50/p99 latency vs plain FP64 GPU path at <=0.1 dB RCS error",
            "impl": "reference", "value": round(v, 6), "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64/f32 (reference value_t = float)", "data": "synthetic (seeded icosphere mesh)",
            "config": {"workload": name, "n_rhs": wl[4], "formulation": "CFIE a=%.1f" % wl[3]},
            "ms_per_step": round(1e3 * wl[4] / v, 3),
            "cpu_baseline": {"value": round(v, 6), "unit": "solves/s", "cores": det["cores"], "kind": det["kind"],
                             "sample": det["sample"]},
            "e2e": {"value": round(v, 6), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "stage_estimates_s": {k: round(det[k], 4) for k in ("init_s", "fill_s", "per_incidence_s")}}
