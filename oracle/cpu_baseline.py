"""CPU baseline -- TEST INFRASTRUCTURE, run only by bench.py's reference arm
and its cpu_baseline field.

The reference's own CFIE path (xiangwei0909/EMFA compiled from its sources,
oracle/_ref) on this machine's host cores, for the dense CFIE job of the
benchmark (7,680 RWG, 360 incidences).  The reference's CFIE is
single-threaded and solves one incidence per run (CFIE::solve, CFIE.cpp:53-88:
fillZ, fillV, BiCGStab to 1e-2), so all host cores run as a farm of
processes.

reference_arm (bench.py --impl reference) MEASURES: one full stock job per
host core at once, each at its own incidence of the 360 (init, fillZ,
fillV, BiCGStab, the monostatic RCS direction), timed stage by stage inside
the reference process.  From those stage times the 360-incidence job is
composed as one process per core that fills Z once and then solves its share
of incidences (ceil(360 / cores) x (fillV + BiCGStab + RCS)); that is
generous to the reference, whose stock code fills Z again for every
incidence, so the stock per-run figure (cores solves per farm wall time) is
reported beside it.  The bounded-sample model below is reported with its
error against the measurement.

measure (the cpu_baseline field of the GPU arm: 10-30 s of CPU work) times
a bounded sample -- the leading rows x rows block of the fill, fillV, one
Armadillo complex GEMV of the full order (BiCGStab runs two per iteration,
EMIterative/iml.cpp:22,29) and one getBiRCS direction per process -- and
scales it to the job with the reference's own BiCGStab iteration counts at
this size (recorded from the reference binary in the C2 fixture).

When the reference cannot be built here, the sample is timed with the
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

FIXTURE = {"c2_cfie_sphere_7680x360": "c2_cfie_sphere_7680"}


def reference_iterations(name):
    """The reference binary's own BiCGStab iteration counts on this job (its
    CFIE::solve at the C2 fixture's incidences, recorded when the fixture was
    made from the compiled reference); None when absent."""
    import numpy as np
    fx = FIXTURE.get(name)
    p = os.path.join(ROOT, "tests", "golden", (fx or "") + ".npz")
    if not fx or not os.path.exists(p):
        return None
    d = np.load(p)
    return [int(x) for x in d["ref_bicgstab_iters"]] if "ref_bicgstab_iters" in d.files else None


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


def _job_files(wl, phi="0"):
    from emfa_gb300 import mesh as M
    sub, radius, freq, alpha, n_inc = wl
    d = tempfile.mkdtemp(prefix="emfa_cpu_")
    m = M.icosphere(sub, radius)
    nas = os.path.join(d, "job.nas")
    M.write_nas(m, nas)
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver="CFIE", mesh_path=nas, frequency=repr(freq), alpha=repr(alpha), theta="90",
                   phi=phi, pole="0")
    return d, cfg, m


def measured_farm(wl, procs, timeout=1800):
    """One full stock reference job per process, all at once, each at its
    own incidence (theta = 90, phi spread over the 360 of the job).  Returns
    the per-process stage records and the farm's wall time."""
    from emfa_gb300 import mesh as M
    exe = ensure_reference()
    if exe is None:
        return None, None
    sub, radius, freq, alpha, n_inc = wl
    d = tempfile.mkdtemp(prefix="emfa_farm_")
    m = M.icosphere(sub, radius)
    nas = os.path.join(d, "job.nas")
    M.write_nas(m, nas)
    cmds = []
    t0 = time.perf_counter()
    for p in range(procs):
        cfg = os.path.join(d, "CONFIG_%d.yml" % p)
        M.write_config(cfg, EMSolver="CFIE", mesh_path=nas, frequency=repr(freq), alpha=repr(alpha), theta="90",
                       phi=str(int(round(p * 360.0 / procs)) % 360), pole="0")
        cwd = tempfile.mkdtemp(prefix="emfa_farm_p%d_" % p)
        cmds.append(subprocess.Popen([exe, "job", cfg], cwd=cwd, stdin=subprocess.DEVNULL, stdout=subprocess.PIPE,
                                     stderr=subprocess.DEVNULL, text=True))
    out = []
    for c in cmds:
        so, _ = c.communicate(timeout=timeout)
        line = [l[l.index('{"n"'):] for l in so.splitlines() if '{"n"' in l]
        if c.returncode != 0 or not line:
            raise RuntimeError("reference job failed")
        out.append(json.loads(line[-1]))
    return out, time.perf_counter() - t0


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


def measure(wl, name, rows=1024, procs=None, steps=1, warmup=0, iters=None):
    """Returns (values, detail): RCS solves/s of the reference's CPU path per
    timed step, from the bounded sample, and what was measured."""
    procs = procs or (os.cpu_count() or 1)
    d, cfg, m = _job_files(wl)
    n_inc = wl[4]
    if iters is None:
        it = reference_iterations(name)
        iters = statistics.mean(it) if it else 10.0
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
                              "job: fill once per process + ceil(%d/%d) incidences x (fillV + %.1f BiCGStab "
                              "iterations (the reference's own count at this size) x 2 GEMV + 1 RCS)"
                              % (rows, rows, m.n_rwg_closed(), procs if exe else 1, n_inc, procs if exe else 1,
                                 iters))})
    return vals, detail


def reference_arm(args, wl, name):
    """bench.py --impl reference: the JSON line of the reference's CPU path,
    measured on full stock jobs (see the module docstring)."""
    procs = os.cpu_count() or 1
    n_inc = wl[4]
    metric = "RCS solves/s + p50/p99 latency vs plain FP64 GPU path at <=0.1 dB RCS error"
    config = {"workload": name, "n_rwg": 7680 if wl[0] == 4 else None, "n_rhs": n_inc,
              "formulation": "CFIE a=%.1f" % wl[3], "solver": "GMRES(30)+refinement tol 1e-6",
              "parallelism": "replicas"}
    recs, wall = measured_farm(wl, procs)
    if recs is None:
        vals, det = measure(wl, name, rows=1024, steps=1)
        v = vals[0]
        line_extra = {"measured": None, "model": det}
        kind, sample = det["kind"], det["sample"]
    else:
        mean = lambda k: statistics.mean(r[k] for r in recs)  # noqa: E731
        per_inc = statistics.mean(r["fillv_s"] + r["solve_s"] + r["rcs_s"] for r in recs)
        t_job = mean("init_s") + mean("fill_s") + math.ceil(n_inc / procs) * per_inc
        v = n_inc / t_job
        iters = [r["iters"] for r in recs]
        # the bounded-sample model with the farm's own iteration counts, and its error
        mvals, mdet = measure(wl, name, rows=1024, steps=1, iters=statistics.mean(iters))
        line_extra = {
            "measured": {"processes": procs, "farm_wall_s": round(wall, 2),
                         "init_s": round(mean("init_s"), 3), "fill_s": round(mean("fill_s"), 3),
                         "per_incidence_s": round(per_inc, 3), "solve_s": round(mean("solve_s"), 3),
                         "bicgstab_iterations": iters, "converged": sum(r["converged"] for r in recs),
                         "composed_job_s": round(t_job, 2),
                         "stock_solves_per_s": round(procs / wall, 4),
                         "stock": "the reference as shipped: one incidence per run, Z filled every run"},
            "model": {"value": round(mvals[0], 6), "rel_error_vs_measured": round(mvals[0] / v - 1.0, 4),
                      "sample": mdet["sample"]}}
        kind = "reference"
        sample = ("%d full stock CFIE jobs at once (7,680 RWG; theta = 90, phi spread over the 360), stage times "
                  "measured in each process; job composed as fill once per process + ceil(%d/%d) incidences x "
                  "(fillV + BiCGStab to 1e-2 + 1 RCS direction)" % (procs, n_inc, procs))
    return {"metric": metric, "impl": "reference", "value": round(v, 6), "unit": "solves/s", "n_gpus": args.gpus,
            "steps": 1, "steps_requested": args.steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64/f32 (reference value_t = float)",
            "data": "synthetic (seeded icosphere mesh)", "config": config,
            "ms_per_step": round(1e3 * n_inc / v, 3),
            "cpu_baseline": {"value": round(v, 6), "unit": "solves/s", "cores": procs, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(v, 6), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            **line_extra}
