"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own EFIE / CFIE solvers (xiangwei0909/EMFA, compiled from
its sources by oracle/build_ref.sh into oracle/_ref/) on small seeded meshes
and stores what they compute: RWG table, Z, V, the iterated current and the
bistatic RCS.  Run in the container that has the reference sources:

    bash oracle/build_ref.sh && python tests/golden/make_golden.py [names]

The fixtures are the pins of the oracle restatement (oracle/emfa_oracle.c)
and of the GPU path when the reference itself is not available.

The full-size cases (c1_*, c2_*, c3_*) are the sizes the benchmarks run at:
1,920- and 7,680-unknown dense problems and a 122,880-unknown MLFMA problem.
Their matrices are too large to store, so they keep what pins every entry in
aggregate (Z times two closed-form vectors), a few full rows, the
excitations, the exact solution I* = Z64^-1 V64 of the FP64 reference matrix
and the reference's RCS of I*.  The meshes are not stored: the generators are
deterministic, and a hash of the vertex and triangle arrays is kept to check
that a regenerated mesh is the one the reference ran on.  The C2 fill takes
about 150 s of one core in the reference, the C3 run a few minutes.
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from emfa_gb300 import mesh as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (mesh factory, solver, config overrides, solver tol, keep full Z, Z row sample)
    "sphere1_efie": (lambda: M.icosphere(1, 0.5), "efie", {"frequency": "3e8"}, 1e-4, True, None),
    "sphere1_cfie": (lambda: M.icosphere(1, 0.5), "cfie", {"frequency": "3e8", "alpha": "0.5"}, 1e-4, True, None),
    "cube2_efie_edm": (lambda: M.cube(2, 4.0), "efie", {"frequency": "3e8"}, 0, True, None),
    "ellipsoid3_cfie": (lambda: M.ellipsoid(3, (0.4, 0.3, 0.25)), "cfie",
                        {"frequency": "5e8", "alpha": "0.3", "theta": "30", "phi": "45", "pole": "30",
                         "phi_from": "45", "phi_to": "45"}, 1e-4, False, 32),
    "sphere2_cfie": (lambda: M.icosphere(2, 1.0), "cfie", {"frequency": "3e8", "alpha": "0.5"}, 1e-2, False, 16),
}


def run_mlfma_case(name, factory, over, seed=7):
    """The reference's MLFMA: octree plan, V, one mat-vec of a seeded vector
    (near part and total), BiCGStab current and RCS (box order)."""
    mesh = factory()
    tmp = tempfile.mkdtemp(prefix="golden_")
    nas = os.path.join(tmp, name + ".nas")
    M.write_nas(mesh, nas)
    cfg = os.path.join(tmp, "CONFIG.yml")
    M.write_config(cfg, **{"EMSolver": "MLFMA", "mesh_path": nas, **over})
    out = os.path.join(tmp, "out")
    O.run_reference("mlfma", cfg, out, seed, prec=32)
    d = O.load_dump(out, 32)
    rec = {"verts": mesh.verts, "tris": mesh.tris, "rwg": d["rwg"], "perm": d["perm"],
           "level_boxes": d["level_boxes"], "poles": d["poles"], "V": d["V"], "mv_x": d["mv_x"],
           "mv_y": d["mv_y"], "mv_near": d["mv_near"], "I": d["I"], "iters": d["iters"], "rcs": d["rcs"],
           "rcs_dirs": d["rcs_dirs"], "near_nnz": np.array(len(d["near_val"]))}
    rec["meta"] = np.array(repr(dict(solver="mlfma", **{k: str(v) for k, v in over.items()})))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, mesh.n_tri, "tri", d["rwg"].shape[0], "rwg", "levels", d["level_boxes"])


MLFMA_CASES = {
    "sphere3_mlfma": (lambda: M.icosphere(3, 1.0), {"frequency": "3e8", "alpha": "0.5", "mlfma_box_threshold": "0.25",
                                                    "iteration_threshold": "1e-3", "max_iteration_number": "200"}),
    "ellipsoid8_mlfma": (lambda: M.ellipsoid(8, (1.2, 0.8, 0.6)),
                         {"frequency": "4e8", "alpha": "0.3", "mlfma_box_threshold": "0.3", "theta": "40",
                          "phi": "20", "pole": "45", "phi_from": "20", "phi_to": "20",
                          "iteration_threshold": "1e-3", "max_iteration_number": "200"}),
}


def mesh_hash(mesh) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.verts, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(mesh.tris, dtype=np.int32).tobytes())
    return h.hexdigest()


BIG_CASES = {
    # name: (mesh factory, solver, config overrides, incidences (theta, phi, pole), sampled Z rows, rcs)
    # C1: plain EFIE, r = 0.5 m sphere (icosphere 3), incidence along -z, theta-polarised, bistatic RCS
    "c1_efie_sphere_1920": (lambda: M.icosphere(3, 0.5), "efie",
                            {"frequency": "3e8", "theta": "0", "phi": "0", "pole": "0", "theta_from": "0",
                             "theta_to": "180", "theta_delta": "1", "phi_from": "0", "phi_to": "0"},
                            [("0", "0", "0")], (0, 641, 1283, 1919), "bistatic"),
    # C2: CFIE alpha 0.5, r = 1 m sphere (icosphere 4), theta = 90 incidences, monostatic RCS
    "c2_cfie_sphere_7680": (lambda: M.icosphere(4, 1.0), "cfie",
                            {"frequency": "3e8", "alpha": "0.5", "theta": "90", "phi": "0", "pole": "0"},
                            [("90", "0", "0"), ("90", "137", "0")], (0, 2561, 5123, 7679), "monostatic"),
}


def run_big_case(name, factory, solver, over, incs, rows, rcs_kind):
    """One fill per precision in the reference, the excitation of every
    incidence, I* from the FP64 matrix (LAPACK through numpy) and the
    reference's RCS of I* in both precisions."""
    mesh = factory()
    tmp = tempfile.mkdtemp(prefix="golden_big_")
    nas = os.path.join(tmp, name + ".nas")
    M.write_nas(mesh, nas)
    cfg = os.path.join(tmp, "CONFIG.yml")
    M.write_config(cfg, **{"EMSolver": solver.upper(), "mesh_path": nas, **over})
    incfile = os.path.join(tmp, "inc.txt")
    with open(incfile, "w") as f:
        for t, p, q in incs:
            f.write("%s %s %s\n" % (t, p, q))
    outs = {prec: os.path.join(tmp, "out%d" % prec) for prec in (32, 64)}
    # the FP32 reference also runs its own solve per incidence (CFIE::solve's
    # BiCGStab to 1e-2): its iteration counts are the stock solver's work
    solve = {32: 1 if solver == "cfie" else 0, 64: 0}
    with ThreadPoolExecutor(2) as ex:
        list(ex.map(lambda prec: O.run_reference_args("big", cfg, outs[prec], [solver, incfile, solve[prec]],
                                                      prec=prec), (32, 64)))
    n = None
    rec = {"mesh_sha256": np.array(mesh_hash(mesh)), "n_vert": np.array(mesh.verts.shape[0]),
           "n_tri": np.array(mesh.tris.shape[0])}
    Istar = None
    for prec in (64, 32):
        d = O.load_dump(outs[prec], prec)
        n = d["n"]
        tag = "f32" if prec == 32 else "f64"
        rec["rwg_sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(d["rwg"]).tobytes()).hexdigest())
        Z = d["Z"]
        V = d["V"].reshape(len(incs), n)
        rec["inc_" + tag] = d["inc"].reshape(len(incs), 10)
        rec["V_" + tag] = V
        rec["Zrows_" + tag] = Z[list(rows)]
        if prec == 64:
            rec["Zdiag_f64"] = np.diag(Z).copy()
        # Z times two closed-form vectors, summed in complex128 (stored in
        # the dump's own precision): every entry enters these sums
        xs = np.stack([O.closed_form_vector(n, prec=64), O.closed_form_vector(n, 6007, 15485863, prec=64)])
        rec["Zx_" + tag] = (Z.astype(np.complex128) @ xs.T).T.astype(Z.dtype)
        if prec == 32 and "iters" in d:
            rec["ref_bicgstab_iters"] = d["iters"]
        if prec == 64:
            Istar = np.linalg.solve(Z, V.T).T
            rec["Istar"] = Istar
            rec["Istar_resid"] = np.array(np.linalg.norm(Z @ Istar.T - V.T) / np.linalg.norm(V))
        del Z
    rec["Zrows_index"] = np.array(rows, dtype=np.int32)
    # the reference's RCS of I*
    for prec in (32, 64):
        tag = "f32" if prec == 32 else "f64"
        cdt = np.complex64 if prec == 32 else np.complex128
        ifile = os.path.join(tmp, "I%d.bin" % prec)
        Istar.astype(cdt).tofile(ifile)
        out = os.path.join(tmp, "rcs%d" % prec)
        dirfile = os.path.join(tmp, "dirs.txt")
        if rcs_kind == "monostatic":
            kin = rec["inc_f64"][:, :3]
            with open(dirfile, "w") as f:
                for k in kin:
                    f.write("%.17g %.17g %.17g\n" % tuple(-k))
            O.run_reference_args("rcs_of", cfg, out, [solver, ifile, dirfile, "mono"], prec=prec)
            rec["rcs_dirs_" + tag] = -kin
        else:
            O.run_reference_args("rcs_of", cfg, out, [solver, ifile, dirfile, "config"], prec=prec)
            rec["rcs_dirs_" + tag] = np.fromfile(os.path.join(out, "rcs_dirs.bin"),
                                                 np.float32 if prec == 32 else np.float64).reshape(-1, 3)
        rec["rcs_" + tag] = np.fromfile(os.path.join(out, "rcs.bin"),
                                        np.float32 if prec == 32 else np.float64).reshape(len(incs), -1)
    meta = dict(solver=solver, incidences=[list(i) for i in incs], rcs=rcs_kind, **{k: str(v) for k, v in over.items()})
    rec["meta"] = np.array(repr(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, mesh.n_tri, "tri", n, "rwg", "I* residual", float(rec["Istar_resid"]))


C3_CASE = ("c3_mlfma_sphere_122880", lambda: M.icosphere(6, 5.0 * 299792458.0 / 3e8),
           {"frequency": "3e8", "alpha": "0.5", "mlfma_box_threshold": "0.25", "iteration_threshold": "1e-3",
            "max_iteration_number": "200", "thread_number": "8", "theta": "0", "phi": "0", "pole": "0",
            "theta_from": "0", "theta_to": "180", "theta_delta": "1", "phi_from": "0", "phi_to": "0"}, 8)


def run_c3_case(name, factory, over, stride):
    """The reference's MLFMA at 122,880 unknowns: plan, the product of the
    closed-form vector (seed 0) sampled every <stride> entries with the full
    norms, the excitation sample, BiCGStab iterations and bistatic RCS."""
    mesh = factory()
    tmp = tempfile.mkdtemp(prefix="golden_c3_")
    nas = os.path.join(tmp, name + ".nas")
    M.write_nas(mesh, nas)
    cfg = os.path.join(tmp, "CONFIG.yml")
    M.write_config(cfg, **{"EMSolver": "MLFMA", "mesh_path": nas, **over})
    out = os.path.join(tmp, "out")
    O.run_reference("mlfma", cfg, out, 0, prec=32, timeout=7200)
    d = O.load_dump(out, 32)
    n = d["n"]
    x = O.closed_form_vector(n)
    assert np.array_equal(x, d["mv_x"]), "closed-form vector differs from the reference's"
    idx = np.arange(0, n, stride)
    rec = {"mesh_sha256": np.array(mesh_hash(mesh)), "n_rwg": np.array(n),
           "rwg_sha256": np.array(hashlib.sha256(np.ascontiguousarray(d["rwg"]).tobytes()).hexdigest()),
           "perm_sha256": np.array(hashlib.sha256(np.ascontiguousarray(d["perm"]).tobytes()).hexdigest()),
           "perm_head": d["perm"][:4096].copy(),
           "level_boxes": d["level_boxes"], "poles": d["poles"], "sample_index": idx.astype(np.int32),
           "V_sample": d["V"][idx], "V_norm": np.array(np.linalg.norm(d["V"].astype(np.complex128))),
           "mv_y_sample": d["mv_y"][idx], "mv_y_norm": np.array(np.linalg.norm(d["mv_y"].astype(np.complex128))),
           "mv_near_sample": d["mv_near"][idx],
           "mv_near_norm": np.array(np.linalg.norm(d["mv_near"].astype(np.complex128))),
           "I_sample": d["I"][idx], "I_norm": np.array(np.linalg.norm(d["I"].astype(np.complex128))),
           "iters": d["iters"], "rcs": d["rcs"], "rcs_dirs": d["rcs_dirs"],
           "near_nnz": np.array(len(d["near_val"]))}
    rec["meta"] = np.array(repr(dict(solver="mlfma", **{k: str(v) for k, v in over.items()})))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, mesh.n_tri, "tri", n, "rwg", "levels", d["level_boxes"], "iters", d["iters"])


def run_case(name, factory, solver, over, tol, full_z, rows):
    mesh = factory()
    tmp = tempfile.mkdtemp(prefix="golden_")
    nas = os.path.join(tmp, name + ".nas")
    M.write_nas(mesh, nas)
    cfg = os.path.join(tmp, "CONFIG.yml")
    M.write_config(cfg, **{"EMSolver": solver.upper(), "mesh_path": nas, **over})
    rec = {"verts": mesh.verts, "tris": mesh.tris}
    for prec in (32, 64):
        out = os.path.join(tmp, "out%d" % prec)
        O.run_reference(solver, cfg, out, tol if tol > 0 else -1, prec=prec)
        d = O.load_dump(out, prec)
        tag = "f32" if prec == 32 else "f64"
        rec["rwg"] = d["rwg"]
        rec["inc_" + tag] = d["inc"]
        Z = d["Z"]
        if full_z:
            rec["Z_" + tag] = Z
            if "Z_arma" in d:
                rec["Zarma_" + tag] = d["Z_arma"]
        else:
            rec["Zrows_" + tag] = Z[:rows]
            rec["Zdiag_" + tag] = np.diag(Z).copy()
        rec["V_" + tag] = d["V"]
        if "I" in d:
            rec["I_" + tag] = d["I"]
            rec["rcs_" + tag] = d["rcs"]
            rec["rcs_dirs_" + tag] = d["rcs_dirs"]
        if "iters" in d:
            rec["iters_" + tag] = d["iters"]
    meta = dict(solver=solver, tol=tol, **{k: str(v) for k, v in over.items()})
    rec["meta"] = np.array(repr(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, mesh.n_tri, "tri", rec["rwg"].shape[0], "rwg")


if __name__ == "__main__":
    if O.ref_binary(32) is None or O.ref_binary(64) is None:
        sys.exit("reference binaries missing: run oracle/build_ref.sh first")
    only = sys.argv[1:]
    for name, args in CASES.items():
        if only and name not in only:
            continue
        run_case(name, *args)
    for name, (factory, over) in MLFMA_CASES.items():
        if only and name not in only:
            continue
        run_mlfma_case(name, factory, over)
    # full-size cases: only when named (minutes of reference CPU time each)
    for name, args in BIG_CASES.items():
        if name in only:
            run_big_case(name, *args)
    if C3_CASE[0] in only:
        run_c3_case(*C3_CASE)
