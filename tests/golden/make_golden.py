"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own EFIE / CFIE solvers (xiangwei0909/EMFA, compiled from
its sources by oracle/build_ref.sh into oracle/_ref/) on small seeded meshes
and stores what they compute: RWG table, Z, V, the iterated current and the
bistatic RCS.  Run in the container that has the reference sources:

    bash oracle/build_ref.sh && python tests/golden/make_golden.py

The fixtures are the pins of the oracle restatement (oracle/emfa_oracle.c)
and of the GPU path when the reference itself is not available.
"""
from __future__ import annotations

import os
import sys
import tempfile

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
