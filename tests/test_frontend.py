"""C++ front end with the reference's solver surface (emfa_launcher):
config parsing and error mapping (CPU), and the EFIE / CFIE lifecycle with
the reference's output files (GPU)."""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import load_golden
from emfa_gb300 import mesh as M

LAUNCHER = os.path.join(os.path.dirname(__file__), "..", "emfa_gb300", "_build", "emfa_launcher")


def run(args, stdin=None, cwd=None, timeout=600):
    return subprocess.run([LAUNCHER, *args], input=stdin, capture_output=True, text=True, cwd=cwd, timeout=timeout)


def test_config_parsing(emfa_lib):
    d = tempfile.mkdtemp()
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver="CFIE", alpha="0.3", frequency="5e8", theta="30", phi="45", pole="30",
                   Sigma="(0.0025,0)", mesh_path="/x/y/mesh.nas")
    with open(cfg, "a") as f:
        f.write("# a comment line\n    gpu_precision: f64\n")
    r = run(["--check-config", cfg])
    assert r.returncode == 0, r.stdout + r.stderr
    v = json.loads(r.stdout)
    assert v["solver"] == "CFIE" and abs(v["alpha"] - 0.3) < 1e-7 and v["freq"] == 5e8
    assert v["theta"] == 30 and v["pole"] == 30 and v["sigma"] == [0.0025, 0]
    assert v["gpu_precision"] == "f64" and v["precond"] == 0


def test_config_errors_map_like_the_reference(emfa_lib):
    d = tempfile.mkdtemp()
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, alpha="zero")
    r = run(["--check-config", cfg])
    assert r.returncode == 2 and "fail parsing combined coefficient" in r.stdout
    M.write_config(cfg, row_threshold="0.5")
    r = run([cfg])
    # missing mesh file surfaces as a File Error through the full launcher
    assert "Exit State: [File Error]" in r.stdout or "Exit State: [Runtime Error]" in r.stdout
    r = run([os.path.join(d, "missing.yml")])
    assert "Exit State: [ConfigParameter Error]fail opening config file" in r.stdout
    with open(cfg, "w") as f:
        f.write("EMSolver: EFIE\n")
    r = run([cfg])
    assert "Exit State: [Unrecognized Error]" in r.stdout  # missing key: std::out_of_range


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["efie", "cfie"])
def test_launcher_end_to_end_vs_reference(emfa_lib, solver):
    """CONFIG.yml in, the reference's bistatic RCS files out, values within
    0.1 dB of the reference's own run on the same mesh."""
    g = load_golden("sphere1_" + solver)
    d = tempfile.mkdtemp()
    nas = os.path.join(d, "sph.nas")
    M.write_nas(M.TriMesh(g["verts"], g["tris"]), nas)
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver=solver.upper(), mesh_path=nas, frequency="3e8", alpha="0.5")
    r = run([], stdin=cfg + "\n", cwd=d)
    assert "Exit State: OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
    out = os.path.join(d, "sph_EFIE" if solver == "efie" else "sph_CFIE_0.5")
    for fn, sl in (("bistatic_rcs_phi_0.dat", slice(0, 181)), ("bistatic_rcs_theta_90.dat", slice(181, 541))):
        lines = open(os.path.join(out, fn)).read().splitlines()
        assert lines[0].split() == ["Theta", "RCS(dBm^2)"]
        vals = np.array([float(l.split()[1]) for l in lines[1:]])
        ref = g["rcs_f32"][sl]
        assert len(vals) == len(ref)
        assert np.abs(vals - ref).max() < 0.1, np.abs(vals - ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("precond", ["false", "true"])
def test_launcher_mlfma_vs_reference(emfa_lib, precond):
    """MLFMA through CONFIG.yml, without and with the SAI preconditioner
    (preconditioning: true, row/col thresholds 0.9/0.87): bistatic RCS within
    0.1 dB of the reference's own (unpreconditioned) MLFMA run on the same
    mesh."""
    g = load_golden("sphere3_mlfma")
    d = tempfile.mkdtemp()
    nas = os.path.join(d, "sph.nas")
    M.write_nas(M.TriMesh(g["verts"], g["tris"]), nas)
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver="MLFMA", mesh_path=nas, frequency="3e8", alpha="0.5", mlfma_box_threshold="0.25",
                   iteration_threshold="1e-3", max_iteration_number="200", preconditioning=precond)
    r = run([cfg], cwd=d)
    assert "Exit State: OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
    out = os.path.join(d, "sph_MLFMA_CFIE_0.5")
    lines = open(os.path.join(out, "bistatic_rcs_phi_0.dat")).read().splitlines()
    vals = np.array([float(l.split()[1]) for l in lines[1:]])
    assert np.abs(vals - g["rcs"][:181]).max() < 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["efie", "cfie"])
def test_launcher_monostatic_sweep(emfa_lib, oracle_mod, solver):
    """result_type: MonostaticRCS writes the reference's monostatic layout
    (Result::getMonostaticRCS, EMComponent/Result.h:106-155): one file per phi
    cut over theta, then the theta = 90 ring, each value the backscatter RCS
    of its own incidence, all solved as one block of right-hand sides.  Each
    of the 374 values is checked against a separate solve of that incidence
    by the oracle restatement of the reference's fill, excitation and RCS
    (FP64, direct solve), within 0.01 dB; the solver runs to a tight
    tolerance (gpu_efie_tol / gpu_cfie_tol) in FP64."""
    O = oracle_mod
    g = load_golden("sphere1_" + solver)
    d = tempfile.mkdtemp()
    nas = os.path.join(d, "sph.nas")
    M.write_nas(M.TriMesh(g["verts"], g["tris"]), nas)
    cfg = os.path.join(d, "CONFIG.yml")
    M.write_config(cfg, EMSolver=solver.upper(), mesh_path=nas, frequency="3e8", alpha="0.5",
                   result_type="MonostaticRCS", theta_from="0", theta_to="180", theta_delta="30", phi_from="0",
                   phi_to="90", phi_delta="90", pole="0", gpu_precision="f64", gpu_efie_tol="1e-10",
                   gpu_cfie_tol="1e-10")
    r = run([cfg], cwd=d)
    assert "Exit State: OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
    out = os.path.join(d, "sph_EFIE" if solver == "efie" else "sph_CFIE_0.5")
    angles, vals = [], []
    for fn, phi in (("monostatic_rcs_phi_0.dat", 0.0), ("monostatic_rcs_phi_90.dat", 90.0),
                    ("monostatic_rcs_theta_90.dat", None)):
        lines = open(os.path.join(out, fn)).read().splitlines()
        assert lines[0].split() == ["Theta", "RCS(dBm^2)"]
        rows = [l.split() for l in lines[1:]]
        assert len(rows) == (7 if phi is not None else 360)
        for a, v in rows:
            angles.append((float(a), phi) if phi is not None else (90.0, float(a)))
            vals.append(float(v))
    assert not os.path.exists(os.path.join(out, "bistatic_rcs_phi_0.dat"))
    ang = np.array(angles)
    og = O.Geometry(g["verts"], g["tris"], g["rwg"], 64)
    k = O.wavenumber(3e8, 64)
    if solver == "efie":
        Z = O.fill_z_efie(og, k)
    else:
        Z = O.fill_z_cfie(og, k, 0.5)
    inc = np.stack([O.incidence(t, p, 0.0, prec=64) for t, p in ang])
    V = O.fill_v(og, k, inc, cfie=solver == "cfie", alpha=0.5)
    I = np.linalg.solve(Z, V.T).T
    th, ph = np.deg2rad(ang[:, 0]), np.deg2rad(ang[:, 1])
    dirs = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    ref = np.array([O.rcs(og, k, I[i:i + 1], dirs[i:i + 1])[0, 0] for i in range(len(ang))])
    assert np.abs(np.array(vals) - ref).max() < 0.01, np.abs(np.array(vals) - ref).max()
