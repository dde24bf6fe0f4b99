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
