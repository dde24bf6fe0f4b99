"""Parity at the benchmark sizes, against the reference's own runs at those
sizes (tests/golden/c1_*, c2_*, c3_*, made by tests/golden/make_golden.py
from the compiled reference):

  C1  plain EFIE, r = 0.5 m sphere, icosphere 3: 1,920 RWG, -z incidence,
      bistatic RCS (theta cut + theta = 90 ring, 541 directions)
  C2  CFIE alpha 0.5, r = 1 m sphere, icosphere 4: 7,680 RWG, theta = 90
      incidences at phi = 0 and 137 degrees, monostatic RCS
  C3  MLFMA CFIE alpha 0.5, 5-wavelength sphere, icosphere 6: 122,880 RWG,
      0.25-wavelength boxes, one plane wave along -z, bistatic RCS

The full matrices are not stored: each fixture keeps a few full rows, the
diagonal (FP64) and Z times two closed-form vectors, which every entry
enters.  Tolerances (written in the asserts):
  FP64 fill        rows floored rel 1e-11, normwise 1e-12; Z x normwise 1e-12
  FP32 fill        rows floored (floor 1e-3 max|Z|) no worse than 1.5x the
                   reference's own FP32 fill against its FP64 fill (at least
                   1e-5); Z x normwise likewise
  excitation       2e-6 of max|V| (FP32), 1e-12 (FP64)
  current          rel L2 1e-4 against I* = Z64^-1 V64 of the reference's
                   FP64 matrix (solved with LAPACK when the fixture was made)
  RCS              0.1 dB against the reference's RCS of I* (the north-star
                   bar); the plain FP64 path 1e-4 dB
  MLFMA product    near part rel 1e-5, total 2e-4, far part 1e-3 (on every
                   8th entry, plus the full norms)
  MLFMA RCS        0.1 dB against the reference's MLFMA run (its BiCGStab
                   to 1e-3), away from the pattern's deep nulls
"""
import hashlib

import numpy as np
import pytest

from conftest import load_golden
from emfa_gb300 import mesh as M

pytestmark = pytest.mark.gpu

LAMBDA_300MHZ = 299792458.0 / 3e8
MESHES = {
    "c1_efie_sphere_1920": lambda: M.icosphere(3, 0.5),
    "c2_cfie_sphere_7680": lambda: M.icosphere(4, 1.0),
    "c3_mlfma_sphere_122880": lambda: M.icosphere(6, 5.0 * LAMBDA_300MHZ),
}
DENSE = ["c1_efie_sphere_1920", "c2_cfie_sphere_7680"]


def mesh_sha(m):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(m.verts, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(m.tris, dtype=np.int32).tobytes())
    return h.hexdigest()


def floored_rel(a, b, floor=1e-3):
    return np.abs(a - b) / np.maximum(np.abs(b), floor * np.abs(b).max())


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def closed_form(n):
    from oracle import oracle as O
    return np.stack([O.closed_form_vector(n, prec=64), O.closed_form_vector(n, 6007, 15485863, prec=64)])


def fill_params(g, prec):
    from emfa_gb300 import api
    m = g["meta"]
    alpha = float(np.float32(float(m.get("alpha", 1))))
    return api.fill_params(m["solver"], prec, float(m["frequency"]), alpha)


def angles(g):
    return np.array([[float(t), float(p), float(q)] for t, p, q in g["meta"]["incidences"]])


@pytest.fixture(scope="module")
def dense(ctx):
    """Per dense config: fixture, mesh, geometry (RWG by the library's own
    builder) and the FP32 / FP64 matrices, filled once."""
    from emfa_gb300 import api
    out = {}
    for name in DENSE:
        g = load_golden(name)
        m = MESHES[name]()
        geo = api.Geometry(ctx, m)
        out[name] = {"g": g, "mesh": m, "geo": geo}
    yield out
    for v in out.values():
        v.pop("Z32", None)
        v.pop("Z64", None)
        v["geo"].close()


def matrix(case, prec):
    from emfa_gb300 import api
    key = "Z32" if prec == "f32" else "Z64"
    if key not in case:
        for k in ("Z32", "Z64"):  # one matrix at a time on the device
            case.pop(k, None)
        case[key] = api.fill_z(case["geo"], fill_params(case["g"], prec))
    return case[key]


@pytest.mark.parametrize("name", DENSE)
def test_mesh_and_rwg_are_the_reference_run(dense, name):
    c = dense[name]
    assert mesh_sha(c["mesh"]) == str(c["g"]["mesh_sha256"])
    rwg = np.ascontiguousarray(c["geo"].rwg, dtype=np.int32)
    assert hashlib.sha256(rwg.tobytes()).hexdigest() == str(c["g"]["rwg_sha256"])


@pytest.mark.parametrize("name", DENSE)
def test_fill_fp64_at_config_size(dense, name):
    import torch
    c, g = dense[name], dense[name]["g"]
    Z = matrix(c, "f64")
    rows = g["Zrows_index"].astype(np.int64)
    Zr = Z[torch.as_tensor(rows, device=Z.device)].cpu().numpy()
    assert floored_rel(Zr, g["Zrows_f64"]).max() < 1e-11
    assert rel(Zr, g["Zrows_f64"]) < 1e-12
    assert floored_rel(torch.diagonal(Z).cpu().numpy(), g["Zdiag_f64"]).max() < 1e-11
    xs = torch.as_tensor(closed_form(Z.shape[0]), device=Z.device)
    Zx = (Z @ xs.T).T.cpu().numpy()
    assert rel(Zx, g["Zx_f64"]) < 1e-12, rel(Zx, g["Zx_f64"])


@pytest.mark.parametrize("name", DENSE)
def test_fill_fp32_at_config_size(dense, name):
    import torch
    c, g = dense[name], dense[name]["g"]
    Z = matrix(c, "f32")
    rows = g["Zrows_index"].astype(np.int64)
    Zr = Z[torch.as_tensor(rows, device=Z.device)].cpu().numpy()
    ref_own = floored_rel(g["Zrows_f32"], g["Zrows_f64"]).max()
    ours = floored_rel(Zr, g["Zrows_f64"]).max()
    assert ours <= max(1e-5, 1.5 * ref_own), (ours, ref_own)
    xs = torch.as_tensor(closed_form(Z.shape[0]), device=Z.device)
    Zx = (Z.to(torch.complex128) @ xs.T).T.cpu().numpy()
    ref_own_x = rel(g["Zx_f32"], g["Zx_f64"])
    assert rel(Zx, g["Zx_f64"]) <= max(1e-5, 1.5 * ref_own_x), (rel(Zx, g["Zx_f64"]), ref_own_x)


@pytest.mark.parametrize("name", DENSE)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_excitation_at_config_size(dense, name, prec):
    from emfa_gb300 import api
    c, g = dense[name], dense[name]["g"]
    V = api.fill_v(c["geo"], fill_params(g, prec), angles(g)).cpu().numpy()
    Vr = g["V_" + prec]
    tol = 2e-6 if prec == "f32" else 1e-12
    assert np.abs(V - Vr).max() <= tol * np.abs(Vr).max()


def _rcs_dirs(g, prec):
    d = g["rcs_dirs_" + prec].astype(np.float64)
    if g["meta"]["rcs"] == "monostatic":
        return d[:, None, :], True
    return d, False


@pytest.mark.parametrize("name", DENSE)
def test_plain_fp64_solve_and_rcs(dense, name):
    """The plain path: FP64 fill, FP64 GMRES(30) to 1e-10."""
    import torch
    from emfa_gb300 import api
    c, g = dense[name], dense[name]["g"]
    fp = fill_params(g, "f64")
    Z = matrix(c, "f64")
    V = api.fill_v(c["geo"], fp, angles(g))
    X, info = api.solve(c["geo"].ctx, Z, V, api.solver_params("gmres", restart=30, tol=1e-10, max_iter=20000))
    assert info.converged == V.shape[0], (info.iterations, info.max_rel_residual)
    I = X.cpu().numpy()
    assert rel(I, g["Istar"]) < 1e-8, rel(I, g["Istar"])
    d, per = _rcs_dirs(g, "f64")
    r = api.rcs(c["geo"], fp, X, d, per_rhs=per)
    assert np.abs(r - g["rcs_f64"]).max() < 1e-4, np.abs(r - g["rcs_f64"]).max()
    del torch


@pytest.mark.parametrize("name", DENSE)
def test_mixed_solve_current_and_rcs(dense, name):
    """The mixed path of each config: FP32 fill (FP64 self terms), then
    split-FP16 GMRES(30) with FP64 refinement to 1e-6 for CFIE, the FP32 LU
    with FP64 refinement for EFIE."""
    from emfa_gb300 import api
    c, g = dense[name], dense[name]["g"]
    fp = fill_params(g, "f32")
    Z = matrix(c, "f32")
    V = api.fill_v(c["geo"], fp, angles(g))
    method = "lu" if g["meta"]["solver"] == "efie" else "gmres"
    X, info = api.solve(c["geo"].ctx, Z, V, api.solver_params(method, restart=30, tol=1e-6, max_iter=3000))
    assert info.converged == V.shape[0], (info.iterations, info.max_rel_residual)
    I = X.cpu().numpy()
    err = rel(I, g["Istar"])
    # the FP32 fill itself moves the exact solution: for the first-kind EFIE
    # (condition number ~1e3 here) by more than for CFIE; the current of the
    # mixed path is held to the benchmark spec's 1e-4 where the FP32 matrix's own
    # solution is (its FP64 solve is the bound), and to 1e-4 always for CFIE
    if g["meta"]["solver"] == "cfie":
        assert err < 1e-4, err
    else:
        Xd, _ = api.solve(c["geo"].ctx, Z, V, api.solver_params("lu", tol=1e-12, max_iter=50))
        floor = rel(Xd.cpu().numpy(), g["Istar"])
        assert err < max(1e-4, 1.1 * floor), (err, floor)
    d, per = _rcs_dirs(g, "f32")
    r = api.rcs(c["geo"], fp, X, d, per_rhs=per)
    assert np.abs(r - g["rcs_f64"]).max() < 0.1, np.abs(r - g["rcs_f64"]).max()


def test_c2_job_end_to_end_from_host_buffers(dense):
    """The headline job's host-buffer entry point (emfa_dense_rcs), on the
    fixture's incidences: monostatic RCS within 0.1 dB of the reference's."""
    from emfa_gb300 import api
    c, g = dense["c2_cfie_sphere_7680"], dense["c2_cfie_sphere_7680"]["g"]
    c.pop("Z32", None)
    c.pop("Z64", None)
    ang = angles(g)
    out, info, I = api.dense_rcs(c["geo"].ctx, c["mesh"], fill_params(g, "f32"), ang,
                                 api.solver_params("gmres", restart=30, tol=1e-6, max_iter=3000),
                                 api.monostatic_dirs(ang), per_rhs=True, want_current=True)
    assert info.converged == len(ang)
    assert np.abs(out - g["rcs_f64"]).max() < 0.1, np.abs(out - g["rcs_f64"]).max()
    assert rel(I, g["Istar"]) < 1e-4, rel(I, g["Istar"])


def test_c1_against_the_mie_series(dense):
    """Independent check: the plain FP64 path's bistatic RCS against the
    analytic Mie series of the sphere, no further than the reference's own
    discretisation is (0.18 dB at this mesh) plus 0.01 dB."""
    from emfa_gb300 import api
    from oracle import mie
    c, g = dense["c1_efie_sphere_1920"], dense["c1_efie_sphere_1920"]["g"]
    fp = fill_params(g, "f64")
    Z = matrix(c, "f64")
    V = api.fill_v(c["geo"], fp, angles(g))
    X, info = api.solve(c["geo"].ctx, Z, V, api.solver_params("gmres", restart=30, tol=1e-8, max_iter=20000))
    d = g["rcs_dirs_f64"].astype(np.float64)
    r = api.rcs(c["geo"], fp, X, d)[0]
    inc = g["inc_f64"][0]
    exact = mie.pec_sphere_rcs_db(0.5, 3e8, inc[:3], inc[3:6], d)
    ref_err = np.abs(g["rcs_f64"][0] - exact).max()
    assert np.abs(r - exact).max() <= ref_err + 0.01, (np.abs(r - exact).max(), ref_err)


# --------------------------------------------------------------------------
# C3: MLFMA at 122,880 unknowns
# --------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c3(ctx):
    from emfa_gb300 import api
    g = load_golden("c3_mlfma_sphere_122880")
    m = MESHES["c3_mlfma_sphere_122880"]()
    geo = api.Geometry(ctx, m)
    mt = g["meta"]
    mp = api.mlfma_params(float(mt["frequency"]), float(np.float32(float(mt["alpha"]))),
                          float(np.float32(float(mt["mlfma_box_threshold"]))))
    ml = api.Mlfma(geo, mp)
    yield g, m, geo, ml
    ml.close()
    geo.close()


def test_c3_plan(c3):
    g, m, geo, ml = c3
    assert mesh_sha(m) == str(g["mesh_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(geo.rwg, dtype=np.int32).tobytes()).hexdigest() == str(g["rwg_sha256"])
    assert np.array_equal(ml.level_boxes, g["level_boxes"])
    assert np.array_equal(ml.poles, g["poles"])
    assert np.array_equal(ml.perm[:4096], g["perm_head"])
    assert hashlib.sha256(np.ascontiguousarray(ml.perm, dtype=np.int32).tobytes()).hexdigest() == str(g["perm_sha256"])
    # the reference's sparse matrix drops entries that are exactly zero
    assert int(g["near_nnz"]) <= ml.nnz <= int(g["near_nnz"]) + 64


def test_c3_operator(c3):
    import torch
    from oracle import oracle as O
    g, m, geo, ml = c3
    idx = g["sample_index"].astype(np.int64)
    x = torch.as_tensor(O.closed_form_vector(geo.n), device="cuda")
    near = ml.apply_part(x, 1).cpu().numpy()
    assert rel(near[idx], g["mv_near_sample"]) < 1e-5
    assert abs(np.linalg.norm(near) / float(g["mv_near_norm"]) - 1) < 1e-5
    y = ml.apply(x[None])[0].cpu().numpy()
    assert rel(y[idx], g["mv_y_sample"]) < 2e-4, rel(y[idx], g["mv_y_sample"])
    assert abs(np.linalg.norm(y) / float(g["mv_y_norm"]) - 1) < 2e-4
    far = ml.apply_part(x, 2).cpu().numpy()
    far_ref = g["mv_y_sample"] - g["mv_near_sample"]
    assert rel(far[idx], far_ref) < 1e-3, rel(far[idx], far_ref)


def test_c3_excitation(c3):
    g, m, geo, ml = c3
    V = ml.fill_v(np.array([[0.0, 0.0, 0.0]])).cpu().numpy()[0]
    idx = g["sample_index"].astype(np.int64)
    assert np.abs(V[idx] - g["V_sample"]).max() <= 2e-6 * np.abs(g["V_sample"]).max()
    assert abs(np.linalg.norm(V) / float(g["V_norm"]) - 1) < 1e-6


def test_c3_solve_and_rcs(c3):
    """GMRES(30) to 1e-3 (the configuration's solver) against the
    reference's BiCGStab(1e-3) run: currents within 1e-2, bistatic RCS
    within 0.1 dB wherever the pattern is within 20 dB of its peak (at the
    deep nulls of a 5-wavelength sphere's pattern two solutions converged to
    1e-3 differ by more in dB while agreeing in field)."""
    import torch
    from emfa_gb300 import api
    g, m, geo, ml = c3
    V = ml.fill_v(np.array([[0.0, 0.0, 0.0]]))
    X, info = ml.solve(V, api.solver_params("gmres", restart=30, tol=1e-3, max_iter=300))
    assert info.converged == 1
    idx = g["sample_index"].astype(np.int64)
    Ibox = X.cpu().numpy()[0]
    assert rel(Ibox[idx], g["I_sample"]) < 1e-2, rel(Ibox[idx], g["I_sample"])
    Irwg = ml.unpermute(X)
    r = api.rcs(geo, api.fill_params("cfie", "f32", 3e8, 0.5), Irwg, g["rcs_dirs"].astype(np.float64))[0]
    ref = g["rcs"]
    keep = ref > ref.max() - 20.0
    assert np.abs(r - ref)[keep].max() < 0.1, np.abs(r - ref)[keep].max()
    del torch


def test_c1_config_discretisation_against_mie(dense):
    """C1 in the discretisation the configuration states (7-point rule,
    self and edge-adjacent extraction): FP64 fill, GMRES to 1e-8; its
    bistatic RCS against the Mie series is no worse than the reference
    discretisation's (0.18 dB), and both errors are reported by the bench."""
    from emfa_gb300 import api
    from oracle import mie
    c, g = dense["c1_efie_sphere_1920"], dense["c1_efie_sphere_1920"]["g"]
    c.pop("Z32", None)
    c.pop("Z64", None)
    fp = api.fill_params("efie", "f64", 3e8, 1.0, discretisation="config")
    Z = api.fill_z(c["geo"], fp)
    V = api.fill_v(c["geo"], fp, angles(g))
    X, info = api.solve(c["geo"].ctx, Z, V, api.solver_params("gmres", restart=30, tol=1e-8, max_iter=20000))
    assert info.converged == 1
    d = g["rcs_dirs_f64"].astype(np.float64)
    r = api.rcs(c["geo"], fp, X, d)[0]
    inc = g["inc_f64"][0]
    exact = mie.pec_sphere_rcs_db(0.5, 3e8, inc[:3], inc[3:6], d)
    ref_err = np.abs(g["rcs_f64"][0] - exact).max()
    assert np.abs(r - exact).max() <= ref_err, (np.abs(r - exact).max(), ref_err)
