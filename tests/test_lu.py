"""Dense LU solve (EMFA_LU) through the C ABI: FP32 LU with row exchanges
inside each 64-row diagonal block, explicit inverses of the diagonal blocks,
FP64 iterative refinement on the true residual, GMRES-IR when a pivot is zero
or the refinement stalls.  The reference has no dense direct solver on this
path (its dense solves are GMRES/BiCGStab), so the checks are against numpy's
FP64 solve of the same FP32-rounded matrix, and against the reference's own
golden EFIE current.

Tolerances (written here):
  true residual ||b - Z x|| / ||b||, recomputed in FP64     < 2e-6 at tol 1e-6
  solution vs numpy FP64 solve, random matrices (cond < 10)  rel L2 < 1e-5
  EFIE current vs I* = Z64^-1 V64                             rel L2 < 1e-4 (as the Krylov tests)
"""
import numpy as np
import pytest

from conftest import load_golden
from emfa_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _f32(a):
    return np.asarray(a).astype(np.complex64).astype(np.complex128)


def _solve(ctx, Z, B, tol=1e-6, **kw):
    import torch
    from emfa_gb300 import api
    Zd = torch.from_numpy(np.ascontiguousarray(Z.astype(np.complex64))).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B.astype(np.complex64))).cuda()
    X, info = api.solve(ctx, Zd, Bd, api.solver_params("lu", tol=tol, **kw))
    return X.cpu().numpy(), info


def _check(Z, B, X, err_bound=1e-5):
    Z32, B32 = _f32(Z), _f32(B)
    res = np.linalg.norm(B32 - X @ Z32.T, axis=1) / np.linalg.norm(B32, axis=1)
    assert res.max() < 2e-6, res.max()
    Xs = np.linalg.solve(Z32, B32.T).T
    err = np.linalg.norm(X - Xs) / np.linalg.norm(Xs)
    assert err < err_bound, err


def _random(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Z += 3.0 * np.sqrt(n) * np.eye(n)
    B = rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))
    return Z, B


@pytest.mark.parametrize("n,nrhs", [(1, 1), (63, 3), (64, 8), (65, 1), (130, 9), (1000, 8), (1537, 17), (700, 100)])
def test_lu_random_matches_numpy(ctx, n, nrhs):
    """Block edges (n = 63, 64, 65, a ragged last block), one to 100
    right-hand sides (several sweep chunks of 8, a ragged last chunk)."""
    Z, B = _random(n, nrhs, n)
    X, info = _solve(ctx, Z, B)
    assert info.converged == nrhs, (info.iterations, info.max_rel_residual)
    assert info.iterations <= 4  # refinement passes
    _check(Z, B, X)


def test_lu_pivots_inside_blocks(ctx):
    """Every diagonal entry is small: each 64-row block is a shifted identity
    (a derangement) plus noise, so each pivot comes from another row of the
    block."""
    rng = np.random.default_rng(5)
    n = 200
    Z = 0.05 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    for k0 in range(0, n, 64):
        nb = min(64, n - k0)
        for i in range(nb):
            Z[k0 + i, k0 + (i + 1) % nb] += 4.0 + 1.0j
        for i in range(nb):
            Z[k0 + i, k0 + i] = 1e-3 * (rng.standard_normal() + 1j * rng.standard_normal())
    B = rng.standard_normal((4, n)) + 1j * rng.standard_normal((4, n))
    X, info = _solve(ctx, Z, B)
    assert info.converged == 4
    _check(Z, B, X)


def test_lu_zero_pivot_hands_over_to_gmres(ctx):
    """The leading 64 x 64 block is zero, so the first diagonal block has no
    pivot within its rows; the factor records it and GMRES-IR carries the
    solve."""
    rng = np.random.default_rng(6)
    n = 128
    E = 0.05 * (rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))) / 8
    Z = np.zeros((n, n), dtype=np.complex128)
    Z[:64, 64:] = np.eye(64) + E
    Z[64:, :64] = np.eye(64) + E.T
    Z[64:, 64:] = 0.5 * np.eye(64)
    B = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    X, info = _solve(ctx, Z, B, max_iter=2000)
    assert info.converged == 2, (info.iterations, info.max_rel_residual)
    _check(Z, B, X)


def test_lu_bad_precision_rejected(ctx):
    import torch
    from emfa_gb300 import api, _lib as L
    Z = torch.eye(4, dtype=torch.complex128, device="cuda")
    B = torch.ones((1, 4), dtype=torch.complex128, device="cuda")
    with pytest.raises(Exception):
        api.solve(ctx, Z, B, api.solver_params("lu"))


@pytest.mark.parametrize("name", ["sphere1_efie", "sphere1_cfie"])
def test_lu_golden_current(ctx, name):
    """The FP32 fill of the reference's C1-shaped EFIE and CFIE cases solved
    by LU: the current matches I* = Z64^-1 V64 of the reference's FP64
    matrix as tightly as the Krylov solves do, in a few refinement passes."""
    from emfa_gb300 import api
    g = load_golden(name)
    geo = api.Geometry(ctx, M.TriMesh(g["verts"], g["tris"]), g["rwg"])
    m = g["meta"]
    fp = api.fill_params(m["solver"], "f32", float(m["frequency"]), float(np.float32(float(m.get("alpha", 1)))))
    ang = np.array([[float(m.get("theta", 0)), float(m.get("phi", 0)), float(m.get("pole", 0))]])
    Z = api.fill_z(geo, fp)
    V = api.fill_v(geo, fp, ang)
    X, info = api.solve(ctx, Z, V, api.solver_params("lu", tol=1e-6))
    assert info.converged == 1 and info.iterations <= 4, (info.iterations, info.max_rel_residual)
    Istar = np.linalg.solve(g["Z_f64"], g["V_f64"]) if "Z_f64" in g else None
    if Istar is not None:
        I = X.cpu().numpy()[0]
        assert np.linalg.norm(I - Istar) / np.linalg.norm(Istar) < 1e-4


def test_lu_agrees_with_gmres_on_batch_problem(ctx):
    """A C4-shaped EFIE problem (ellipsoid at lambda/10, 8 incidences, about
    3,000 unknowns): LU and GMRES(250) reach the same currents."""
    from emfa_gb300 import api, workloads as W
    probs = W.batch_set(seed=0, count=64)
    sizes = [api.build_rwg(m.tris).shape[0] for (m, f, a, d) in probs]
    i = int(np.argmin([abs(s - 3000) for s in sizes]))
    m, f, ang, d = probs[i]
    geo = api.Geometry(ctx, m)
    fp = api.fill_params("efie", "f32", f, 1.0)
    Z = api.fill_z(geo, fp)
    V = api.fill_v(geo, fp, ang)
    Xl, il = api.solve(ctx, Z, V, api.solver_params("lu", tol=1e-5))
    Xg, ig = api.solve(ctx, Z, V, api.solver_params("gmres", restart=250, max_iter=5000, tol=1e-5))
    assert il.converged == V.shape[0] and ig.converged == V.shape[0]
    a, b = Xl.cpu().numpy(), Xg.cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-3  # both within 1e-5 residual of an EFIE system
