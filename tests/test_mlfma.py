"""MLFMA: the octree plan (CPU) and the operator (GPU) against the
reference's own MLFMA run on the same meshes (tests/golden/*_mlfma.npz).

Tolerances:
  plan (levels, boxes per level, multipoles, box order)  exact
  near-field part of the mat-vec                         rel L2 1e-5 (FP32 fill)
  full mat-vec (near + far)                              rel L2 2e-4: the translation
      operators are tabulated per box offset from exact offsets and summed in a
      different order; the far field itself is accurate to ~1e-3
  current vs the reference's BiCGStab(1e-3) current       rel L2 1e-2
  current vs the dense CFIE solution                      no worse than the reference's own
      MLFMA current (1.1x + 2e-3): the reference's MLFMA is 5-16% off the dense
      solution on these meshes
  bistatic RCS vs the reference                           0.1 dB
"""
import numpy as np
import pytest

from conftest import load_golden
from emfa_gb300 import mesh as M

CASES = ["sphere3_mlfma", "ellipsoid8_mlfma"]


def params(g):
    from emfa_gb300 import api
    m = g["meta"]
    return api.mlfma_params(float(m["frequency"]), float(np.float32(float(m["alpha"]))),
                            float(np.float32(float(m["mlfma_box_threshold"]))))


def angles(g):
    m = g["meta"]
    return np.array([[float(m.get("theta", 0)), float(m.get("phi", 0)), float(m.get("pole", 0))]])


@pytest.mark.parametrize("name", CASES)
def test_plan_matches_reference(emfa_lib, name):
    from emfa_gb300 import api
    g = load_golden(name)
    lev, lb, poles, perm = api.mlfma_plan(M.TriMesh(g["verts"], g["tris"]), g["rwg"], params(g))
    assert np.array_equal(lb, g["level_boxes"])
    assert np.array_equal(poles, g["poles"])
    assert np.array_equal(perm, g["perm"])


def test_plan_errors(emfa_lib):
    from emfa_gb300 import api, _lib
    g = load_golden("sphere3_mlfma")
    with pytest.raises(_lib.EmfaError):  # a box threshold above the object: fewer than 2 levels
        api.mlfma_plan(M.TriMesh(g["verts"], g["tris"]), g["rwg"], api.mlfma_params(3e8, 0.5, 10.0))


@pytest.fixture(scope="module")
def ops(ctx):
    from emfa_gb300 import api
    out = {}
    for name in CASES:
        g = load_golden(name)
        geo = api.Geometry(ctx, M.TriMesh(g["verts"], g["tris"]), g["rwg"])
        out[name] = (g, geo, api.Mlfma(geo, params(g)))
    yield out
    for g, geo, ml in out.values():
        ml.close()
        geo.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_operator_matches_reference(ops, name):
    import torch
    g, geo, ml = ops[name]
    # the reference's sparse matrix drops entries that are exactly zero
    assert int(g["near_nnz"]) <= ml.nnz <= int(g["near_nnz"]) + 8
    x = torch.tensor(g["mv_x"], device="cuda")
    near = ml.apply_part(x, 1).cpu().numpy()
    err_near = np.linalg.norm(near - g["mv_near"]) / np.linalg.norm(g["mv_near"])
    assert err_near < 1e-5, err_near
    y = ml.apply(x[None])[0].cpu().numpy()
    err = np.linalg.norm(y - g["mv_y"]) / np.linalg.norm(g["mv_y"])
    assert err < 2e-4, err
    far_ref = g["mv_y"] - g["mv_near"]
    far = ml.apply_part(x, 2).cpu().numpy()
    assert np.linalg.norm(far - far_ref) / np.linalg.norm(far_ref) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("nr", [3, 8, 10])
def test_multi_rhs_apply_equals_single(ops, nr):
    """Several right-hand sides in one operator pass (up to 8 per pass; 10
    = 8 + 2) give each vector's single-RHS product exactly: per right-hand
    side the kernels sum in the same order."""
    import torch
    g, geo, ml = ops[CASES[0]]
    rng = np.random.default_rng(nr)
    X = torch.tensor((rng.standard_normal((nr, geo.n)) + 1j * rng.standard_normal((nr, geo.n))).astype(np.complex64),
                     device="cuda")
    Y = ml.apply(X).cpu().numpy()
    for r in range(nr):
        y1 = ml.apply(X[r:r + 1].contiguous())[0].cpu().numpy()
        assert np.array_equal(Y[r], y1), (r, np.abs(Y[r] - y1).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_excitation_box_order(ops, name):
    g, geo, ml = ops[name]
    V = ml.fill_v(angles(g)).cpu().numpy()[0]
    assert np.abs(V - g["V"]).max() <= 2e-6 * np.abs(g["V"]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_solve_and_rcs(ops, name, method):
    import torch
    from emfa_gb300 import api
    g, geo, ml = ops[name]
    V = ml.fill_v(angles(g))
    X, info = ml.solve(V, api.solver_params(method, restart=30, tol=1e-3 if method == "bicgstab" else 1e-4,
                                            max_iter=300))
    assert info.converged == 1
    Ibox = X.cpu().numpy()[0]
    # against the reference's own BiCGStab current (box order, tolerance 1e-3)
    assert np.linalg.norm(Ibox - g["I"]) / np.linalg.norm(g["I"]) < 1e-2
    # against the dense CFIE solution (RWG order)
    Irwg = ml.unpermute(X).cpu().numpy()[0]
    fp = api.fill_params("cfie", "f64", float(g["meta"]["frequency"]),
                         float(np.float32(float(g["meta"]["alpha"]))))
    Z = api.fill_z(geo, fp)
    Vd = api.fill_v(geo, fp, angles(g))
    Xd, _ = api.solve(ml.ctx, Z, Vd, api.solver_params("gmres", tol=1e-10, max_iter=3000))
    Id = Xd.cpu().numpy()[0]
    # the reference's own MLFMA is this far from the dense CFIE solution on these
    # meshes (its multipole rule and clamped stencils at 0.13-0.25 lambda boxes)
    ref_err = np.linalg.norm(g["I"] - Id[g["perm"]]) / np.linalg.norm(Id)
    our_err = np.linalg.norm(Irwg - Id) / np.linalg.norm(Id)
    assert our_err <= 1.1 * ref_err + 2e-3, (our_err, ref_err)
    # RCS from the MLFMA current vs the reference's MLFMA RCS
    r = api.rcs(geo, api.fill_params("cfie", "f32", float(g["meta"]["frequency"]), 0.5),
                torch.tensor(Irwg[None], device="cuda"), g["rcs_dirs"].astype(np.float64))[0]
    assert np.abs(r - g["rcs"]).max() < 0.1


@pytest.fixture(scope="module")
def sai(ctx):
    from emfa_gb300 import api
    g = load_golden("sphere3_mlfma")
    geo = api.Geometry(ctx, M.TriMesh(g["verts"], g["tris"]), g["rwg"])
    m = g["meta"]
    mp = api.mlfma_params(float(m["frequency"]), float(np.float32(float(m["alpha"]))),
                          float(np.float32(float(m["mlfma_box_threshold"]))), precond=True)
    ml = api.Mlfma(geo, mp)
    yield g, geo, ml
    ml.close()
    geo.close()


@pytest.mark.gpu
def test_sai_lists_and_values_match_restatement(sai):
    """SAI preconditioner: the per-box lists hold each box's own unknowns
    contiguously at `own`, columns are a subset of rows, and the values of P
    (batched FP32 Householder QR on the device) match the numpy restatement
    of MLFMA::parallelPreconditioner on the same near-field matrix (the
    operator's near part, itself checked against the reference above) to
    1e-4 in Frobenius norm."""
    import torch
    from oracle import oracle as O
    g, geo, ml = sai
    n = geo.n
    rptr, rows, cptr, cols, own = ml.precond_lists()
    assert len(own) == len(rptr) - 1 and (own >= 0).all()
    for b in range(len(own)):
        r = set(rows[rptr[b]:rptr[b + 1]].tolist())
        assert set(cols[cptr[b]:cptr[b + 1]].tolist()) <= r
    # near-field matrix, column by column (box order)
    Zn = np.zeros((n, n), dtype=np.complex128)
    e = torch.zeros(n, dtype=torch.complex64, device="cuda")
    for j in range(n):
        e.zero_()
        e[j] = 1.0
        Zn[:, j] = ml.apply_part(e, 1).cpu().numpy()
    ptr, col, val = ml.precond_csr()
    P = np.zeros((n, n), dtype=np.complex128)
    for i in range(n):
        P[i, col[ptr[i]:ptr[i + 1]]] = val[ptr[i]:ptr[i + 1]]
    Po = O.sai_preconditioner(Zn, rptr, rows, cptr, cols, own)
    assert np.count_nonzero(P) == np.count_nonzero(Po)
    assert np.linalg.norm(P - Po) / np.linalg.norm(Po) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_sai_preconditioned_solve(ops, sai, method):
    """P Z x = P b (left preconditioning, as MLFMA::iterativeSolve): the same
    current as the unpreconditioned solve within the solver tolerance, in
    fewer iterations."""
    from emfa_gb300 import api
    g, geo, mlp = sai
    _, _, ml = ops["sphere3_mlfma"]
    sp = api.solver_params(method, restart=30, tol=1e-4, max_iter=600)
    V = ml.fill_v(angles(g))
    X0, i0 = ml.solve(V, sp)
    X1, i1 = mlp.solve(V, sp)
    assert i0.converged == 1 and i1.converged == 1
    a, b = X1.cpu().numpy()[0], X0.cpu().numpy()[0]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-3
    assert i1.iterations < i0.iterations, (i1.iterations, i0.iterations)


def test_plan_with_the_configuration_truncation(emfa_lib):
    """truncation "config" (int(kd + 1.8 d0^(2/3) kd^(1/3)), d0 = 3): the same
    tree and box order as the reference's rule, fewer multipoles per level,
    and exactly the formula's count given the reference's (both from the
    same kd = sqrt(3) k side, with side halving per level)."""
    from emfa_gb300 import api
    g = load_golden("sphere3_mlfma")
    mesh = M.TriMesh(g["verts"], g["tris"])
    p_ref = params(g)
    m = g["meta"]
    p_cfg = api.mlfma_params(float(m["frequency"]), float(np.float32(float(m["alpha"]))),
                             float(np.float32(float(m["mlfma_box_threshold"]))), truncation="config")
    lev_r, lb_r, poles_r, perm_r = api.mlfma_plan(mesh, g["rwg"], p_ref)
    lev_c, lb_c, poles_c, perm_c = api.mlfma_plan(mesh, g["rwg"], p_cfg)
    assert lev_r == lev_c and np.array_equal(lb_r, lb_c) and np.array_equal(perm_r, perm_c)
    assert np.all(poles_c < poles_r)
    # kd of the finest level from its reference count, then each coarser level doubles it
    for i in range(len(poles_r)):
        kd_lo = [x for x in np.linspace(0.1, 200, 400001) if int(x + 6 * np.cbrt(x)) == poles_r[i]]
        lo, hi = min(kd_lo), max(kd_lo)
        cands = {int(x + 1.8 * np.cbrt(9.0) * np.cbrt(x)) for x in np.linspace(lo, hi, 200)}
        assert poles_c[i] in cands, (i, poles_c[i], cands)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_operator_with_the_configuration_truncation(ops, name):
    """The operator with the configuration's multipole truncation against
    the dense CFIE product of the same mesh: on these small meshes (finest
    boxes of 0.16-0.2 wavelength) the reference's own MLFMA formulation is
    already 4-9 % off the dense product (its Gauss-Legendre phi samples and
    clamped stencils); the configuration's rule, with fewer multipoles,
    adds at most a quarter to that error."""
    import torch
    from emfa_gb300 import api
    g, geo, ml = ops[name]
    m = g["meta"]
    f, a = float(m["frequency"]), float(np.float32(float(m["alpha"])))
    mlc = api.Mlfma(geo, api.mlfma_params(f, a, float(np.float32(float(m["mlfma_box_threshold"]))),
                                          truncation="config"))
    assert np.all(mlc.poles < ml.poles)
    Z = api.fill_z(geo, api.fill_params("cfie", "f64", f, a))
    x = torch.tensor(g["mv_x"], device="cuda")[None]
    errs = []
    for op in (ml, mlc):
        y = op.unpermute(op.apply(x).to(torch.complex128))[0]
        yd = Z @ op.unpermute(x.to(torch.complex128))[0]
        errs.append(float(torch.linalg.norm(y - yd) / torch.linalg.norm(yd)))
    mlc.close()
    assert errs[1] <= 1.25 * errs[0], errs
