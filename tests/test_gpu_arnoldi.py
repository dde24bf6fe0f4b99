"""The fused Arnoldi step (k_arnoldi_step: a cluster of CTAs per right-hand
side; Gram-Schmidt coefficients summed through distributed shared memory;
update, normalisation and FP16 packing in the same launch) against the same
CGS1 step as separate passes (orth "cgs1_split").

The two forms sum the coefficients in different orders (FP32 within a warp,
FP64 across warps, CTAs and blocks in both), so their iterates agree to
rounding.  Tolerances: both meet the target (true residual 1e-6), iteration
counts within one step, solutions within 1e-5 of each other (relative L2; the
test matrices have condition numbers near 2).

Shapes cover every cluster form: one CTA per right-hand side (N <= 1024),
clusters of 2, 3 and 8, one to four elements per thread, the largest N the
fused step takes (16384) and one past it (the separate passes again).  The
right-hand-side counts keep the grids small enough for the fused step
(n_rhs x CTAs per right-hand side <= 4 x the SM count); the last test checks
the choice by grid size.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(n, nrhs, seed):
    """Z = 2 I + 0.7 G / sqrt(n) (G complex normal: eigenvalues in a disk of
    radius ~0.7 about 2, ~20 GMRES steps to 1e-6), random right-hand sides
    of different scales, and one zero right-hand side (inactive from the
    start)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    Z = torch.randn(n, n, dtype=torch.complex64, device="cuda", generator=g) * (0.7 / np.sqrt(n))
    Z.diagonal().add_(2.0)
    B = torch.randn(nrhs, n, dtype=torch.complex64, device="cuda", generator=g)
    B *= torch.logspace(-3, 3, nrhs, device="cuda").to(torch.complex64)[:, None]
    B[nrhs // 2] = 0
    return Z, B


def _solve(ctx, Z, B, orth, matvec, restart=30, basis="f32"):
    from emfa_gb300 import api
    sp = api.solver_params("gmres", restart=restart, tol=1e-6, max_iter=2000, matvec=matvec, orth=orth, basis=basis)
    X, info = api.solve(ctx, Z, B, sp)
    return X, info


def _true_residual(Z, B, X):
    import torch
    R = B.to(torch.complex128) - X @ Z.to(torch.complex128).T
    nb = torch.linalg.norm(B.to(torch.complex128), dim=1)
    nr = torch.linalg.norm(R, dim=1)
    return torch.where(nb > 0, nr / torch.where(nb > 0, nb, 1), nr).cpu().numpy()


@pytest.mark.parametrize("n,nrhs,matvec", [
    (300, 40, "f16x"),     # one CTA per right-hand side, one element per thread
    (1500, 24, "f16x"),    # clusters of 2
    (2500, 12, "f32"),     # clusters of 3, unpacked operator (FP32 CUDA-core product)
    (7680, 16, "f16x"),    # clusters of 8, two elements per thread
    (7680, 6, "tf32"),
    (12000, 6, "f16x"),    # four elements per thread
    (16384, 4, "f16x"),    # the largest N of the fused step
    (16385, 3, "f16x"),    # separate passes
])
def test_fused_step_matches_separate_passes(ctx, n, nrhs, matvec):
    import torch
    Z, B = _system(n, nrhs, seed=n)
    Xf, inf_f = _solve(ctx, Z, B, "cgs1", matvec)
    Xs, inf_s = _solve(ctx, Z, B, "cgs1_split", matvec)
    assert inf_f.converged == nrhs and inf_s.converged == nrhs
    assert abs(inf_f.iterations - inf_s.iterations) <= 1, (inf_f.iterations, inf_s.iterations)
    assert inf_f.iterations >= 10  # the step ran many times, across several basis lengths
    rf, rs = _true_residual(Z, B, Xf), _true_residual(Z, B, Xs)
    assert rf.max() < 1e-6 and rs.max() < 1e-6, (rf.max(), rs.max())
    zero = nrhs // 2
    assert torch.count_nonzero(Xf[zero]) == 0
    d = torch.linalg.norm(Xf - Xs, dim=1) / torch.linalg.norm(Xs, dim=1).clamp_min(1e-300)
    d[zero] = 0
    assert d.max().item() < 1e-5, d.max().item()


def test_fused_step_restart_boundaries(ctx):
    """Restart lengths 1, 2, 7 and 32 (the longest the fused step takes; 33
    goes back to the separate passes): the last step of a cycle and the
    restart from the true residual."""
    Z, B = _system(4096, 8, seed=7)
    for m in (1, 2, 7, 32, 33):
        Xf, inf_f = _solve(ctx, Z, B, "cgs1", "f16x", restart=m)
        Xs, inf_s = _solve(ctx, Z, B, "cgs1_split", "f16x", restart=m)
        assert inf_f.converged == 8 and inf_s.converged == 8, m
        assert abs(inf_f.iterations - inf_s.iterations) <= max(1, inf_s.iterations // 20), (m, inf_f.iterations,
                                                                                             inf_s.iterations)
        rf = _true_residual(Z, B, Xf)
        assert rf.max() < 1e-6, (m, rf.max())


def test_fused_step_reproducible(ctx):
    """Fixed-order sums: the same solve twice gives the same bits."""
    import torch
    Z, B = _system(7680, 10, seed=3)
    X1, i1 = _solve(ctx, Z, B, "cgs1", "f16x")
    X2, i2 = _solve(ctx, Z, B, "cgs1", "f16x")
    assert i1.iterations == i2.iterations
    assert torch.equal(X1, X2)


def _launches(ctx, Z, B, orth, basis="f32"):
    before = ctx.launches()
    X, info = _solve(ctx, Z, B, orth, "f16x", basis=basis)
    return ctx.launches() - before, info


def test_auto_choice_by_grid_size(ctx):
    """Tens of right-hand sides take the fused step (one launch a step);
    hundreds at N = 7680 (clusters of 8: more than four CTAs an SM) take the
    separate passes (coefficients, update, column, normalisation: four)."""
    from emfa_gb300 import api
    Z, B = _system(7680, 400, seed=11)
    few = B[:16].contiguous()
    # the first product of a shape times the tile-shape candidates (more
    # launches): tune both shapes before counting
    api.matvec(ctx, Z, few, "f16x")
    api.matvec(ctx, Z, B, "f16x")
    n_auto, i_auto = _launches(ctx, Z, few, "cgs1")
    n_split, i_split = _launches(ctx, Z, few, "cgs1_split")
    assert i_auto.iterations == i_split.iterations
    # at least two launches fewer per Arnoldi step (three kernels become one)
    assert n_split - n_auto >= 2 * i_split.iterations, (n_auto, n_split, i_split.iterations)
    n_auto, i_auto = _launches(ctx, Z, B, "cgs1")
    n_split, i_split = _launches(ctx, Z, B, "cgs1_split")
    assert i_auto.iterations == i_split.iterations and n_auto == n_split
    # orth "cgs1_fused" takes the fused step at any grid size, same solution
    n_fused, i_fused = _launches(ctx, Z, B, "cgs1_fused")
    assert abs(i_fused.iterations - i_split.iterations) <= 1 and n_split - n_fused >= 2 * i_fused.iterations


# ---------------------------------------------------------------------------
# FP16 basis (basis "f16", the default where the separate passes feed the
# split-FP16 product): the basis vectors are the product's own FP16 operand
# rows, each scaled by a power of two.  Against the FP32 basis: the same
# target met (true residual 1e-6), iteration counts within 10 % (at least 2),
# solutions within 1e-5 of each other.
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n,nrhs,restart", [
    (300, 40, 30),     # one Gram-Schmidt chunk, one finish chunk
    (1500, 24, 30),    # a ragged last chunk (1500 = 1024 + 476)
    (4096, 8, 1),      # restart lengths 1, 2, 7, 32 and 33 (the longest the
    (4096, 8, 2),      #   FP32-step path of the finish pass takes is 32;
    (4096, 8, 7),      #   33 runs the unfused finish on the FP32 basis)
    (4096, 8, 32),
    (4096, 8, 33),
    (7680, 360, 30),   # the dense CFIE job's shape
    (16385, 3, 30),    # N past the fused step
    (1501, 24, 30),    # odd N: 8-byte W accesses, a half pair at the end
    (7681, 40, 30),    #   of every row; a ragged last chunk of the finish
    (4097, 8, 7),
])
def test_fp16_basis_matches_fp32_basis(ctx, n, nrhs, restart):
    import torch
    Z, B = _system(n, nrhs, seed=n + restart)
    Xh, ih = _solve(ctx, Z, B, "cgs1_split", "f16x", restart=restart, basis="f16")
    Xs, i_s = _solve(ctx, Z, B, "cgs1_split", "f16x", restart=restart, basis="f32")
    assert ih.converged == nrhs and i_s.converged == nrhs
    assert abs(ih.iterations - i_s.iterations) <= max(2, i_s.iterations // 10), (ih.iterations, i_s.iterations)
    rh = _true_residual(Z, B, Xh)
    assert rh.max() < 1e-6, rh.max()
    zero = nrhs // 2
    assert torch.count_nonzero(Xh[zero]) == 0
    d = torch.linalg.norm(Xh - Xs, dim=1) / torch.linalg.norm(Xs, dim=1).clamp_min(1e-300)
    d[zero] = 0
    assert d.max().item() < 1e-5, d.max().item()


def test_fp16_basis_reproducible_and_launches(ctx):
    """Fixed-order sums on the FP16 basis: the same solve twice gives the same
    bits, with as many launches as on the FP32 basis (the first basis vector
    is packed into the basis instead of the product's own buffer)."""
    import torch
    Z, B = _system(7680, 200, seed=5)
    _solve(ctx, Z, B, "cgs1_split", "f16x", basis="f16")  # tunes the product's tile shape
    n1, i1 = _launches(ctx, Z, B, "cgs1_split", basis="f16")
    X1, _ = _solve(ctx, Z, B, "cgs1_split", "f16x", basis="f16")
    X2, i2 = _solve(ctx, Z, B, "cgs1_split", "f16x", basis="f16")
    assert i1.iterations == i2.iterations and torch.equal(X1, X2)
    n32, i32 = _launches(ctx, Z, B, "cgs1_split", basis="f32")
    if i32.iterations == i1.iterations and i32.cycles == i1.cycles:
        assert n1 == n32, (n1, n32)


@pytest.mark.parametrize("matvec,orth", [("f32", "cgs1_split"), ("tf32", "cgs1_split"), ("f16x", "cgs1"),
                                         ("f16x", "cgs2")])
def test_fp16_basis_only_where_the_product_packs(ctx, matvec, orth):
    """basis "f16" changes nothing where it does not apply: unpacked products,
    the fused step (few right-hand sides) and two Gram-Schmidt passes keep the
    FP32 basis, bit for bit."""
    import torch
    Z, B = _system(3000, 6, seed=9)
    X16, i16 = _solve(ctx, Z, B, orth, matvec, basis="f16")
    X32, i32 = _solve(ctx, Z, B, orth, matvec, basis="f32")
    assert i16.iterations == i32.iterations and torch.equal(X16, X32)


@pytest.mark.parametrize("n", [4000, 4001])
def test_auto_basis_is_fp16_for_either_parity(ctx, n):
    """basis "auto" takes the FP16 basis for even and odd N (odd N: 8-byte
    accesses of W's rows and a half pair at the end): bit-identical to
    basis "f16"."""
    import torch
    Z, B = _system(n, 200, seed=n)
    Xa, ia = _solve(ctx, Z, B, "cgs1_split", "f16x", basis="auto")
    Xp, ip = _solve(ctx, Z, B, "cgs1_split", "f16x", basis="f16")
    assert ia.iterations == ip.iterations and torch.equal(Xa, Xp)
