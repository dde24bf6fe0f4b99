"""Tile-shape autotuner of the split-FP16 inner product (emfa_autotune_*).

The first product of a shape bucket times every candidate tile shape and
keeps the fastest; later products of the bucket launch that shape.  Every
shape accumulates each output over K in the same order, so the product's
bits do not depend on the choice: the tests compare the tuned products with
those of the fixed rule (EMFA_AUTOTUNE=0, in a child process) bit for bit.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SHAPES = [(1500, 40), (640, 3), (7680, 360)]


def _operands(n, r, seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    Z = torch.randn(n, n, dtype=torch.complex64, device="cuda", generator=g)
    X = torch.randn(r, n, dtype=torch.complex64, device="cuda", generator=g)
    return Z, X


def test_autotune_choice_is_the_fastest_candidate_and_is_kept(ctx):
    import torch
    from emfa_gb300 import api
    api.autotune_clear()
    n, r = SHAPES[0]
    assert api.autotune_query(0, n, r) == (None, {})
    Z, X = _operands(n, r, 1)
    Y1 = api.matvec(ctx, Z, X, "f16x")
    shape, times = api.autotune_query(0, n, r)
    assert shape in api.TILE_SHAPES
    assert set(times) == set(api.TILE_SHAPES)  # 80 columns of B, N > 128: all four
    assert times[shape] == min(times.values()) > 0
    l0 = ctx.launches()
    Y2 = api.matvec(ctx, Z, X, "f16x")
    assert ctx.launches() - l0 == 4  # Z's max and split, packing, one product: no second tuning
    assert torch.equal(Y1, Y2)
    # a neighbour in the same bucket takes the recorded shape
    assert api.autotune_query(0, n - 100, r)[0] == shape
    # few right-hand sides: only the 64-column shapes are candidates
    Zs, Xs = _operands(640, 3, 2)
    api.matvec(ctx, Zs, Xs, "f16x")
    s2, t2 = api.autotune_query(0, 640, 3)
    assert set(t2) == {"64x128", "64x256"} and s2 in t2
    # accuracy of the tuned product against FP64: the split-FP16 product's
    # bar (11-bit significands on both sides, the normwise error of a TF32
    # product)
    ref = (Z.cpu().numpy().astype(np.complex128) @ X.cpu().numpy().astype(np.complex128).T).T
    err = np.linalg.norm(Y2.cpu().numpy() - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 2e-3, err.max()


def test_tuned_products_equal_the_fixed_rule_bitwise(ctx, tmp_path):
    import torch
    from emfa_gb300 import api
    api.autotune_clear()
    code = textwrap.dedent("""
        import sys, os
        sys.path.insert(0, %r)
        import numpy as np, torch
        sys.path.insert(0, os.path.join(%r, "tests"))
        from test_gpu_autotune import _operands, SHAPES
        from emfa_gb300 import api
        ctx = api.Context(0)
        for i, (n, r) in enumerate(SHAPES):
            Z, X = _operands(n, r, 10 + i)
            Y = api.matvec(ctx, Z, X, "f16x")
            np.save(os.path.join(%r, "y%%d.npy" %% i), Y.cpu().numpy())
            assert api.autotune_query(0, n, r)[0] is None  # the tuner is off
        ctx.close()
        print("ok")
    """ % (ROOT, ROOT, str(tmp_path)))
    env = dict(os.environ, EMFA_AUTOTUNE="0")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0 and p.stdout.strip().endswith("ok"), p.stderr[-3000:]
    for i, (n, r) in enumerate(SHAPES):
        Z, X = _operands(n, r, 10 + i)
        api.matvec(ctx, Z, X, "f16x")  # tunes the bucket
        Y = api.matvec(ctx, Z, X, "f16x").cpu().numpy()  # the chosen shape
        fixed = np.load(str(tmp_path / ("y%d.npy" % i)))
        assert np.array_equal(Y, fixed), (n, r, api.autotune_query(0, n, r))
