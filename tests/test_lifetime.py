"""Handle lifetimes: a context, its geometries and MLFMA operators may be
closed in any order, or left to the interpreter's shutdown, where garbage
cycles run their finalizers in an order nobody controls.  The library keeps
a context (its stream and bookkeeping) alive while a geometry or operator
built on it exists, and a geometry while an operator uses it.

Each scenario runs in a child interpreter, so a heap error at exit (glibc
aborts the process) fails the test instead of the test session."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

PRELUDE = textwrap.dedent("""
    import sys
    sys.path.insert(0, %r)
    import numpy as np
    import torch
    from emfa_gb300 import api, mesh
    m = mesh.icosphere(2, 1.0)
""" % ROOT)

SCENARIOS = {
    # the context first, then the operator's geometry, then the operator
    "context_first": """
        ctx = api.Context(0)
        geo = api.Geometry(ctx, m)
        ml = api.Mlfma(geo, api.mlfma_params(3e8, 0.5, 0.25))
        Z = api.fill_z(geo, api.fill_params("cfie", "f32", 3e8, 0.5))
        ctx.close()
        geo.close()
        ml.close()
        print("ok")
    """,
    # a closed geometry stays usable by the operator built on it
    "geometry_before_operator": """
        ctx = api.Context(0)
        geo = api.Geometry(ctx, m)
        ml = api.Mlfma(geo, api.mlfma_params(3e8, 0.5, 0.25))
        x = ml.fill_v(np.array([[0.0, 0.0, 0.0]]))
        y0 = ml.apply(x)
        geo.close()
        y1 = ml.apply(x)
        assert torch.equal(y0, y1)
        ml.close()
        ctx.close()
        print("ok")
    """,
    # handles in a reference cycle, left to the shutdown
    "cycle_at_exit": """
        class Holder:
            pass
        h = Holder()
        h.ctx = api.Context(0)
        h.geo = api.Geometry(h.ctx, m)
        h.ml = api.Mlfma(h.geo, api.mlfma_params(3e8, 0.5, 0.25))
        h.self = h
        out, info, _ = api.dense_rcs(h.ctx, m, api.fill_params("cfie", "f32", 3e8, 0.5),
                                     np.array([[90.0, 0.0, 0.0]]), api.solver_params("gmres", tol=1e-6),
                                     api.monostatic_dirs(np.array([[90.0, 0.0, 0.0]])), per_rhs=True)
        del h
        print("ok")
    """,
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_close_order_and_shutdown(emfa_lib, name):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    code = PRELUDE + textwrap.dedent(SCENARIOS[name])
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr[-3000:])
    assert r.stdout.strip().endswith("ok"), r.stdout
    for bad in ("corrupted", "double free", "free():", "munmap_chunk", "Aborted"):
        assert bad not in r.stderr, r.stderr[-3000:]
