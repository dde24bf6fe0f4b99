"""Host-side logic that needs no GPU: the C ABI library loads and exports
every declared symbol, the RWG builder reproduces the reference's order and
orientation, argument errors come back as status codes, mesh generators and
the reference text formats round-trip."""
import os
import tempfile

import numpy as np
import pytest

from conftest import load_golden
from emfa_gb300 import mesh as M


def test_library_exports_every_header_symbol(emfa_lib):
    from emfa_gb300 import _lib
    syms = _lib.header_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(emfa_lib, s), s
    assert b"sm_103a" in emfa_lib.emfa_version()


@pytest.mark.parametrize("name", ["sphere1_efie", "cube2_efie_edm", "ellipsoid3_cfie", "sphere2_cfie"])
def test_rwg_builder_matches_reference_fixture(emfa_lib, name):
    from emfa_gb300 import api
    g = load_golden(name)
    assert np.array_equal(api.build_rwg(g["tris"]), g["rwg"])


@pytest.mark.parametrize("factory", [lambda: M.icosphere(3, 1.0), lambda: M.cube(5, 2.0),
                                     lambda: M.ellipsoid(6, (1.0, 0.6, 0.4))])
def test_rwg_builder_matches_oracle(emfa_lib, oracle_mod, factory):
    from emfa_gb300 import api
    m = factory()
    r = api.build_rwg(m.tris)
    assert r.shape[0] == m.n_rwg_closed()
    assert np.array_equal(r, oracle_mod.build_rwg(m.tris))


def test_rwg_builder_open_mesh(emfa_lib, oracle_mod):
    """Boundary edges are dropped, as CommonEdge::buildCommonEdge does."""
    from emfa_gb300 import api
    m = M.icosphere(2, 1.0)
    keep = m.verts[m.tris].mean(1)[:, 2] > 0.1  # cap: an open surface
    tris = m.tris[keep]
    r = api.build_rwg(tris)
    assert 0 < r.shape[0] < 3 * tris.shape[0] // 2
    assert np.array_equal(r, oracle_mod.build_rwg(tris))
    # every RWG's triangles hold its edge, + triangle traverses (v1, v2)
    for v1, v2, vp, vm, tp, tm in r:
        assert {v1, v2, vp} == set(tris[tp]) and {v1, v2, vm} == set(tris[tm])


@pytest.mark.parametrize("case", ["duplicated", "flipped", "both", "shuffled_both"])
def test_rwg_builder_non_manifold_matches_oracle(emfa_lib, oracle_mod, case):
    """Meshes where a directed edge is open in several triangles at once
    (duplicated triangles) or never closes (flipped triangles): every open
    half-edge that a later triangle's reversed edge matches is closed by it,
    as the reference's scan does."""
    from emfa_gb300 import api
    rng = np.random.default_rng(len(case))
    tris = M.icosphere(2, 1.0).tris.copy()
    if case in ("duplicated", "both", "shuffled_both"):
        tris = np.concatenate([tris, tris[rng.choice(len(tris), 12, replace=False)]])
    if case in ("flipped", "both", "shuffled_both"):
        idx = rng.choice(len(tris), 9, replace=False)
        tris[idx] = tris[idx][:, ::-1]
    if case == "shuffled_both":
        tris = tris[rng.permutation(len(tris))]
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    r = api.build_rwg(tris)
    assert r.shape[0] > 0
    assert np.array_equal(r, oracle_mod.build_rwg(tris))


def test_rwg_builder_errors(emfa_lib):
    import ctypes
    tris = np.array([[0, 1, 1]], dtype=np.int32)
    out = np.zeros((4, 6), dtype=np.int32)
    n = ctypes.c_int()
    st = emfa_lib.emfa_build_rwg(tris.ctypes.data_as(ctypes.c_void_p), 1, out.ctypes.data_as(ctypes.c_void_p), 4,
                                 ctypes.byref(n))
    assert st == 5  # EMFA_ERR_MESH: degenerate triangle
    assert b"degenerate" in emfa_lib.emfa_last_error(None)
    st = emfa_lib.emfa_build_rwg(None, 0, None, 0, ctypes.byref(n))
    assert st == 1  # EMFA_ERR_INVALID
    m = M.icosphere(1, 1.0)
    t = np.ascontiguousarray(m.tris)
    st = emfa_lib.emfa_build_rwg(t.ctypes.data_as(ctypes.c_void_p), t.shape[0], out.ctypes.data_as(ctypes.c_void_p), 4,
                                 ctypes.byref(n))
    assert st == 1 and n.value == 120  # capacity too small reports the needed count


def test_ctx_create_without_gpu_reports_cuda_error(emfa_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import ctypes
    h = ctypes.c_void_p()
    st = emfa_lib.emfa_ctx_create(0, 0, ctypes.byref(h))
    assert st == 2 and not h.value  # EMFA_ERR_CUDA, no context


def test_mesh_generators_closed_and_outward():
    for m in (M.icosphere(2, 1.0), M.cube(3, 1.0), M.ellipsoid(4, (1, 2, 3))):
        v, t = m.verts, m.tris
        n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
        assert np.all((n * v[t].mean(1)).sum(1) > 0)  # outward (centred at origin)
        # Euler characteristic of a sphere
        edges = {tuple(sorted(e)) for tri in t for e in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0]))}
        assert m.n_vert - len(edges) + m.n_tri == 2
        # 6-significant-digit grid (the reference's NAS round trip)
        assert np.array_equal(v, M.round6(v))
    assert M.icosphere(3, 0.5).n_tri == 1280 and M.icosphere(4, 1).n_tri == 5120


def test_nas_roundtrip_and_config():
    m = M.ellipsoid(3, (0.4, 0.3, 0.25))
    d = tempfile.mkdtemp()
    p = os.path.join(d, "e.nas")
    M.write_nas(m, p)
    r = M.read_nas(p)
    assert np.array_equal(r.verts, m.verts) and np.array_equal(r.tris, m.tris)
    cfg = M.write_config(os.path.join(d, "c.yml"), EMSolver="CFIE", alpha="0.3")
    txt = open(os.path.join(d, "c.yml")).read()
    assert "EMSolver: CFIE" in txt and cfg["alpha:"] == "0.3" and cfg["Sigma:"] == "(0,0)"
