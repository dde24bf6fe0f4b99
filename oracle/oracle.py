"""ctypes front end of the oracle -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module, and only as the checker.  It wraps:

* ``oracle/_build/libemfa_oracle.so`` -- the C restatement of the reference's
  fill / excitation / RCS / RWG routines (``emfa_oracle.c``,
  ``oracle_common.c``), float and double instances;
* ``oracle/_ref/emfa_ref_f32|f64`` -- the reference itself compiled from its
  own sources (``build_ref.sh``), when it was built on this machine.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libemfa_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build() -> None:
    subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True,
                   stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _rt(prec):
    return (np.float32, ctypes.c_float, "or32_") if prec == 32 else (np.float64, ctypes.c_double, "or64_")


class Geometry:
    """Mesh + RWG table in the oracle's precision."""

    def __init__(self, verts, tris, rwg, prec=32):
        dt, _, _ = _rt(prec)
        self.prec = prec
        self.verts = np.ascontiguousarray(verts, dtype=dt)
        self.tris = np.ascontiguousarray(tris, dtype=np.int32)
        self.rwg = np.ascontiguousarray(rwg, dtype=np.int32)
        self.len = _edge_len(self.verts, self.rwg, dt)
        self.n = int(self.rwg.shape[0])


def _edge_len(v, rwg, dt):
    # CommonEdge::buildCommonEdge: (vertex1 - vertex2).Norm(), x*x + y*y + z*z in order
    d = (v[rwg[:, 0]] - v[rwg[:, 1]]).astype(dt)
    s = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(dt) + d[:, 2] * d[:, 2]
    return np.sqrt(s.astype(dt)).astype(dt)


def build_rwg(tris) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    nt = tris.shape[0]
    out = np.zeros((3 * nt // 2 + 8, 6), dtype=np.int32)
    f = lib().or_build_rwg
    f.restype = ctypes.c_int
    n = f(_p(tris), ctypes.c_int(nt), _p(out), ctypes.c_int(out.shape[0]))
    if n < 0:
        raise RuntimeError("or_build_rwg: capacity")
    return out[:n].copy()


def wavenumber(freq, prec=32):
    """k = PI2 * f / cc in the reference's precision (EFIE.cpp:47)."""
    dt = np.float32 if prec == 32 else np.float64
    pi = dt(np.pi)
    pi2 = dt(2.0) * pi
    return dt(dt(pi2 * dt(freq)) / dt(299792458.0))


def incidence(theta, phi, pole, prec=32):
    dt, ct, pf = _rt(prec)
    out = np.zeros(9, dtype=dt)
    getattr(lib(), pf + "incidence")(ct(theta), ct(phi), ct(pole), _p(out))
    return out


def fill_z_efie(g: Geometry, k, threshold_edm=1e30, sigma=(0.0, 0.0), edm_mode=0):
    dt, ct, pf = _rt(g.prec)
    Z = np.zeros((g.n, g.n, 2), dtype=dt)
    getattr(lib(), pf + "fill_z_efie")(_p(g.verts), _p(g.tris), _p(g.rwg), _p(g.len), ctypes.c_int(g.n),
                                       ct(k), ct(threshold_edm), ct(sigma[0]), ct(sigma[1]),
                                       ctypes.c_int(edm_mode), _p(Z))
    return Z[..., 0] + 1j * Z[..., 1]


def fill_z_cfie(g: Geometry, k, alpha):
    dt, ct, pf = _rt(g.prec)
    Z = np.zeros((g.n, g.n, 2), dtype=dt)
    getattr(lib(), pf + "fill_z_cfie")(_p(g.verts), _p(g.tris), _p(g.rwg), _p(g.len), ctypes.c_int(g.n),
                                       ct(k), ct(alpha), _p(Z))
    return Z[..., 0] + 1j * Z[..., 1]


def fill_z_efie_cfg(g: Geometry, k, sigma=(0.0, 0.0)):
    """EFIE in the configurations' discretisation (not the reference's): 7 x
    7-point regular pairs, singularity extraction on self and edge-adjacent
    pairs (emfa_oracle.c, fill_z_efie_cfg)."""
    dt, ct, pf = _rt(g.prec)
    Z = np.zeros((g.n, g.n, 2), dtype=dt)
    getattr(lib(), pf + "fill_z_efie_cfg")(_p(g.verts), _p(g.tris), _p(g.rwg), _p(g.len), ctypes.c_int(g.n), ct(k),
                                           ct(sigma[0]), ct(sigma[1]), _p(Z))
    return Z[..., 0] + 1j * Z[..., 1]


def potential_integrals(tri, r, prec=64):
    """(int_T 1/R dS', int_T (rho' - rho)/R dS') for triangle tri (3 x 3) and
    observation point r, by the closed forms the configuration fill uses."""
    dt, _, pf = _rt(prec)
    t = np.ascontiguousarray(tri, dtype=dt).reshape(9)
    rr = np.ascontiguousarray(r, dtype=dt).reshape(3)
    i1 = np.zeros(1, dtype=dt)
    ir = np.zeros(3, dtype=dt)
    getattr(lib(), pf + "potential_integrals")(_p(t), _p(rr), _p(i1), _p(ir))
    return float(i1[0]), ir.astype(np.float64)


def fill_v(g: Geometry, k, inc, cfie=False, alpha=1.0):
    dt, ct, pf = _rt(g.prec)
    inc = np.ascontiguousarray(np.atleast_2d(inc), dtype=dt)
    V = np.zeros((inc.shape[0], g.n, 2), dtype=dt)
    getattr(lib(), pf + "fill_v")(_p(g.verts), _p(g.tris), _p(g.rwg), _p(g.len), ctypes.c_int(g.n),
                                  ct(k), ctypes.c_int(1 if cfie else 0), ct(alpha), _p(inc),
                                  ctypes.c_int(inc.shape[0]), _p(V))
    return V[..., 0] + 1j * V[..., 1]


def rcs(g: Geometry, k, I, dirs):
    dt, ct, pf = _rt(g.prec)
    I = np.atleast_2d(I)
    Ib = np.ascontiguousarray(np.stack([I.real, I.imag], -1), dtype=dt)
    dirs = np.ascontiguousarray(dirs, dtype=dt)
    out = np.zeros((I.shape[0], dirs.shape[0]), dtype=dt)
    getattr(lib(), pf + "rcs")(_p(g.verts), _p(g.tris), _p(g.rwg), _p(g.len), ctypes.c_int(g.n), ct(k),
                               _p(Ib), ctypes.c_int(I.shape[0]), _p(dirs), ctypes.c_int(dirs.shape[0]),
                               _p(out))
    return out


def tri_geometry(verts, tris, prec=32):
    dt, _, pf = _rt(prec)
    verts = np.ascontiguousarray(verts, dtype=dt)
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    nt = tris.shape[0]
    nrm = np.zeros((nt, 3), dtype=dt)
    q3 = np.zeros((nt, 3, 3), dtype=dt)
    q7 = np.zeros((nt, 7, 3), dtype=dt)
    area = np.zeros(nt, dtype=dt)
    getattr(lib(), pf + "tri_geometry")(_p(verts), _p(tris), ctypes.c_int(nt), _p(nrm), _p(q3), _p(q7), _p(area))
    return nrm, q3, q7, area


# ---------------------------------------------------------------------------
# the reference binary (oracle/_ref), when built here
# ---------------------------------------------------------------------------
def ref_binary(prec=32):
    p = os.path.join(REF_DIR, "emfa_ref_f32" if prec == 32 else "emfa_ref_f64")
    return p if os.path.exists(p) else None


def run_reference(mode, config_path, outdir, arg, prec=32, cwd=None, timeout=3600):
    """Run the reference harness; it writes binary dumps into outdir.  The
    reference's mesh loader writes ./temp.dat, so it runs in a scratch cwd."""
    exe = ref_binary(prec)
    if exe is None:
        raise FileNotFoundError("reference binary not built (oracle/build_ref.sh)")
    cwd = cwd or tempfile.mkdtemp(prefix="emfa_ref_")
    r = subprocess.run([exe, mode, os.path.abspath(config_path), os.path.abspath(outdir), str(arg)],
                       cwd=cwd, stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    return r.stdout


def run_reference_args(mode, config_path, outdir, args, prec=32, timeout=7200):
    """Run a harness mode that takes several trailing arguments (``big``,
    ``rcs_of``), in a scratch cwd like run_reference."""
    exe = ref_binary(prec)
    if exe is None:
        raise FileNotFoundError("reference binary not built (oracle/build_ref.sh)")
    cwd = tempfile.mkdtemp(prefix="emfa_ref_")
    r = subprocess.run([exe, mode, os.path.abspath(config_path), os.path.abspath(outdir)] + [str(a) for a in args],
                       cwd=cwd, stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    return r.stdout


def closed_form_vector(n, a=7919, b=104729, prec=32):
    """The seeded test vector of the harness's MLFMA mode with seed 0:
    x_i = ((i a) mod 2001 - 1000) / 1000 + j ((i b) mod 2003 - 1001) / 1001,
    each part one correctly rounded division, so numpy and the reference's
    C++ give the same bits."""
    dt = np.float32 if prec == 32 else np.float64
    i = np.arange(n, dtype=np.int64)
    re = ((i * a) % 2001 - 1000).astype(dt) / dt(1000)
    im = ((i * b) % 2003 - 1001).astype(dt) / dt(1001)
    return (re + 1j * im).astype(np.complex64 if prec == 32 else np.complex128)


def time_reference(config_path, kind, rows, solve=0, prec=32, timeout=3600):
    exe = ref_binary(prec)
    cwd = tempfile.mkdtemp(prefix="emfa_ref_")
    r = subprocess.run([exe, "time", os.path.abspath(config_path), kind, str(rows), str(solve)],
                       cwd=cwd, stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference timing failed: %s" % r.stderr[-2000:])
    line = [l[l.index('{"n"'):] for l in r.stdout.splitlines() if '{"n"' in l][-1]
    return json.loads(line)


def load_dump(outdir, prec=32):
    """Read a harness dump directory into numpy arrays."""
    dt = np.float32 if prec == 32 else np.float64
    cdt = np.complex64 if prec == 32 else np.complex128
    d = {}
    meta = np.fromfile(os.path.join(outdir, "meta.bin"), np.int32)
    nv, nt, n = (int(x) for x in meta)
    d["n"] = n
    d["verts"] = np.fromfile(os.path.join(outdir, "verts.bin"), dt).reshape(nv, 3)
    d["tris"] = np.fromfile(os.path.join(outdir, "tris.bin"), np.int32).reshape(nt, 3)
    d["normals"] = np.fromfile(os.path.join(outdir, "normals.bin"), dt).reshape(nt, 3)
    d["rwg"] = np.fromfile(os.path.join(outdir, "rwg.bin"), np.int32).reshape(n, 6)
    d["len"] = np.fromfile(os.path.join(outdir, "rwg_len.bin"), dt)
    d["inc"] = np.fromfile(os.path.join(outdir, "inc.bin"), dt) if os.path.exists(
        os.path.join(outdir, "inc.bin")) else None
    for name in ("Z", "Z_arma", "V", "I", "mv_x", "mv_y", "mv_near"):
        p = os.path.join(outdir, name + ".bin")
        if os.path.exists(p):
            a = np.fromfile(p, cdt)
            d[name] = a.reshape(n, n) if name.startswith("Z") else a
    for name, t in (("rcs", dt), ("rcs_dirs", dt), ("perm", np.int32), ("iters", np.int32),
                    ("poles", np.int32), ("level_boxes", np.int32), ("box_len", dt)):
        p = os.path.join(outdir, name + ".bin")
        if os.path.exists(p):
            d[name] = np.fromfile(p, t)
    if "rcs_dirs" in d:
        d["rcs_dirs"] = d["rcs_dirs"].reshape(-1, 3)
    p = os.path.join(outdir, "near_rc.bin")
    if os.path.exists(p):
        d["near_rc"] = np.fromfile(p, np.int32).reshape(-1, 2)
        d["near_val"] = np.fromfile(os.path.join(outdir, "near_val.bin"), cdt)
    return d


def sai_preconditioner(Znear, rptr, rows, cptr, cols, own):
    """Restatement of MLFMA::parallelPreconditioner (EMSolver/MLFMA.cpp:1346-1391),
    in complex128 with numpy's QR.  Per finest box b: A = Znear(rows_b, cols_b),
    A = Q R (economy), and P(cols_b, unknowns of b) = R^-1 Q(own rows, :)^H
    (Armadillo's .t() of a complex matrix is the conjugate transpose).  Znear
    is the box-order near-field matrix (zero off the near pattern, as the
    reference's sparse nearZ_); the box lists are the ones of
    MLFMA::preparepreconditioner (MLFMA.cpp:1320-1344).  Returns dense P."""
    n = Znear.shape[0]
    nbox = len(own)
    offs = [int(rows[rptr[b] + own[b]]) for b in range(nbox)]
    cnts = [(offs[b + 1] if b + 1 < nbox else n) - offs[b] for b in range(nbox)]
    P = np.zeros((n, n), dtype=np.complex128)
    for b in range(nbox):
        r = rows[rptr[b]:rptr[b + 1]]
        c = cols[cptr[b]:cptr[b + 1]]
        A = Znear[np.ix_(r, c)].astype(np.complex128)
        Q, R = np.linalg.qr(A)
        sel = Q[own[b]:own[b] + cnts[b], :]
        P[np.ix_(c, np.arange(offs[b], offs[b] + cnts[b]))] = np.linalg.solve(R, sel.conj().T)
    return P
