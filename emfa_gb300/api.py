"""Python front end over the C ABI (emfa_gb300._lib).

Device memory comes from torch tensors (plumbing only: every computation
runs in libemfa_cuda.so kernels).  Complex arrays are torch complex64 /
complex128 tensors, RHS-major: shape (n_rhs, N).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib as L
from .mesh import TriMesh

vp = ctypes.c_void_p


def _ptr(t):
    """Device pointer of a tensor the C ABI reads as a dense row-major array."""
    if not t.is_contiguous():
        raise ValueError("emfa: tensor arguments must be contiguous (got strides %s)" % (tuple(t.stride()),))
    return vp(t.data_ptr())


def build_rwg(tris: np.ndarray) -> np.ndarray:
    """RWG table (N x 6: v1 v2 vxp vxm tp tm), host only."""
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    cap = 3 * tris.shape[0] // 2 + 16
    out = np.zeros((cap, 6), dtype=np.int32)
    n = ctypes.c_int(0)
    L.check(L.lib().emfa_build_rwg(tris.ctypes.data_as(vp), tris.shape[0], out.ctypes.data_as(vp), cap,
                                   ctypes.byref(n)))
    return out[: n.value].copy()


def fill_params(kind="cfie", precision="f32", freq=3e8, alpha=0.5, sigma=(0.0, 0.0), edm_mode=0,
                discretisation="reference") -> L.FillParams:
    """discretisation: "reference" (3 x 3 points, self-pair extraction, as
    the reference) or "config" (7 x 7 points, self and edge-adjacent pair
    extraction; EFIE)."""
    return L.FillParams(L.EMFA_CFIE if kind == "cfie" else L.EMFA_EFIE,
                        L.EMFA_F64 if precision == "f64" else L.EMFA_F32,
                        float(freq), float(alpha), float(sigma[0]), float(sigma[1]), int(edm_mode),
                        {"reference": 0, "config": 1}[discretisation])


def solver_params(method="gmres", restart=30, max_iter=600, tol=1e-6, tol_absolute=False, matvec="auto",
                  max_refine=0, orth="auto", inner_reduction=0.0, basis="auto") -> L.SolverParams:
    mv = {"auto": 0, "f64": 1, "f32": 2, "tf32": 3, "f16x": 4}[matvec]
    og = {"auto": 0, "cgs1": 1, "cgs2": 2, "cgs1_split": 3, "cgs1_fused": 4}[orth]
    bs = {"auto": 0, "f32": 1, "f16": 2}[basis]
    meth = {"gmres": L.EMFA_GMRES, "bicgstab": L.EMFA_BICGSTAB, "lu": L.EMFA_LU}[method]
    return L.SolverParams(meth, int(restart), int(max_iter), float(tol), int(bool(tol_absolute)), mv, int(max_refine),
                          og, float(inner_reduction), bs)


class Context:
    def __init__(self, device=0, hbm_budget=0):
        self.h = vp()
        L.check(L.lib().emfa_ctx_create(device, hbm_budget, ctypes.byref(self.h)))
        self.device = device

    def close(self):
        """Releases the caller's hold on the context; geometries and MLFMA
        operators still open on it keep its stream until they are closed."""
        self._ext = None
        if self.h:
            L.lib().emfa_ctx_destroy(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status):
        return L.check(status, self.h)

    def memory(self):
        u, p, b = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        self.check(L.lib().emfa_ctx_memory(self.h, ctypes.byref(u), ctypes.byref(p), ctypes.byref(b)))
        return u.value, p.value, b.value

    def launches(self) -> int:
        c = ctypes.c_int64()
        self.check(L.lib().emfa_ctx_launch_count(self.h, ctypes.byref(c)))
        return c.value

    def synchronize(self):
        self.check(L.lib().emfa_ctx_synchronize(self.h))

    def stream_ptr(self) -> int:
        s = vp()
        self.check(L.lib().emfa_ctx_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def join_torch(self):
        """Makes torch's current stream wait for the work queued so far on
        the context's stream (no host wait), so torch reads of a result
        written there see it."""
        torch = _torch()
        if getattr(self, "_ext", None) is None:
            self._ext = torch.cuda.ExternalStream(self.stream_ptr(), device="cuda:%d" % self.device)
        torch.cuda.current_stream().wait_stream(self._ext)

    KERNEL_TIMERS = {"fill_z": 0, "gemm": 1, "residual": 2}

    def kernel_timing(self, on: bool):
        """Turns per-kernel event timing on or off (and clears its records)."""
        self.check(L.lib().emfa_ctx_set_kernel_timing(self.h, 1 if on else 0))

    def kernel_time(self, kernel: str):
        """(launches, summed device ms, summed algorithmic work) of one timed
        kernel since timing was turned on; work is FLOPs for the products and
        Z entries for the fill."""
        n, ms, w = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        self.check(L.lib().emfa_ctx_kernel_time(self.h, self.KERNEL_TIMERS[kernel], ctypes.byref(n), ctypes.byref(ms),
                                                ctypes.byref(w)))
        return n.value, ms.value, w.value


class Geometry:
    def __init__(self, ctx: Context, mesh: TriMesh, rwg: np.ndarray | None = None):
        self.ctx = ctx
        self.verts = np.ascontiguousarray(mesh.verts, dtype=np.float64)
        self.tris = np.ascontiguousarray(mesh.tris, dtype=np.int32)
        self.rwg = build_rwg(self.tris) if rwg is None else np.ascontiguousarray(rwg, dtype=np.int32)
        self.n = int(self.rwg.shape[0])
        self.h = vp()
        ctx.check(L.lib().emfa_geom_create(ctx.h, self.verts.ctypes.data_as(vp), self.verts.shape[0],
                                           self.tris.ctypes.data_as(vp), self.tris.shape[0],
                                           self.rwg.ctypes.data_as(vp), self.n, ctypes.byref(self.h)))

    def close(self):
        if self.h:
            L.lib().emfa_geom_destroy(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _torch():
    import torch
    return torch


def fill_z(geom: Geometry, fp: L.FillParams, out=None):
    torch = _torch()
    dt = torch.complex128 if fp.precision == L.EMFA_F64 else torch.complex64
    n = geom.n
    Z = out if out is not None else torch.empty((n, n), dtype=dt, device="cuda:%d" % geom.ctx.device)
    torch.cuda.current_stream().synchronize()
    geom.ctx.check(L.lib().emfa_fill_z(geom.ctx.h, geom.h, ctypes.byref(fp), _ptr(Z), Z.stride(0), None))
    geom.ctx.join_torch()
    return Z


def fill_v(geom: Geometry, fp: L.FillParams, angles, out=None):
    """angles: (n_inc, 3) theta, phi, pole in degrees."""
    torch = _torch()
    a = np.ascontiguousarray(np.atleast_2d(angles), dtype=np.float64)
    dt = torch.complex128 if fp.precision == L.EMFA_F64 else torch.complex64
    V = out if out is not None else torch.empty((a.shape[0], geom.n), dtype=dt, device="cuda:%d" % geom.ctx.device)
    torch.cuda.current_stream().synchronize()  # an `out` written on torch's stream
    geom.ctx.check(L.lib().emfa_fill_v(geom.ctx.h, geom.h, ctypes.byref(fp), a.ctypes.data_as(vp), a.shape[0],
                                       _ptr(V), None))
    geom.ctx.join_torch()
    return V


def matvec(ctx: Context, Z, X, matvec="auto"):
    torch = _torch()
    prec = L.EMFA_F64 if Z.dtype == torch.complex128 else L.EMFA_F32
    mv = {"auto": 0, "f64": 1, "f32": 2, "tf32": 3, "f16x": 4}[matvec]
    Y = torch.empty_like(X)
    torch.cuda.current_stream().synchronize()  # inputs written on torch's stream
    ctx.check(L.lib().emfa_matvec(ctx.h, prec, mv, _ptr(Z), Z.shape[0], _ptr(X), X.shape[0], _ptr(Y), None))
    ctx.synchronize()  # the product runs on the context's stream
    return Y


TILE_SHAPES = ("64x128", "64x256", "144x128", "144x256")


def autotune_query(device: int, n: int, n_rhs: int):
    """The inner product's tuned tile shape for (n, n_rhs) on a device:
    (shape name or None if not tuned yet, {shape: best ms} of the timed
    candidates)."""
    v = ctypes.c_int()
    ms = (ctypes.c_float * 4)()
    L.check(L.lib().emfa_autotune_query(device, n, n_rhs, ctypes.byref(v), ms))
    times = {TILE_SHAPES[i]: ms[i] for i in range(4) if ms[i] >= 0}
    return (TILE_SHAPES[v.value] if v.value >= 0 else None), times


def autotune_clear():
    L.check(L.lib().emfa_autotune_clear())


def residual(ctx: Context, Z, X, B, matvec="auto"):
    """R = B - Z X (complex128) with the refinement residual of a matvec mode;
    X complex128, B in Z's precision."""
    torch = _torch()
    prec = L.EMFA_F64 if Z.dtype == torch.complex128 else L.EMFA_F32
    mv = {"auto": 0, "f64": 1, "f32": 2, "tf32": 3, "f16x": 4}[matvec]
    R = torch.empty(X.shape, dtype=torch.complex128, device=X.device)
    torch.cuda.current_stream().synchronize()
    ctx.check(L.lib().emfa_residual(ctx.h, prec, mv, _ptr(Z), Z.shape[0], _ptr(X), _ptr(B), X.shape[0], _ptr(R), None))
    ctx.synchronize()
    return R


def solve(ctx: Context, Z, B, sp: L.SolverParams):
    """Returns (X complex128 (n_rhs, N), SolveInfo); raises on errors other
    than non-convergence (reported in info.converged)."""
    torch = _torch()
    prec = L.EMFA_F64 if Z.dtype == torch.complex128 else L.EMFA_F32
    X = torch.empty(B.shape, dtype=torch.complex128, device=B.device)
    torch.cuda.current_stream().synchronize()
    info = L.SolveInfo()
    st = L.lib().emfa_solve(ctx.h, prec, _ptr(Z), Z.shape[0], _ptr(B), B.shape[0], _ptr(X), ctypes.byref(sp),
                            ctypes.byref(info), None)
    if st not in (L.EMFA_OK, 4):
        ctx.check(st)
    return X, info


def rcs(geom: Geometry, fp: L.FillParams, I, dirs, per_rhs=False) -> np.ndarray:
    _torch().cuda.current_stream().synchronize()
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    n_rhs = I.shape[0]
    n_dir = d.shape[-2] if d.ndim == 3 else d.shape[0]
    out = np.zeros((n_rhs, n_dir), dtype=np.float64)
    geom.ctx.check(L.lib().emfa_rcs(geom.ctx.h, geom.h, ctypes.byref(fp), _ptr(I), n_rhs, d.ctypes.data_as(vp),
                                    n_dir, int(per_rhs), out.ctypes.data_as(vp), None))
    return out


def dense_rcs(ctx: Context, mesh: TriMesh, fp: L.FillParams, angles, sp: L.SolverParams, dirs, per_rhs=False,
              want_current=False):
    """End-to-end job from host buffers (emfa_dense_rcs)."""
    a = np.ascontiguousarray(np.atleast_2d(angles), dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    n_dir = d.shape[-2] if d.ndim == 3 else d.shape[0]
    verts = np.ascontiguousarray(mesh.verts, dtype=np.float64)
    tris = np.ascontiguousarray(mesh.tris, dtype=np.int32)
    out = np.zeros((a.shape[0], n_dir), dtype=np.float64)
    cur = np.zeros((a.shape[0], 3 * tris.shape[0] // 2 * 2), dtype=np.float64) if want_current else None
    info = L.SolveInfo()
    st = L.lib().emfa_dense_rcs(ctx.h, verts.ctypes.data_as(vp), verts.shape[0], tris.ctypes.data_as(vp),
                                tris.shape[0], ctypes.byref(fp), a.ctypes.data_as(vp), a.shape[0], ctypes.byref(sp),
                                d.ctypes.data_as(vp), n_dir, int(per_rhs), out.ctypes.data_as(vp),
                                cur.ctypes.data_as(vp) if cur is not None else None, ctypes.byref(info))
    if st not in (L.EMFA_OK, 4):
        ctx.check(st)
    I = None
    if cur is not None:
        n = 3 * tris.shape[0] // 2
        I = cur[:, : 2 * n].reshape(a.shape[0], n, 2)
        I = I[..., 0] + 1j * I[..., 1]
    return out, info, I


def bistatic_dirs(theta_from=0.0, theta_to=180.0, theta_delta=1.0, phi=0.0, ring=True) -> np.ndarray:
    """Directions of Result::getBistaticRCS (EMComponent/Result.h:59-98) in
    float arithmetic: the phi cut over theta, then the theta = 90 ring."""
    # angles in float; sin/cos in double through libm (math.*: numpy's
    # vectorised sin/cos are not libm's) as the reference's
    # unqualified calls bind to); cos(phi), sin(phi) stored as float; each
    # component rounded once to float
    f = np.float32
    d2r = f(np.pi) / f(180.0)
    ph = f(phi) * d2r
    cp, sp_ = f(math.cos(float(ph))), f(math.sin(float(ph)))
    out = []
    td = f(theta_from)
    while td <= f(theta_to):
        th = float(td * d2r)
        out.append((f(math.sin(th) * float(cp)), f(math.sin(th) * float(sp_)), f(math.cos(th))))
        td = f(td + f(theta_delta))
    if ring:
        pd = f(0.0)
        while pd < f(360.0):
            p = float(pd * d2r)
            out.append((f(math.cos(p)), f(math.sin(p)), f(0.0)))
            pd = f(pd + f(1.0))
    return np.array(out, dtype=np.float64)


def monostatic_dirs(angles) -> np.ndarray:
    """Backscatter direction (-k_inc) of each incidence (theta, phi) in degrees:
    r_hat(theta, phi), shape (n_inc, 1, 3)."""
    a = np.atleast_2d(np.asarray(angles, dtype=np.float64))
    th, ph = np.deg2rad(a[:, 0]), np.deg2rad(a[:, 1])
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1)
    return d[:, None, :]


# ---------------------------------------------------------------------------
# MLFMA
# ---------------------------------------------------------------------------
def mlfma_params(freq=3e8, alpha=0.5, box_threshold=0.25, precond=False, row_threshold=0.9,
                 col_threshold=0.87, truncation="reference") -> L.MlfmaParams:
    """truncation: "reference" (int(kd + 6 kd^(1/3)), as the reference) or
    "config" (int(kd + 1.8 d0^(2/3) kd^(1/3)), d0 = 3)."""
    return L.MlfmaParams(float(freq), float(alpha), float(box_threshold), int(bool(precond)), float(row_threshold),
                         float(col_threshold), {"reference": 0, "config": 1}[truncation])


def mlfma_plan(mesh: TriMesh, rwg: np.ndarray, mp: L.MlfmaParams):
    """Host-only octree plan: (levels, boxes per level, poles per level, perm)."""
    verts = np.ascontiguousarray(mesh.verts, dtype=np.float64)
    rwg = np.ascontiguousarray(rwg, dtype=np.int32)
    lev = ctypes.c_int()
    lb = np.zeros(64, dtype=np.int32)
    poles = np.zeros(64, dtype=np.int32)
    perm = np.zeros(rwg.shape[0], dtype=np.int32)
    L.check(L.lib().emfa_mlfma_plan(verts.ctypes.data_as(vp), verts.shape[0], rwg.ctypes.data_as(vp), rwg.shape[0],
                                    ctypes.byref(mp), ctypes.byref(lev), lb.ctypes.data_as(vp), 64,
                                    poles.ctypes.data_as(vp), perm.ctypes.data_as(vp)))
    return lev.value, lb[: lev.value + 1].copy(), poles[: lev.value - 1].copy(), perm


class Mlfma:
    def __init__(self, geom: Geometry, mp: L.MlfmaParams):
        self.geom = geom
        self.ctx = geom.ctx
        self.h = vp()
        self.ctx.check(L.lib().emfa_mlfma_create(self.ctx.h, geom.h, ctypes.byref(mp), ctypes.byref(self.h)))
        lev = ctypes.c_int()
        nnz = ctypes.c_size_t()
        self.perm = np.zeros(geom.n, dtype=np.int32)
        lb = np.zeros(64, dtype=np.int32)
        poles = np.zeros(64, dtype=np.int32)
        self.ctx.check(L.lib().emfa_mlfma_info(self.h, ctypes.byref(lev), lb.ctypes.data_as(vp),
                                               poles.ctypes.data_as(vp), ctypes.byref(nnz),
                                               self.perm.ctypes.data_as(vp)))
        self.levels = lev.value
        self.level_boxes = lb[: lev.value + 1].copy()
        self.poles = poles[: lev.value - 1].copy()
        self.nnz = nnz.value

    def close(self):
        if self.h:
            L.lib().emfa_mlfma_destroy(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply(self, X):
        torch = _torch()
        X = X.reshape(-1, self.geom.n).contiguous()
        Y = torch.empty_like(X)
        torch.cuda.current_stream().synchronize()
        self.ctx.check(L.lib().emfa_mlfma_apply(self.h, _ptr(X), _ptr(Y), X.shape[0], None))
        self.ctx.synchronize()
        return Y

    def apply_part(self, x, part):
        """part 0: near + far, 1: near only, 2: far only (one vector)."""
        torch = _torch()
        x = x.reshape(self.geom.n).contiguous()
        y = torch.empty_like(x)
        torch.cuda.current_stream().synchronize()
        self.ctx.check(L.lib().emfa_mlfma_apply_part(self.h, _ptr(x), _ptr(y), int(part), None))
        self.ctx.synchronize()
        return y

    def fill_v(self, angles):
        torch = _torch()
        a = np.ascontiguousarray(np.atleast_2d(angles), dtype=np.float64)
        V = torch.empty((a.shape[0], self.geom.n), dtype=torch.complex64, device="cuda:%d" % self.ctx.device)
        torch.cuda.current_stream().synchronize()
        self.ctx.check(L.lib().emfa_mlfma_fill_v(self.h, a.ctypes.data_as(vp), a.shape[0], _ptr(V), None))
        self.ctx.join_torch()
        return V

    def solve(self, B, sp: L.SolverParams):
        torch = _torch()
        X = torch.empty(B.shape, dtype=torch.complex128, device=B.device)
        info = L.SolveInfo()
        torch.cuda.current_stream().synchronize()
        st = L.lib().emfa_mlfma_solve(self.h, _ptr(B), B.shape[0], _ptr(X), ctypes.byref(sp), ctypes.byref(info),
                                      None)
        if st not in (L.EMFA_OK, 4):
            self.ctx.check(st)
        return X, info

    def unpermute(self, Xbox):
        torch = _torch()
        X = torch.empty_like(Xbox)
        self.ctx.check(L.lib().emfa_mlfma_unpermute(self.h, _ptr(Xbox), Xbox.shape[0], _ptr(X), None))
        return X

    def precond_csr(self):
        """SAI preconditioner as (ptr, col, val complex64) over box-order rows, or None."""
        nnz = ctypes.c_size_t()
        self.ctx.check(L.lib().emfa_mlfma_precond_csr(self.h, ctypes.byref(nnz), None, None, None))
        if nnz.value == 0:
            return None
        ptr = np.zeros(self.geom.n + 1, dtype=np.int32)
        col = np.zeros(nnz.value, dtype=np.int32)
        val = np.zeros(nnz.value, dtype=np.complex64)
        self.ctx.check(L.lib().emfa_mlfma_precond_csr(self.h, ctypes.byref(nnz), ptr.ctypes.data_as(vp),
                                                      col.ctypes.data_as(vp), val.ctypes.data_as(vp)))
        return ptr, col, val

    def precond_lists(self):
        """Per-box SAI lists: (rptr, rows, cptr, cols, own)."""
        nb, nr, nc = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
        f = L.lib().emfa_mlfma_precond_lists
        self.ctx.check(f(self.h, ctypes.byref(nb), ctypes.byref(nr), ctypes.byref(nc), None, None, None, None, None))
        rptr = np.zeros(nb.value + 1, dtype=np.int32)
        rows = np.zeros(nr.value, dtype=np.int32)
        cptr = np.zeros(nb.value + 1, dtype=np.int32)
        cols = np.zeros(nc.value, dtype=np.int32)
        own = np.zeros(nb.value, dtype=np.int32)
        self.ctx.check(f(self.h, ctypes.byref(nb), ctypes.byref(nr), ctypes.byref(nc), rptr.ctypes.data_as(vp),
                         rows.ctypes.data_as(vp), cptr.ctypes.data_as(vp), cols.ctypes.data_as(vp),
                         own.ctypes.data_as(vp)))
        return rptr, rows, cptr, cols, own


# ---------------------------------------------------------------------------
# batched and served solves (emfa_serve)
# ---------------------------------------------------------------------------
class RcsRequest:
    """One RCS problem for serve(): a host mesh, a formulation, incidences
    and RCS directions (per_rhs: one set of directions per incidence, e.g.
    the monostatic one)."""

    def __init__(self, mesh: TriMesh, freq: float, angles, dirs, kind="cfie", alpha=0.5, method="auto",
                 per_rhs=False, tol=0.0, max_iter=0, box_threshold=0.25, arrival_s=0.0):
        self.mesh = mesh
        self.verts = np.ascontiguousarray(mesh.verts, dtype=np.float64)
        self.tris = np.ascontiguousarray(mesh.tris, dtype=np.int32)
        self.angles = np.ascontiguousarray(np.atleast_2d(angles), dtype=np.float64)
        self.dirs = np.ascontiguousarray(dirs, dtype=np.float64)
        self.n_dir = self.dirs.shape[-2] if self.dirs.ndim == 3 else self.dirs.shape[0]
        self.rcs = np.zeros((self.angles.shape[0], self.n_dir), dtype=np.float64)
        self.kind = L.EMFA_CFIE if kind == "cfie" else L.EMFA_EFIE
        self.method = {"auto": 0, "dense": 1, "mlfma": 2}[method]
        self.freq, self.alpha, self.per_rhs = float(freq), float(alpha), bool(per_rhs)
        self.tol, self.max_iter, self.box_threshold = float(tol), int(max_iter), float(box_threshold)
        self.arrival_s = float(arrival_s)

    def c_struct(self) -> L.Request:
        return L.Request(self.verts.ctypes.data, self.verts.shape[0], self.tris.ctypes.data, self.tris.shape[0],
                         self.kind, self.method, self.freq, self.alpha, self.angles.ctypes.data, self.angles.shape[0],
                         self.dirs.ctypes.data, self.n_dir, int(self.per_rhs), self.tol, self.max_iter,
                         self.box_threshold, self.arrival_s, self.rcs.ctypes.data)


def serve(requests, device=0, lanes=0, hbm_budget=0, dense_max=0, realtime=False, max_wait_s=0.0):
    """Runs the requests through emfa_serve; each request's rcs array is
    filled in place.  Returns the per-request results (status, method,
    unknowns, iterations, timing in seconds from the start)."""
    n = len(requests)
    arr = (L.Request * n)(*[r.c_struct() for r in requests])
    res = (L.RequestResult * n)()
    opts = L.ServeOpts(int(lanes), int(hbm_budget), int(dense_max), int(bool(realtime)), float(max_wait_s))
    L.check(L.lib().emfa_serve(int(device), arr, n, ctypes.byref(opts), res))
    return list(res)


def serve_simulate(arrival, duration, nbytes, lanes=6, hbm_budget=0, realtime=True, max_wait_s=0.0):
    """The admitter of serve() on a simulated clock: (start times, lanes)."""
    a = np.ascontiguousarray(arrival, dtype=np.float64)
    d = np.ascontiguousarray(duration, dtype=np.float64)
    b = np.ascontiguousarray(nbytes, dtype=np.uint64)
    n = a.shape[0]
    start = np.zeros(n, dtype=np.float64)
    lane = np.zeros(n, dtype=np.int32)
    opts = L.ServeOpts(int(lanes), int(hbm_budget), 0, int(bool(realtime)), float(max_wait_s))
    L.check(L.lib().emfa_serve_simulate(a.ctypes.data_as(vp), d.ctypes.data_as(vp), b.ctypes.data_as(vp), n,
                                        ctypes.byref(opts), start.ctypes.data_as(vp), lane.ctypes.data_as(vp)))
    return start, lane


# ---------------------------------------------------------------------------
# binary dumps
# ---------------------------------------------------------------------------
_DUMP_DTYPES = {np.dtype(np.complex64): 1, np.dtype(np.complex128): 2, np.dtype(np.float32): 3,
                np.dtype(np.float64): 4, np.dtype(np.int32): 5}
_DUMP_NP = {v: k for k, v in _DUMP_DTYPES.items()}


def dump_save(path: str, array, name: str = "", freq: float = 0.0):
    """Writes a 1-D or 2-D array (numpy, or a CUDA torch tensor) as an EMFA dump."""
    on_dev = not isinstance(array, np.ndarray)
    if on_dev:
        torch = _torch()
        dt = np.dtype({torch.complex64: np.complex64, torch.complex128: np.complex128, torch.float32: np.float32,
                       torch.float64: np.float64, torch.int32: np.int32}[array.dtype])
        shape = tuple(array.shape)
        ptr = _ptr(array)
    else:
        array = np.ascontiguousarray(array)
        dt, shape, ptr = array.dtype, array.shape, array.ctypes.data_as(vp)
    rows, cols = (shape[0], int(np.prod(shape[1:]))) if len(shape) > 1 else (1, shape[0])
    L.check(L.lib().emfa_dump_save(path.encode(), name.encode(), _DUMP_DTYPES[dt], rows, cols, float(freq), ptr,
                                   int(on_dev)))


def dump_info(path: str):
    name = ctypes.create_string_buffer(24)
    dt, rows, cols, freq = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_double()
    L.check(L.lib().emfa_dump_info(path.encode(), name, ctypes.byref(dt), ctypes.byref(rows), ctypes.byref(cols),
                                   ctypes.byref(freq)))
    return {"name": name.value.decode(), "dtype": _DUMP_NP[dt.value], "rows": rows.value, "cols": cols.value,
            "freq": freq.value}


def dump_load(path: str, device=None):
    """Reads a dump into a numpy array, or into a CUDA tensor when device is given."""
    info = dump_info(path)
    shape = (info["rows"], info["cols"]) if info["rows"] > 1 else (info["cols"],)
    if device is None:
        out = np.empty(shape, dtype=info["dtype"])
        L.check(L.lib().emfa_dump_load(path.encode(), out.ctypes.data_as(vp), out.nbytes, 0))
        return out, info
    torch = _torch()
    tdt = {np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128,
           np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
           np.dtype(np.int32): torch.int32}[info["dtype"]]
    out = torch.empty(shape, dtype=tdt, device=device)
    torch.cuda.current_stream().synchronize()
    L.check(L.lib().emfa_dump_load(path.encode(), _ptr(out), out.numel() * out.element_size(), 1))
    return out, info
