"""emfa_matvec_tf32_noalloc: the tensor-core product on static scratch, with
no device allocation inside the call.  Checked through the C ABI against the
context entry point emfa_matvec(EMFA_F32, EMFA_MV_TF32) on the same inputs,
two calls in a row (the second must not see the first one's scratch), plus
the argument checks.  Collected last on purpose: it must pass both in a fresh
process and after every other test has used the library.

Tolerance: both entry points run the same kernels, so results agree to 1e-6
(relative L2); against an FP64 product the TF32 bound of the GEMM tests
(3e-3) applies."""
import ctypes

import numpy as np
import pytest

# (2048, 512) is n * n_rhs exactly at EMFA_NOALLOC_MAX_ELEMS
SIZES = [(998, 37), (1920, 360), (256, 1), (2048, 512)]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(n, nrhs, seed):
    import torch
    rng = np.random.default_rng(seed)
    Z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    X = (rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))).astype(np.complex64)
    return Z, X, torch.from_numpy(Z).cuda(), torch.from_numpy(X).cuda()


def _noalloc(L, Zd, Xd, n, nrhs):
    import torch
    Y = torch.full((nrhs, n), float("nan"), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    st = L.emfa_matvec_tf32_noalloc(_ptr(Zd), n, _ptr(Xd), nrhs, _ptr(Y), None)
    assert st == 0, L.emfa_last_error(None)
    return Y.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("n,nrhs", SIZES)
def test_noalloc_matches_context_entry_point(emfa_lib, ctx, n, nrhs):
    from emfa_gb300 import api
    L = emfa_lib
    for call, seed in enumerate((11, 12)):  # two calls in a row, different inputs
        Z, X, Zd, Xd = _inputs(n, nrhs, seed + n)
        y_new = _noalloc(L, Zd, Xd, n, nrhs)
        y_ctx = api.matvec(ctx, Zd, Xd, "tf32").cpu().numpy()
        assert np.isfinite(y_new).all(), call
        assert _rel(y_new, y_ctx) < 1e-6, (call, _rel(y_new, y_ctx))
        y64 = X.astype(np.complex128) @ Z.astype(np.complex128).T
        assert _rel(y_new, y64) < 3e-3, (call, _rel(y_new, y64))


@pytest.mark.gpu
def test_noalloc_call_reserves_no_device_memory(emfa_lib, ctx):
    """After a first call on the device (which may make the driver load this
    part of the library and reserve its static array), further calls change
    neither the device's free memory nor torch's allocator counters."""
    import torch
    L = emfa_lib
    n, nrhs = 1920, 360
    _, _, Zd, Xd = _inputs(n, nrhs, 5)
    Y = torch.empty((nrhs, n), dtype=torch.complex64, device="cuda")
    assert L.emfa_matvec_tf32_noalloc(_ptr(Zd), n, _ptr(Xd), nrhs, _ptr(Y), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        assert L.emfa_matvec_tf32_noalloc(_ptr(Zd), n, _ptr(Xd), nrhs, _ptr(Y), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0, (free0, free1)
    for key in ("allocation.all.allocated", "segment.all.allocated", "reserved_bytes.all.current"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key


@pytest.mark.gpu
def test_noalloc_rejects_oversized_and_odd(emfa_lib, ctx):
    import torch
    L = emfa_lib
    Zd = torch.zeros((2, 2), dtype=torch.complex64, device="cuda")
    Xd = torch.zeros((1, 2), dtype=torch.complex64, device="cuda")
    Y = torch.zeros((1, 2), dtype=torch.complex64, device="cuda")
    cap = 1048576
    # n * n_rhs one past the static scratch: refused before any device work
    st = L.emfa_matvec_tf32_noalloc(_ptr(Zd), 2, _ptr(Xd), cap // 2 + 1, _ptr(Y), None)
    assert st == 1
    assert b"exceeds the static scratch limit" in L.emfa_last_error(None)
    st = L.emfa_matvec_tf32_noalloc(_ptr(Zd), 3, _ptr(Xd), 1, _ptr(Y), None)
    assert st == 6  # EMFA_ERR_UNSUPPORTED: odd order
    st = L.emfa_matvec_tf32_noalloc(None, 2, _ptr(Xd), 1, _ptr(Y), None)
    assert st == 1
