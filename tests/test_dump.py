"""Binary dump format (emfa_dump_save / info / load): round trips of every
dtype, header fields, and the failures a reader must catch (corrupted
payload, wrong magic, unknown version, short destination)."""
import os
import struct
import tempfile

import numpy as np
import pytest


@pytest.mark.parametrize("dt", [np.complex64, np.complex128, np.float32, np.float64, np.int32])
def test_round_trip_host(emfa_lib, dt):
    from emfa_gb300 import api
    rng = np.random.default_rng(0)
    a = (rng.standard_normal((37, 11)) * 100).astype(dt) if dt != np.complex64 and dt != np.complex128 else \
        (rng.standard_normal((37, 11)) + 1j * rng.standard_normal((37, 11))).astype(dt)
    p = os.path.join(tempfile.mkdtemp(), "a.emfa")
    api.dump_save(p, a, name="Z", freq=3e8)
    info = api.dump_info(p)
    assert info["name"] == "Z" and info["rows"] == 37 and info["cols"] == 11 and info["freq"] == 3e8
    assert info["dtype"] == np.dtype(dt)
    b, _ = api.dump_load(p)
    assert b.dtype == a.dtype and np.array_equal(a, b)
    assert os.path.getsize(p) == 128 + a.nbytes


def test_vector_and_header_layout(emfa_lib):
    from emfa_gb300 import api
    v = np.arange(5, dtype=np.complex128)
    p = os.path.join(tempfile.mkdtemp(), "v.emfa")
    api.dump_save(p, v, name="I")
    raw = open(p, "rb").read()
    assert raw[:8] == b"EMFADUMP"
    version, dtype, rows, cols = struct.unpack_from("<IIQQ", raw, 8)
    assert (version, dtype, rows, cols) == (1, 2, 1, 5)
    b, _ = api.dump_load(p)
    assert np.array_equal(b, v)


def test_corruption_and_errors_are_caught(emfa_lib):
    from emfa_gb300 import api, _lib
    a = np.ones((4, 4), dtype=np.complex64)
    d = tempfile.mkdtemp()
    p = os.path.join(d, "a.emfa")
    api.dump_save(p, a)
    raw = bytearray(open(p, "rb").read())
    bad = os.path.join(d, "bad.emfa")
    raw2 = bytearray(raw)
    raw2[128 + 5] ^= 0xFF  # one payload byte flipped
    open(bad, "wb").write(raw2)
    with pytest.raises(_lib.EmfaError, match="hash mismatch"):
        api.dump_load(bad)
    raw3 = bytearray(raw)
    raw3[0:8] = b"NOTADUMP"
    open(bad, "wb").write(raw3)
    with pytest.raises(_lib.EmfaError):
        api.dump_info(bad)
    raw4 = bytearray(raw)
    raw4[8:12] = struct.pack("<I", 99)
    open(bad, "wb").write(raw4)
    with pytest.raises(_lib.EmfaError):
        api.dump_info(bad)
    open(bad, "wb").write(raw[:100])
    with pytest.raises(_lib.EmfaError):
        api.dump_info(bad)
    small = np.empty(3, dtype=np.complex64)
    st = _lib.lib().emfa_dump_load(p.encode(), small.ctypes.data, small.nbytes, 0)
    assert st == 1


@pytest.mark.gpu
def test_round_trip_device(ctx):
    import torch
    from emfa_gb300 import api
    g = torch.Generator(device="cuda").manual_seed(2)
    Z = torch.randn((300, 300), dtype=torch.complex64, device="cuda", generator=g)
    p = os.path.join(tempfile.mkdtemp(), "z.emfa")
    api.dump_save(p, Z, name="Z", freq=1e8)
    Z2, info = api.dump_load(p, device="cuda")
    assert torch.equal(Z, Z2) and info["name"] == "Z"
    h, _ = api.dump_load(p)
    assert np.array_equal(h, Z.cpu().numpy())
