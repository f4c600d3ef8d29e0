"""The allocation-free compute_tend entry (GPU), collected last.

mpaso_sw_compute_tend_noalloc serves callers that may not allocate device
memory while they run (tasks inside a runtime that pools all device memory,
or code that cannot take cudaMalloc's device-wide synchronisation): it stages
through a static device array instead of allocated scratch.  It must give the
same result as mpaso_sw_compute_tend -- bit for bit, the tolerance of the
per-task tests -- on two calls in a row, so a second call cannot see stale
contents of the shared array."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_tend_matches_regular_entry_twice():
    torch = pytest.importorskip("torch")
    import mpaso
    import mpaso.gpu as G
    from mpaso._lib import check, lib

    mesh = mpaso.Mesh.icosa(4)
    dm = G.DeviceMesh(mesh, reorder=True)
    L = 2
    nC, nE = mesh.nCells, mesh.nEdges
    rng = np.random.default_rng(42)
    # the context's own device memory before any per-task call: the entry under
    # test runs first on this fresh context and must not grow it
    bytes0 = dm.device_bytes()
    for call in range(2):
        host = dict(he=900 + 100 * rng.random((nE, L)), h=1000 + 100 * rng.random((nC, L)),
                    u=10 * rng.standard_normal((nE, L)), ke=rng.random((nC, L)),
                    pve=1e-5 * rng.standard_normal((nE, L)))
        dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
        outs = [(torch.full((nC, L), np.nan, dtype=torch.float64, device="cuda"),
                 torch.full((nE, L), np.nan, dtype=torch.float64, device="cuda")) for _ in range(2)]
        torch.cuda.synchronize()
        args = [_ptr(dev[k]) for k in ("he", "h", "u", "ke", "pve")]
        check(lib().mpaso_sw_compute_tend_noalloc(dm.handle, L, *args, _ptr(outs[1][0]), _ptr(outs[1][1]),
                                                  None))
        if call == 0:
            assert dm.device_bytes() == bytes0, "the allocation-free entry grew the context's scratch"
        check(lib().mpaso_sw_compute_tend(dm.handle, L, *args, _ptr(outs[0][0]), _ptr(outs[0][1]), None))
        torch.cuda.synchronize()  # both entries ran on the context's stream: wait for the device
        ref_h, ref_u = outs[0][0].cpu().numpy(), outs[0][1].cpu().numpy()
        got_h, got_u = outs[1][0].cpu().numpy(), outs[1][1].cpu().numpy()
        assert np.isfinite(ref_h).all() and np.isfinite(ref_u).all()
        assert np.array_equal(got_h, ref_h), f"call {call}: tend_h differs"
        assert np.array_equal(got_u, ref_u), f"call {call}: tend_u differs"


def test_noalloc_rejects_oversized_mesh_and_host_pointers():
    torch = pytest.importorskip("torch")
    import mpaso
    import mpaso.gpu as G
    from mpaso._lib import lib

    mesh = mpaso.Mesh.icosa(5)
    dm = G.DeviceMesh(mesh, reorder=True)
    nC, nE = mesh.nCells, mesh.nEdges
    L = 64  # (4 nE + 3 nC) * 64 exceeds the static array
    he = torch.zeros((nE, L), dtype=torch.float64, device="cuda")
    c = torch.zeros((nC, L), dtype=torch.float64, device="cuda")
    rc = lib().mpaso_sw_compute_tend_noalloc(dm.handle, L, _ptr(he), _ptr(c), _ptr(he), _ptr(c), _ptr(he),
                                             _ptr(c), _ptr(he), None)
    assert rc == 1 and b"too large" in lib().mpaso_last_error()
    hh = np.zeros((nE, 1))
    rc = lib().mpaso_sw_compute_tend_noalloc(dm.handle, 1, hh.ctypes.data_as(ctypes.c_void_p), _ptr(c),
                                             _ptr(he), _ptr(c), _ptr(he), _ptr(c), _ptr(he), None)
    assert rc == 1 and b"device pointer" in lib().mpaso_last_error()
