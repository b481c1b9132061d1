"""ttn_qr_noalloc (workspace in a static device array, no device allocation) against the
allocating QR entry point ttn_debug_qr, through the C-ABI, on two calls in a row.

The two entry points run different kernels: ttn_qr_noalloc the column-by-column
cooperative Householder QR (k_qr_coop), ttn_debug_qr the sweep's panel-blocked one
(k_qr_blocked).  Both follow LAPACK's zgeqrf/zungqr conventions, so their factors agree to
rounding; the check uses the QR parity tolerance of the other device tests (relative
1e-12), and Q R = A and Q^H Q = I are checked on their own.  This file sorts after every
other test file, so pytest collects it last: a run that stops at the first failure has
run every other test before it.  That the entry point allocates nothing is checked on the
CPU test double (tests/test_host_orchestration.py), which counts allocations.
"""
import ctypes as C

import numpy as np
import pytest

from ttns_lib_gb300 import api

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def qr_allocating(a):
    q = np.ascontiguousarray(a, dtype=np.complex128).copy()
    m, n = q.shape
    r = np.zeros((n, n), dtype=np.complex128)
    api._check(api.lib().ttn_debug_qr(m, n, api._dp(q.view(np.float64)), api._dp(r.view(np.float64)), 0))
    return q, r


def qr_noalloc(torch, a):
    m, n = a.shape
    da = torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)).to("cuda:0")
    dr = torch.full((n, 2 * n), float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    api._check(api.lib().ttn_qr_noalloc(m, n, C.c_void_p(da.data_ptr()), C.c_void_p(dr.data_ptr()), stream, 0))
    q = da.cpu().numpy().view(np.complex128).reshape(m, n)
    r = dr.cpu().numpy().view(np.complex128).reshape(n, n)
    return q, r


def test_noalloc_qr_matches_allocating_entry_point_twice_in_a_row():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    shapes = [(4096, 64), (777, 17)]
    for m, n in shapes:
        a = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
        a[:, 3] *= 1e-160   # a tiny column exercises the scaled reflector path
        q0, r0 = qr_allocating(a)
        q1, r1 = qr_noalloc(torch, a)
        assert rel(q1, q0) < 1e-12, (m, n)
        assert rel(r1, r0) < 1e-12, (m, n)
        assert np.allclose(np.tril(r1, -1), 0.0)
        assert rel(q1 @ r1, a) < 1e-12
        assert np.abs(q1.conj().T @ q1 - np.eye(n)).max() < 1e-12


def test_noalloc_qr_rejects_sizes_beyond_its_workspace():
    torch = pytest.importorskip("torch")
    m, n = 256, 65
    da = torch.zeros((m, 2 * n), dtype=torch.float64, device="cuda:0")
    dr = torch.zeros((n, 2 * n), dtype=torch.float64, device="cuda:0")
    rc = api.lib().ttn_qr_noalloc(m, n, C.c_void_p(da.data_ptr()), C.c_void_p(dr.data_ptr()), None, 0)
    assert rc == api.TTN_ECAPACITY
    assert b"64 columns" in api.lib().ttn_last_error()
