"""CPU-side checks of the C-ABI library: it loads, exports every symbol declared in
include/*.h (the boundary ttn_gb300.h and the test-only ttn_gb300_testing.h), and
validates its inputs on the host (no compute calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    inc = os.path.join(ROOT, "include")
    text = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc)) if f.endswith(".h"))
    return sorted(set(re.findall(r"\b(ttn_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = api.lib()
    names = declared_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the Python mirror binds all of them with explicit signatures
    assert set(names) <= set(api.SIGNATURES)


def test_version_string():
    assert b"sm_103a" in api.lib().ttn_version()


def test_tree_validation_on_host():
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3)
    t = api.Tree(m.topology)  # valid tree
    n = C.c_int()
    api._check(api.lib().ttn_tree_num_nodes(t.h, C.byref(n)))
    assert n.value == m.topology.nnodes
    size = C.c_longlong()
    api._check(api.lib().ttn_tree_state_size(t.h, C.byref(size)))
    assert size.value == m.topology.state_size()
    tp = m.topology

    def raw(parent, hrank):
        h = C.c_void_p()
        return api.lib().ttn_tree_create(len(parent), api._ip(parent), api._ip(hrank), api._ip(tp.leaf_mode),
                                         api._ip(tp.leaf_dim), C.byref(h))

    bad = tp.parent.copy()
    bad[3] = 7  # not pre-order
    assert raw(bad, tp.hrank) == api.TTN_EINVAL
    assert b"pre-order" in api.lib().ttn_last_error()
    hr = tp.hrank.copy()
    hr[2] = 10 ** 4  # exceeds the product of the child dimensions
    assert raw(tp.parent, hr) == api.TTN_EINVAL


def test_operator_validation_on_host():
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3)
    op = api.Operator(m.sop)
    md = np.array([2, 3], dtype=np.int32)
    h = C.c_void_p()
    api._check(api.lib().ttn_sop_create(2, 2, api._ip(md), C.byref(h)))
    mat = np.eye(2, dtype=np.complex128)
    r = np.array([0], dtype=np.int32)
    api._check(api.lib().ttn_sop_bind_dense(h, 0, api._dp(mat.view(np.float64)), api._ip(r), 1))
    # binding a second operator of the same term on the same mode is an error
    rc = api.lib().ttn_sop_bind_dense(h, 0, api._dp(mat.view(np.float64)), api._ip(r), 1)
    assert rc == api.TTN_EINVAL
    assert b"already" in api.lib().ttn_last_error()
    rr = np.array([5], dtype=np.int32)
    assert api.lib().ttn_sop_bind_dense(h, 0, api._dp(mat.view(np.float64)), api._ip(rr), 1) == api.TTN_EINVAL
    assert api.lib().ttn_sop_set_coeff(h, 0, float("nan"), 0.0) == api.TTN_EINVAL
    api.lib().ttn_sop_destroy(h)
    del op


def test_batch_step_validates_on_host():
    L = api.lib()
    failed = C.c_int(5)
    assert L.ttn_batch_step(None, None, 1, 0.0, -1.0, 0, C.byref(failed)) == api.TTN_EINVAL
    empty = (C.c_void_p * 1)()
    assert L.ttn_batch_step(empty, empty, 0, 0.0, -1.0, 0, C.byref(failed)) == api.TTN_OK
    assert failed.value == -1
    assert L.ttn_batch_step(empty, empty, 1, 0.0, -1.0, 0, C.byref(failed)) == api.TTN_EINVAL
    assert b"null instance" in L.ttn_last_error()
    with pytest.raises(ValueError):
        api.batch_step([object()], [], -1j)



def test_adjoint_grad_validates_on_host():
    L = api.lib()
    J = C.c_double()
    z = np.zeros(4)
    dp = z.ctypes.data_as(C.POINTER(C.c_double))
    assert L.ttn_adjoint_grad(None, None, 0.05, 0.0, -1.0, 1, dp, 0, dp, 1, 0, C.byref(J), dp, dp, None) == api.TTN_EINVAL
    assert b"null argument" in L.ttn_last_error()
