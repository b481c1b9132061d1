"""ctypes wrapper of the CPU oracle (test infrastructure only).

Imported by the tests, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py`` -- never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(_HERE, f) for f in ("ttn_oracle.cpp", "ttn_adjoint.hpp", "ttn_expansion.hpp")]
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(os.path.getmtime(s) for s in srcs):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        P = C.c_void_p
        ip = C.POINTER(C.c_int)
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.c_int, ip, ip, ip, ip, C.c_int, dp, C.c_int, ip, dp, ip, ip, C.c_int,
                                 C.c_double, C.c_char_p, C.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_error.restype = C.c_char_p
        L.orc_error.argtypes = [P]
        L.orc_state_size.restype = C.c_longlong
        L.orc_state_size.argtypes = [P]
        for name in ("orc_set_state", "orc_get_state"):
            getattr(L, name).argtypes = [P, dp]
        L.orc_set_threads.argtypes = [P, C.c_int]
        L.orc_step.argtypes = [P, C.c_double, C.c_double, C.c_double]
        L.orc_sweep.argtypes = [P, C.c_double, C.c_double, C.c_double]
        L.orc_prepare.argtypes = [P]
        L.orc_t.restype = C.c_double
        L.orc_t.argtypes = [P]
        L.orc_nh.restype = C.c_longlong
        L.orc_nh.argtypes = [P]
        L.orc_expect.argtypes = [P, C.c_int, dp, dp]
        L.orc_bond_sv.argtypes = [P, C.c_int, dp]
        L.orc_refresh_env.argtypes = [P]
        L.orc_heff.argtypes = [P, C.c_int, dp, dp]
        L.orc_kbond.argtypes = [P, C.c_int, dp, dp]
        L.orc_expm_node.argtypes = [P, C.c_int, C.c_double, C.c_double, C.c_double, dp, C.POINTER(C.c_longlong)]
        L.orc_num_groups.argtypes = [P, C.c_int]
        L.orc_group_info.argtypes = [P, C.c_int, C.c_int, ip]
        L.orc_get_env.argtypes = [P, C.c_int, C.c_int, C.c_int, dp]
        L.orc_qr.argtypes = [C.c_int, C.c_int, dp, dp]
        L.orc_node_times.argtypes = [P, dp]
        L.orc_reset_node_times.argtypes = [P]
        L.orc_tql2.argtypes = [C.c_int, dp, dp, dp]
        L.orc_set_expansion.argtypes = [P, ip, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_uint]
        L.orc_get_hrank.argtypes = [P, ip]
        L.orc_top_eig.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.orc_set_op_update.argtypes = [P, P, P]
        L.orc_expand_prepare.argtypes = [P, C.c_double, ip]
        L.orc_expansion_counts.argtypes = [P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.orc_init_product.argtypes = [P, dp, C.c_uint]
        L.orc_orthogonalise.argtypes = [P]
        L.orc_set_krylov_stop.argtypes = [P, C.c_int]
        L.orc_adjoint.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_int, dp, C.c_int, dp, C.c_int, C.c_int,
                                  dp, dp, dp, dp]
        _lib = L
    return _lib


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """CPU FP64 one-site projector-splitting integrator over a tree."""

    def __init__(self, topo, sop, krylov_dim: int = 12, krylov_tol: float = 1e-12, threads: int = 1):
        L = lib()
        self.topo = topo
        coeff = np.ascontiguousarray(sop.coeffs, dtype=np.complex128)
        op_mode, op_data, bind_ptr, bind_r = sop.flat()
        op_data = np.ascontiguousarray(op_data, dtype=np.complex128)
        err = C.create_string_buffer(512)
        self._keep = (coeff, op_mode, op_data, bind_ptr, bind_r)
        self.h = L.orc_create(topo.nnodes, _ip(topo.parent), _ip(topo.hrank), _ip(topo.leaf_mode),
                              _ip(topo.leaf_dim), sop.nterms, _dp(coeff.view(np.float64)), len(op_mode),
                              _ip(op_mode), _dp(op_data.view(np.float64)), _ip(bind_ptr), _ip(bind_r),
                              krylov_dim, krylov_tol, err, 512)
        if not self.h:
            raise ValueError(err.value.decode())
        L.orc_set_threads(self.h, threads)
        self.offsets = topo.offsets()
        self._nterms = sop.nterms
        self._mode_dims = list(sop.mode_dims)
        self._opdims = [int(sop.mode_dims[m]) for m in op_mode]
        self._opsize = sum(d * d for d in self._opdims)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}: {lib().orc_error(self.h).decode()}")

    def set_state(self, tensors):
        flat = np.concatenate([np.asarray(t, dtype=np.complex128).ravel() for t in tensors])
        assert flat.size == self.current_topology().offsets()[-1]
        self._check(lib().orc_set_state(self.h, _dp(flat.view(np.float64))))

    def get_state(self):
        topo = self.current_topology()
        offs = topo.offsets()
        flat = np.zeros(int(offs[-1]), dtype=np.complex128)
        self._check(lib().orc_get_state(self.h, _dp(flat.view(np.float64))))
        return [flat[offs[i]:offs[i + 1]].reshape(topo.node_shape(i)).copy() for i in range(topo.nnodes)]

    def set_op_update(self, callback):
        """Time-dependent primitive operators: ``callback(mode, op, t, dt, mat)`` before
        every leaf evolution (``mat`` updated in place); ``None`` removes the hook."""
        if callback is None:
            self._check(lib().orc_set_op_update(self.h, None, None))
            self._op_cb = None
            return
        dims = self._mode_dims
        fn_t = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double))

        def trampoline(user, mode, op, t, dt, mat):
            d = dims[mode]
            arr = np.ctypeslib.as_array(mat, shape=(2 * d * d,)).view(np.complex128).reshape(d, d)
            callback(mode, op, t, dt, arr)

        self._op_cb = fn_t(trampoline)
        self._check(lib().orc_set_op_update(self.h, C.cast(self._op_cb, C.c_void_p), None))

    def hrank(self):
        out = np.zeros(self.topo.nnodes, dtype=np.int32)
        self._check(lib().orc_get_hrank(self.h, _ip(out)))
        return out

    def current_topology(self):
        """The tree with its current bond dimensions (they grow under subspace expansion)."""
        from ttns_lib_gb300.model import Topology
        return Topology(self.topo.parent, self.hrank(), self.topo.leaf_mode, self.topo.leaf_dim)

    def set_expansion(self, capacity, spawning_threshold: float = 1e-12, unoccupied_threshold: float = 1e-12,
                      minimum_unoccupied: int = 0, neigenvalues: int = 2, only_when_no_unoccupied: bool = False,
                      seed: int = 0):
        """Enable subspace expansion (adaptive bond dimension) for the following steps;
        ``capacity`` is the largest bond dimension above every node."""
        cap = np.ascontiguousarray(capacity, dtype=np.int32)
        assert cap.size == self.topo.nnodes
        self._check(lib().orc_set_expansion(self.h, _ip(cap), spawning_threshold, unoccupied_threshold,
                                            int(minimum_unoccupied), int(neigenvalues), int(only_when_no_unoccupied),
                                            int(seed)))

    def expand_prepare(self, dt: float) -> bool:
        grew = C.c_int(0)
        self._check(lib().orc_expand_prepare(self.h, dt, C.byref(grew)))
        return bool(grew.value)

    def step(self, dt: float, coeff: complex = -1j):
        self._check(lib().orc_step(self.h, dt, coeff.real, coeff.imag))

    def sweep(self, dt: float, coeff: complex = -1j):
        self._check(lib().orc_sweep(self.h, dt, coeff.real, coeff.imag))

    def prepare(self):
        self._check(lib().orc_prepare(self.h))

    def node_times(self):
        out = np.zeros(self.topo.nnodes)
        self._check(lib().orc_node_times(self.h, _dp(out)))
        return out

    def reset_node_times(self):
        self._check(lib().orc_reset_node_times(self.h))

    @property
    def nh_applications(self) -> int:
        return int(lib().orc_nh(self.h))

    def expansion_counts(self):
        """(one-site, two-site) expansions so far."""
        a, b = C.c_longlong(), C.c_longlong()
        self._check(lib().orc_expansion_counts(self.h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def set_krylov_stop(self, mode: int):
        """0: the full Krylov space of every sub-step (Expokit); 1: stop once the residual
        estimate for the remaining interval is below the tolerance."""
        self._check(lib().orc_set_krylov_stop(self.h, int(mode)))

    def orthogonalise(self):
        """Every non-root node made an isometry, the rest carried to the root."""
        self._check(lib().orc_orthogonalise(self.h))

    def init_product(self, psi0=None, seed: int = 0):
        """The spin-boson driver's start state drawn with std::mt19937(seed)."""
        if psi0 is None:
            self._check(lib().orc_init_product(self.h, None, int(seed)))
        else:
            p = np.ascontiguousarray(psi0, dtype=np.complex128)
            self._check(lib().orc_init_product(self.h, _dp(p.view(np.float64)), int(seed)))

    def expect(self, mode: int, op) -> complex:
        out = np.zeros(2)
        if op is None:
            self._check(lib().orc_expect(self.h, mode, None, _dp(out)))
        else:
            m = np.ascontiguousarray(op, dtype=np.complex128)
            self._check(lib().orc_expect(self.h, mode, _dp(m.view(np.float64)), _dp(out)))
        return complex(out[0], out[1])

    def norm2(self) -> float:
        return self.expect(0, None).real

    def bond_sv(self, node: int):
        out = np.zeros(int(self.topo.hrank[node]))
        self._check(lib().orc_bond_sv(self.h, node, _dp(out)))
        return out

    def refresh_env(self):
        self._check(lib().orc_refresh_env(self.h))

    def heff(self, node: int, v):
        x = np.ascontiguousarray(v, dtype=np.complex128).ravel()
        y = np.zeros_like(x)
        self._check(lib().orc_heff(self.h, node, _dp(x.view(np.float64)), _dp(y.view(np.float64))))
        return y.reshape(self.topo.node_shape(node))

    def kbond(self, node: int, v):
        x = np.ascontiguousarray(v, dtype=np.complex128).ravel()
        y = np.zeros_like(x)
        self._check(lib().orc_kbond(self.h, node, _dp(x.view(np.float64)), _dp(y.view(np.float64))))
        r = int(self.topo.hrank[node])
        return y.reshape(r, r)

    def expm_node(self, node: int, v, tau: float, coeff: complex = -1j):
        x = np.ascontiguousarray(v, dtype=np.complex128).ravel().copy()
        n = C.c_longlong(0)
        self._check(lib().orc_expm_node(self.h, node, tau, coeff.real, coeff.imag, _dp(x.view(np.float64)),
                                        C.byref(n)))
        return x.reshape(self.topo.node_shape(node)), int(n.value)

    def adjoint(self, dt: float, nsteps: int, weights, mode: int, op, checkpoint_every: int = 20,
                coeff: complex = -1j, skip_prepare: bool = False, state_cotangent: bool = False):
        """J = sum_k weights[k] Re <op on mode>(end of step k) over nsteps steps from the
        current state, and its gradients by the adjoint sweep: (J, dJ/dc_r per term,
        cotangent of every operator matrix in binding order[, cotangent of the state])."""
        w = np.ascontiguousarray(weights, dtype=np.float64)
        assert w.size == nsteps
        o = np.ascontiguousarray(op, dtype=np.complex128)
        J = np.zeros(1)
        gc = np.zeros(self._nterms)
        gops = np.zeros(self._opsize, dtype=np.complex128)
        gs = np.zeros(int(self.offsets[-1]), dtype=np.complex128) if state_cotangent else None
        self._check(lib().orc_adjoint(self.h, dt, coeff.real, coeff.imag, nsteps, _dp(w), mode, _dp(o.view(np.float64)),
                                      checkpoint_every, int(skip_prepare), _dp(J), _dp(gc),
                                      _dp(gops.view(np.float64)), _dp(gs.view(np.float64)) if gs is not None else None))
        ops, off = [], 0
        for d in self._opdims:
            ops.append(gops[off:off + d * d].reshape(d, d))
            off += d * d
        out = (float(J[0]), gc, ops)
        return out + (gs,) if state_cotangent else out

    def groups(self, node: int):
        out = []
        for g in range(lib().orc_num_groups(self.h, node)):
            info = np.zeros(6, dtype=np.int32)
            lib().orc_group_info(self.h, node, g, _ip(info))
            out.append(dict(type=int(info[0]), id_spf=bool(info[1]), id_mf=bool(info[2]), nmembers=int(info[3]),
                            nspf=int(info[4]), nmf=int(info[5])))
        return out

    def env(self, node: int, g: int, which: str):
        r = int(self.topo.hrank[node])
        out = np.zeros((r, r), dtype=np.complex128)
        self._check(lib().orc_get_env(self.h, node, g, 0 if which == "spf" else 1, _dp(out.view(np.float64))))
        return out


def qr(a):
    a = np.ascontiguousarray(a, dtype=np.complex128).copy()
    m, n = a.shape
    r = np.zeros((n, n), dtype=np.complex128)
    rc = lib().orc_qr(m, n, _dp(a.view(np.float64)), _dp(r.view(np.float64)))
    assert rc == 0
    return a, r


def top_eig(G, k: int):
    """The k largest eigenpairs of a Hermitian matrix as the subspace expansion computes them."""
    G = np.ascontiguousarray(G, dtype=np.complex128)
    g = G.shape[0]
    vals = np.zeros(k)
    vecs = np.zeros((k, g), dtype=np.complex128)
    n = lib().orc_top_eig(g, k, _dp(G.view(np.float64)), _dp(vals), _dp(vecs.view(np.float64)))
    assert n >= 0
    return vals[:n], vecs[:n]
