"""Python mirror of the reference's integrator interface over the C-ABI of libttn_gb300.

Names follow ttns_lib so that a caller's loop ports unchanged:

    A = httensor(topology)                          # httensor(topology, capacity)
    A.init_product(psi0, seed)                      # the driver's start state
    tdvp = fixed_step_projector_splitting_integrator(A, H, krylov_dim, krylov_tol)
    tdvp.dt = 0.05                                  # tdvp.dt() = dt
    tdvp(A, H, -1j)                                 # one step, returns dt
    tdvp.mel()(sz, 0, A)                            # <psi|O_0|psi>
    tdvp.nh_applications()

(include/ttns_lib/integrators/projector_splitting_integrator.hpp:76-218,
 include/ttns_lib/observables/matrix_element.hpp:264-314, src/spin_boson.cpp:41-107.)

Every call goes to the CUDA library; there is no host fallback.  A missing library or
a missing GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from .model import SOPOperator, Topology

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libttn_gb300.so")

TTN_OK, TTN_EINVAL, TTN_ECAPACITY, TTN_ENUMERIC, TTN_ECUDA, TTN_ETIMEOUT, TTN_ENOTSUP = range(7)
PREC_FP64, PREC_MIXED = 0, 1

_ERRNAMES = {1: "EINVAL", 2: "ECAPACITY", 3: "ENUMERIC", 4: "ECUDA", 5: "ETIMEOUT", 6: "ENOTSUP"}


class TTNError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"TTN_{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class ttn_integ_cfg(C.Structure):
    _fields_ = [("krylov_dim", C.c_int), ("krylov_tol", C.c_double), ("precision", C.c_int), ("device", C.c_int)]


# every exported symbol and its argument types (pointers as void* / double* / int*)
_P, _I, _D, _LL = C.c_void_p, C.c_int, C.c_double, C.c_longlong
_IP, _DP, _LLP = C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)
_PP = C.POINTER(C.c_void_p)
SIGNATURES = {
    "ttn_last_error": (C.c_char_p, []),
    "ttn_version": (C.c_char_p, []),
    "ttn_tree_create": (_I, [_I, _IP, _IP, _IP, _IP, _PP]),
    "ttn_tree_destroy": (_I, [_P]),
    "ttn_tree_num_nodes": (_I, [_P, _IP]),
    "ttn_tree_node_shape": (_I, [_P, _I, _LLP, _IP]),
    "ttn_tree_state_size": (_I, [_P, _LLP]),
    "ttn_sop_create": (_I, [_I, _I, _IP, _PP]),
    "ttn_sop_destroy": (_I, [_P]),
    "ttn_sop_bind_dense": (_I, [_P, _I, _DP, _IP, _I]),
    "ttn_sop_bind_diag": (_I, [_P, _I, _DP, _IP, _I]),
    "ttn_sop_bind_csr": (_I, [_P, _I, _IP, _IP, _DP, _IP, _I]),
    "ttn_sop_set_coeff": (_I, [_P, _I, _D, _D]),
    "ttn_state_create": (_I, [_P, _I, _PP]),
    "ttn_state_destroy": (_I, [_P]),
    "ttn_state_upload": (_I, [_P, _DP]),
    "ttn_state_download": (_I, [_P, _DP]),
    "ttn_state_upload_node": (_I, [_P, _I, _DP]),
    "ttn_state_download_node": (_I, [_P, _I, _DP]),
    "ttn_state_init_product": (_I, [_P, _DP, C.c_uint]),
    "ttn_integrator_create": (_I, [_P, _P, C.POINTER(ttn_integ_cfg), _PP]),
    "ttn_integrator_destroy": (_I, [_P]),
    "ttn_integrator_set_dt": (_I, [_P, _D]),
    "ttn_integrator_dt": (_I, [_P, _DP]),
    "ttn_integrator_t": (_I, [_P, _DP]),
    "ttn_integrator_step": (_I, [_P, _P, _D, _D, _DP]),
    "ttn_integrator_nh_applications": (_I, [_P, _LLP]),
    "ttn_integrator_expansion_counts": (_I, [_P, _LLP, _LLP]),
    "ttn_state_orthogonalise": (_I, [_P, _P]),
    "ttn_integrator_set_krylov_stop": (_I, [_P, _I]),
    "ttn_integrator_reset": (_I, [_P]),
    "ttn_integrator_synchronize": (_I, [_P]),
    "ttn_integrator_prepare": (_I, [_P, _P]),
    "ttn_integrator_set_profiling": (_I, [_P, _I]),
    "ttn_integrator_flops": (_I, [_P, _DP]),
    "ttn_integrator_timer": (_I, [_P, _I, _DP]),
    "ttn_bench_node_op": (_I, [_P, _P, _I, _I, _I, _DP, _DP]),
    "ttn_device_fp64_peak": (_I, [_I, _DP]),
    "ttn_launch_count": (_I, [C.POINTER(C.c_ulonglong)]),
    "ttn_integrator_io_bytes": (_I, [_P, _LLP, _LLP]),
    "ttn_integrator_profile": (_I, [_P, _DP, _LLP]),
    "ttn_host_alloc": (_I, [_LL, _PP]),
    "ttn_host_free": (_I, [_P]),
    "ttn_expect_leaf": (_I, [_P, _P, _I, _DP, _DP, _DP]),
    "ttn_norm2": (_I, [_P, _P, _DP]),
    "ttn_debug_refresh_env": (_I, [_P, _P]),
    "ttn_debug_heff": (_I, [_P, _I, _DP, _DP]),
    "ttn_debug_expm_node": (_I, [_P, _I, _D, _D, _D, _DP, _LLP]),
    "ttn_debug_program_apply": (_I, [_P, _I, _I, _DP, _DP]),
    "ttn_integrator_kernel_phases": (_I, [_P, _DP]),
    "ttn_debug_num_groups": (_I, [_P, _I, _IP]),
    "ttn_debug_get_env": (_I, [_P, _I, _I, _I, _DP]),
    "ttn_debug_qr": (_I, [_I, _I, _DP, _DP, _I]),
    "ttn_debug_qr_phases": (_I, [_I, _I, _DP, _DP, _I, _DP]),
    "ttn_qr_noalloc": (_I, [_I, _I, _P, _P, _P, _I]),
    "ttn_bond_singular_values": (_I, [_P, _P, _I, _DP, C.POINTER(C.c_int)]),
    "ttn_integrator_set_expansion": (_I, [_P, _P, _IP, _D, _D, _I, _I, _I, C.c_uint]),
    "ttn_state_hrank": (_I, [_P, _IP]),
    "ttn_overlap": (_I, [_P, _P, _P, _DP, _DP]),
    "ttn_integrator_save": (_I, [_P, _P, C.c_char_p]),
    "ttn_integrator_set_op_update": (_I, [_P, _P, _P]),
    "ttn_integrator_load": (_I, [_P, _P, C.c_char_p]),
    "ttn_expect_product": (_I, [_P, _P, _P, _I, _IP, _DP, _DP, _DP]),
    "ttn_expect_sop": (_I, [_P, _P, _P, _P, _DP, _DP]),
    "ttn_adjoint_grad": (_I, [_P, _P, _D, _D, _D, _I, _DP, _I, _DP, _I, _I, _DP, _DP, _DP, _DP]),
    "ttn_batch_step": (_I, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _I, _D, _D, _I, C.POINTER(C.c_int)]),
    "ttn_debug_tc_gemm": (_I, [_DP, _DP, _DP, _I, _I, _I]),
}

_lib = None

# void (*)(void* user, int mode, int op, double t, double dt, double* mat)
OP_UPDATE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double))


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m ttns_lib_gb300.build` (or __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != TTN_OK:
        raise TTNError(rc, lib().ttn_last_error().decode())


def _ip(a):
    return a.ctypes.data_as(_IP)


def _dp(a):
    return a.ctypes.data_as(_DP)


def _cplx(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


class Tree:
    def __init__(self, topo: Topology):
        self.topo = topo
        h = C.c_void_p()
        _check(lib().ttn_tree_create(topo.nnodes, _ip(topo.parent), _ip(topo.hrank), _ip(topo.leaf_mode),
                                     _ip(topo.leaf_dim), C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ttn_tree_destroy(self.h)
            self.h = None


class Operator:
    """Device-side copy of a SOPOperator (sop_operator)."""

    def __init__(self, sop: SOPOperator):
        self.sop = sop
        md = np.array(sop.mode_dims, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().ttn_sop_create(sop.nterms, len(md), _ip(md), C.byref(h)))
        self.h = h
        for b in sop.ops:
            r = np.array(b.terms, dtype=np.int32)
            sp = b.sparse_form()
            if sp is not None and sp[0] == "diag":
                dg = _cplx(sp[1])
                _check(lib().ttn_sop_bind_diag(h, b.mode, _dp(dg.view(np.float64)), _ip(r), len(r)))
            elif sp is not None and sp[0] == "csr":
                rp = np.ascontiguousarray(sp[1], dtype=np.int32)
                ci = np.ascontiguousarray(sp[2], dtype=np.int32)
                vals = _cplx(sp[3])
                _check(lib().ttn_sop_bind_csr(h, b.mode, _ip(rp), _ip(ci), _dp(vals.view(np.float64)), _ip(r), len(r)))
            else:
                m = _cplx(b.matrix)
                _check(lib().ttn_sop_bind_dense(h, b.mode, _dp(m.view(np.float64)), _ip(r), len(r)))
        for r, c in enumerate(sop.coeffs):
            _check(lib().ttn_sop_set_coeff(h, r, float(np.real(c)), float(np.imag(c))))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ttn_sop_destroy(self.h)
            self.h = None


class httensor:
    """Device-resident tree tensor network state (one arena, one slab per node)."""

    def __init__(self, topo: Topology, device: int = 0):
        self.topo = topo
        self.tree = Tree(topo)
        self.device = device
        h = C.c_void_p()
        _check(lib().ttn_state_create(self.tree.h, device, C.byref(h)))
        self.h = h
        self.offsets = topo.offsets()

    def __del__(self):
        if getattr(self, "h", None):
            lib().ttn_state_destroy(self.h)
            self.h = None

    def hrank(self) -> np.ndarray:
        """Current bond dimension above every node (grows under subspace expansion)."""
        out = np.zeros(self.topo.nnodes, dtype=np.int32)
        _check(lib().ttn_state_hrank(self.h, _ip(out)))
        return out

    def current_topology(self) -> Topology:
        return Topology(self.topo.parent, self.hrank(), self.topo.leaf_mode, self.topo.leaf_dim)

    def set(self, tensors: Sequence[np.ndarray]):
        topo = self.current_topology()
        flat = np.concatenate([_cplx(t).ravel() for t in tensors])
        if flat.size != topo.offsets()[-1]:
            raise ValueError("tensor sizes do not match the topology")
        _check(lib().ttn_state_upload(self.h, _dp(flat.view(np.float64))))

    def get(self) -> List[np.ndarray]:
        topo = self.current_topology()
        offs = topo.offsets()
        flat = np.zeros(int(offs[-1]), dtype=np.complex128)
        _check(lib().ttn_state_download(self.h, _dp(flat.view(np.float64))))
        return [flat[offs[i]:offs[i + 1]].reshape(topo.node_shape(i)).copy() for i in range(topo.nnodes)]

    def upload_from(self, buf: "PinnedBuffer"):
        _check(lib().ttn_state_upload(self.h, C.cast(buf.ptr, _DP)))

    def download_to(self, buf: "PinnedBuffer"):
        _check(lib().ttn_state_download(self.h, C.cast(buf.ptr, _DP)))

    def init_product(self, psi0: Optional[np.ndarray] = None, seed: int = 0):
        """Spin-boson start state with std::mt19937(seed) unoccupied SPFs (src/spin_boson.cpp:584-649)."""
        if psi0 is None:
            _check(lib().ttn_state_init_product(self.h, None, seed))
        else:
            p = _cplx(psi0)
            _check(lib().ttn_state_init_product(self.h, _dp(p.view(np.float64)), seed))


class PinnedBuffer:
    """Page-locked host buffer holding a whole state (numpy view in ``.array``)."""

    def __init__(self, n_complex: int):
        p = C.c_void_p()
        _check(lib().ttn_host_alloc(int(n_complex) * 16, C.byref(p)))
        self.ptr = p
        self.nbytes = int(n_complex) * 16
        arr_t = C.c_double * (2 * int(n_complex))
        self.array = np.frombuffer(arr_t.from_address(p.value), dtype=np.complex128)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().ttn_host_free(self.ptr)
            self.ptr = None


class matrix_element:
    """<psi|O_mode|psi> and <psi|psi> (matrix_element::operator())."""

    def __init__(self, integ: "fixed_step_projector_splitting_integrator"):
        self.integ = integ

    def overlap(self, bra: "httensor", ket: "httensor") -> complex:
        """<bra|ket> (matrix_element::operator()(bra, ket))."""
        re, im = C.c_double(), C.c_double()
        _check(lib().ttn_overlap(self.integ.h, bra.h, ket.h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def product(self, ops_by_mode: dict, bra: "httensor", ket: Optional["httensor"] = None) -> complex:
        """<bra| prod_m O_m |ket> for a {mode: dense operator} product (ket defaults to bra)."""
        ket = bra if ket is None else ket
        modes = np.array(sorted(ops_by_mode), dtype=np.int32)
        flat = np.concatenate([_cplx(ops_by_mode[int(m)]).ravel() for m in modes]) if len(modes) else np.zeros(1, np.complex128)
        re, im = C.c_double(), C.c_double()
        _check(lib().ttn_expect_product(self.integ.h, bra.h, ket.h, len(modes), _ip(modes), _dp(flat.view(np.float64)),
                                        C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def sop(self, H: SOPOperator, bra: "httensor", ket: Optional["httensor"] = None) -> complex:
        """<bra| H |ket> of a sum-of-product operator (ket defaults to bra)."""
        ket = bra if ket is None else ket
        op = Operator(H)
        re, im = C.c_double(), C.c_double()
        _check(lib().ttn_expect_sop(self.integ.h, bra.h, ket.h, op.h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def __call__(self, *args):
        if len(args) == 1:
            out = C.c_double()
            _check(lib().ttn_norm2(self.integ.h, args[0].h, C.byref(out)))
            return out.value
        op, mode, A = args
        m = _cplx(op)
        re, im = C.c_double(), C.c_double()
        _check(lib().ttn_expect_leaf(self.integ.h, A.h, int(mode), _dp(m.view(np.float64)), C.byref(re), C.byref(im)))
        return complex(re.value, im.value)


class fixed_step_projector_splitting_integrator:
    """One-site projector-splitting integrator with a fixed bond dimension."""

    def __init__(self, A: httensor, H: SOPOperator, krylov_dim: int = 4, krylov_tolerance: float = 1e-12,
                 precision: int = PREC_FP64, device: Optional[int] = None):
        self.topo = A.topo
        self.tree = Tree(A.topo)
        self.op = Operator(H)
        cfg = ttn_integ_cfg(int(krylov_dim), float(krylov_tolerance), int(precision),
                            int(A.device if device is None else device))
        h = C.c_void_p()
        _check(lib().ttn_integrator_create(self.tree.h, self.op.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._mel = matrix_element(self)
        self._sop = H

    def __del__(self):
        if getattr(self, "h", None):
            lib().ttn_integrator_destroy(self.h)
            self.h = None

    @property
    def dt(self) -> float:
        out = C.c_double()
        _check(lib().ttn_integrator_dt(self.h, C.byref(out)))
        return out.value

    @dt.setter
    def dt(self, value: float):
        _check(lib().ttn_integrator_set_dt(self.h, float(value)))

    def t(self) -> float:
        out = C.c_double()
        _check(lib().ttn_integrator_t(self.h, C.byref(out)))
        return out.value

    def __call__(self, A: httensor, H=None, coeff: complex = -1j) -> float:
        out = C.c_double()
        _check(lib().ttn_integrator_step(self.h, A.h, float(np.real(coeff)), float(np.imag(coeff)), C.byref(out)))
        return out.value

    step = __call__

    def nh_applications(self) -> int:
        out = C.c_longlong()
        _check(lib().ttn_integrator_nh_applications(self.h, C.byref(out)))
        return out.value

    def set_krylov_stop(self, mode: int):
        """0: the full Krylov space of every sub-step (default); 1: stop on the residual
        estimate for the remaining interval (the reference's rule)."""
        _check(lib().ttn_integrator_set_krylov_stop(self.h, int(mode)))

    def orthogonalise(self, A: httensor):
        """orthogonaliser(A): every non-root node of A made an isometry, the state unchanged."""
        _check(lib().ttn_state_orthogonalise(self.h, A.h))

    def expansion_counts(self):
        """(Nonesite, Ntwosite): one-site and two-site subspace expansions so far."""
        a, b = C.c_longlong(), C.c_longlong()
        _check(lib().ttn_integrator_expansion_counts(self.h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def prepare(self, A: httensor):
        _check(lib().ttn_integrator_prepare(self.h, A.h))

    def flops(self) -> float:
        out = C.c_double()
        _check(lib().ttn_integrator_flops(self.h, C.byref(out)))
        return out.value

    def timer_start(self):
        _check(lib().ttn_integrator_timer(self.h, 1, None))

    def timer_stop(self) -> float:
        out = C.c_double()
        _check(lib().ttn_integrator_timer(self.h, 0, C.byref(out)))
        return out.value

    PROFILE_KINDS = ["expm_node", "expm_bond", "r2l_qr", "l2r_qr", "mf_update", "spf_update", "apply_to_parent",
                     "apply_from_parent"]
    PROFILE_CLASSES = ["<1K", "<64K", "<1M", ">=1M"]

    def set_profiling(self, on: bool):
        """Synchronising per-operation wall-time breakdown (``profile()``) on or off; clears it."""
        _check(lib().ttn_integrator_set_profiling(self.h, int(bool(on))))

    def profile(self):
        t = np.zeros(32)
        n = np.zeros(32, dtype=np.int64)
        _check(lib().ttn_integrator_profile(self.h, _dp(t), n.ctypes.data_as(_LLP)))
        out = {}
        for k, kn in enumerate(self.PROFILE_KINDS):
            for c, cn in enumerate(self.PROFILE_CLASSES):
                if n[k * 4 + c]:
                    out[f"{kn}[{cn}]"] = (float(t[k * 4 + c]), int(n[k * 4 + c]))
        return out

    KERNEL_PHASES = ["begin", "matvec", "alpha", "reorth_coef", "reorth_norm", "avnorm", "control", "combine"]

    def kernel_phases(self):
        """ms per phase of the Krylov kernel since the last call (needs TTN_PROFILE)."""
        out = np.zeros(16)
        _check(lib().ttn_integrator_kernel_phases(self.h, _dp(out)))
        d = {k: float(out[i]) for i, k in enumerate(self.KERNEL_PHASES)}
        d["substeps"] = int(out[8])
        d["launches"] = int(out[9])
        for i, k in enumerate(["tc_exponents", "tc_chunks", "tc_drain", "tc_output"]):
            d[k] = float(out[10 + i])
        d["tc_tiles"] = int(out[14])
        d["tc_drain_tmem_ld"] = float(out[15])
        return d

    def io_bytes(self):
        a, b = C.c_longlong(), C.c_longlong()
        _check(lib().ttn_integrator_io_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def bench_node_op(self, A: httensor, node: int, kind: int, reps: int):
        ms, fl = C.c_double(), C.c_double()
        _check(lib().ttn_bench_node_op(self.h, A.h, node, kind, reps, C.byref(ms), C.byref(fl)))
        return ms.value, fl.value

    def bond_sv(self, A: httensor, node: int) -> np.ndarray:
        """Schmidt values across the bond above ``node`` (descending)."""
        out = np.zeros(int(self.topo.hrank[node]))
        n = C.c_int()
        _check(lib().ttn_bond_singular_values(self.h, A.h, node, _dp(out), C.byref(n)))
        return out[:n.value]

    def mel(self) -> matrix_element:
        return self._mel

    def set_op_update(self, callback):
        """Time-dependent primitive operators: ``callback(mode, op, t, dt, mat)`` is called
        before every leaf evolution for each operator bound on the leaf's mode (``op`` its
        binding index, ``mat`` its d x d complex matrix, to be updated in place);
        ``None`` removes the hook (primitive::update(t, dt) of the reference)."""
        if callback is None:
            _check(lib().ttn_integrator_set_op_update(self.h, None, None))
            self._op_cb = None
            return
        dims = self._sop.mode_dims

        def trampoline(user, mode, op, t, dt, mat):
            d = dims[mode]
            arr = np.ctypeslib.as_array(mat, shape=(2 * d * d,)).view(np.complex128).reshape(d, d)
            callback(mode, op, t, dt, arr)

        self._op_cb = OP_UPDATE_FN(trampoline)
        _check(lib().ttn_integrator_set_op_update(self.h, C.cast(self._op_cb, C.c_void_p), None))

    def save(self, A: httensor, path: str):
        """Checkpoint of this integrator and the state A (resumable with ``load``)."""
        _check(lib().ttn_integrator_save(self.h, A.h, os.fsencode(path)))

    def load(self, A: httensor, path: str):
        """Resume from a checkpoint written by ``save`` (same tree)."""
        _check(lib().ttn_integrator_load(self.h, A.h, os.fsencode(path)))

    def set_expansion(self, A: httensor, capacity, spawning_threshold: float = 1e-12,
                      unoccupied_threshold: float = 1e-12, minimum_unoccupied: int = 0, neigenvalues: int = 2,
                      only_when_no_unoccupied: bool = False, seed: int = 0):
        """Adaptive bond dimension for the following steps (subspace expansion); ``A`` is
        re-laid for the capacities and must be the state stepped afterwards."""
        cap = np.ascontiguousarray(capacity, dtype=np.int32)
        if cap.size != self.topo.nnodes:
            raise ValueError("one capacity per node")
        _check(lib().ttn_integrator_set_expansion(self.h, A.h, _ip(cap), float(spawning_threshold),
                                                  float(unoccupied_threshold), int(minimum_unoccupied),
                                                  int(neigenvalues), int(only_when_no_unoccupied), int(seed)))

    def adjoint(self, A: httensor, dt: float, nsteps: int, weights, mode: int, op, checkpoint_every: int = 20,
                coeff: complex = -1j, skip_prepare: bool = False, state_cotangent: bool = False):
        """J = sum_k weights[k] Re <op on mode>(end of step k) over ``nsteps`` steps of ``dt``
        from ``A`` (left at the final state) and its gradient by the adjoint sweep on the
        device: (J, dJ/dc_r per term, cotangent of every operator matrix in binding order
        [, cotangent of the prepared state as a list of node tensors]).  The integrator must
        be FP64 and at step 0."""
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.size != nsteps:
            raise ValueError("one weight per step")
        o = np.ascontiguousarray(op, dtype=np.complex128)
        J = C.c_double()
        gc = np.zeros(self._sop.nterms)
        dims = [int(b.matrix.shape[0]) for b in self._sop.ops]
        gops = np.zeros(sum(d * d for d in dims), dtype=np.complex128)
        offs = self.topo.offsets()
        gs = np.zeros(int(offs[-1]), dtype=np.complex128) if state_cotangent else None
        _check(lib().ttn_adjoint_grad(self.h, A.h, float(dt), float(np.real(coeff)), float(np.imag(coeff)), int(nsteps),
                                      _dp(w), int(mode), _dp(o.view(np.float64)), int(checkpoint_every),
                                      int(skip_prepare), C.byref(J), _dp(gc), _dp(gops.view(np.float64)),
                                      _dp(gs.view(np.float64)) if gs is not None else None))
        ops, off = [], 0
        for d in dims:
            ops.append(gops[off:off + d * d].reshape(d, d))
            off += d * d
        out = (J.value, gc, ops)
        if state_cotangent:
            out = out + ([gs[offs[i]:offs[i + 1]].reshape(self.topo.node_shape(i)) for i in range(self.topo.nnodes)],)
        return out

    def synchronize(self):
        _check(lib().ttn_integrator_synchronize(self.h))

    # ---- kernel-level entry points used by the parity tests
    def refresh_env(self, A: httensor):
        _check(lib().ttn_debug_refresh_env(self.h, A.h))

    def heff(self, node: int, v: np.ndarray) -> np.ndarray:
        x = _cplx(v).ravel()
        y = np.zeros_like(x)
        _check(lib().ttn_debug_heff(self.h, node, _dp(x.view(np.float64)), _dp(y.view(np.float64))))
        return y.reshape(self.topo.node_shape(node))

    def program_apply(self, node: int, v: np.ndarray, kind: int = 0) -> np.ndarray:
        """The node's compiled matvec program (kind 0 H_eff, 1 bond) applied once."""
        x = _cplx(v).ravel()
        y = np.zeros_like(x)
        _check(lib().ttn_debug_program_apply(self.h, node, kind, _dp(x.view(np.float64)), _dp(y.view(np.float64))))
        return y.reshape(v.shape)

    def expm_node(self, node: int, v: np.ndarray, tau: float, coeff: complex = -1j):
        x = _cplx(v).ravel().copy()
        n = C.c_longlong()
        _check(lib().ttn_debug_expm_node(self.h, node, tau, coeff.real, coeff.imag, _dp(x.view(np.float64)),
                                         C.byref(n)))
        return x.reshape(self.topo.node_shape(node)), n.value

    def num_groups(self, node: int) -> int:
        out = C.c_int()
        _check(lib().ttn_debug_num_groups(self.h, node, C.byref(out)))
        return out.value

    def env(self, node: int, group: int, which: str) -> np.ndarray:
        r = int(self.topo.hrank[node])
        out = np.zeros((r, r), dtype=np.complex128)
        _check(lib().ttn_debug_get_env(self.h, node, group, 0 if which == "spf" else 1, _dp(out.view(np.float64))))
        return out


class subspace_expansion_projector_splitting_integrator(fixed_step_projector_splitting_integrator):
    """The one-site integrator with subspace expansion (adaptive bond dimension), named and
    parameterised like the reference's subspace_expansion_projector_splitting_integrator
    (include/ttns_lib/integrators/projector_splitting_integrator.hpp:221-393): bonds grow
    up to ``capacity`` (one entry per node; the root's own rank does not grow)."""

    def __init__(self, A: httensor, H: SOPOperator, capacity, krylov_dim: int = 4, krylov_tolerance: float = 1e-12,
                 spawning_threshold: float = 1e-12, unoccupied_threshold: float = 1e-12, minimum_unoccupied: int = 0,
                 neigenvalues: int = 2, only_when_no_unoccupied: bool = False, seed: int = 0,
                 device: Optional[int] = None):
        super().__init__(A, H, krylov_dim=krylov_dim, krylov_tolerance=krylov_tolerance, precision=PREC_FP64,
                         device=device)
        self.set_expansion(A, capacity, spawning_threshold, unoccupied_threshold, minimum_unoccupied, neigenvalues,
                           only_when_no_unoccupied, seed)


def torch_objective(evaluate):
    """Wrap ``evaluate(theta) -> (J, dJ/dtheta)`` (numpy in, numpy out) as a function of a
    1-D torch tensor whose backward returns that gradient, so that the adjoint sweep can
    be checked with torch's autograd tooling (a check harness, not the product path: the
    gradient itself comes from ``ttn_adjoint_grad``)."""
    import torch

    class _Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            J, g = evaluate(theta.detach().cpu().numpy())
            ctx.save_for_backward(torch.as_tensor(np.asarray(g), dtype=theta.dtype, device=theta.device))
            return theta.new_tensor(float(J))

        @staticmethod
        def backward(ctx, gJ):
            (g,) = ctx.saved_tensors
            return gJ * g

    return _Objective.apply


def spin_boson_adjoint(omega, d: int, chi: int, state, dt: float, weights, krylov_dim: int = 12,
                       krylov_tolerance: float = 1e-12, checkpoint_every: int = 20, device: int = 0):
    """``evaluate(theta)`` for ``torch_objective``: theta = (eps, Delta, c_1..c_N) of a
    zero-temperature spin-boson model with bath frequencies ``omega``; J = sum_t w_t <sz>(t)
    over len(weights) steps from ``state``, gradient by the device adjoint sweep."""
    from . import spin_boson as sb
    omega = np.asarray(omega, dtype=np.float64)

    def evaluate(theta):
        theta = np.asarray(theta, dtype=np.float64)
        m = sb.build_from_modes(omega, theta[2:], d, chi, float(theta[0]), float(theta[1]))
        A = httensor(m.topology, device=device)
        A.set(state)
        integ = fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=krylov_dim,
                                                          krylov_tolerance=krylov_tolerance)
        J, _, gops = integ.adjoint(A, dt, len(weights), weights, 0, sb.SZ, checkpoint_every=checkpoint_every)
        g = sb.parameter_gradient(m, gops)
        return J, np.concatenate([[g["eps"], g["delta"]], g["coupling"]])

    return evaluate


def launch_count() -> int:
    out = C.c_ulonglong()
    _check(lib().ttn_launch_count(C.byref(out)))
    return out.value


def fp64_peak_tflops(device: int = 0) -> float:
    out = C.c_double()
    _check(lib().ttn_device_fp64_peak(device, C.byref(out)))
    return out.value


def device_tc_gemm(a: np.ndarray, b: np.ndarray, device: int = 0) -> np.ndarray:
    """D = A B^T on the tensor cores (A 128 x K, B N x K, real)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    assert a.shape[0] == 128 and a.shape[1] == b.shape[1]
    d = np.zeros((128, b.shape[0]), dtype=np.float64)
    _check(lib().ttn_debug_tc_gemm(_dp(a), _dp(b), _dp(d), a.shape[1], b.shape[0], device))
    return d


def device_qr(a: np.ndarray, device: int = 0):
    a = _cplx(a).copy()
    m, n = a.shape
    r = np.zeros((n, n), dtype=np.complex128)
    _check(lib().ttn_debug_qr(m, n, _dp(a.view(np.float64)), _dp(r.view(np.float64)), device))
    return a, r


def device_qr_phases(a: np.ndarray, device: int = 0):
    """device_qr with the shared-memory QR kernel's phase clock (microseconds per phase)."""
    a = _cplx(a).copy()
    m, n = a.shape
    r = np.zeros((n, n), dtype=np.complex128)
    ph = np.zeros(16)
    _check(lib().ttn_debug_qr_phases(m, n, _dp(a.view(np.float64)), _dp(r.view(np.float64)), device, _dp(ph)))
    names = ["barrier", "col_sums", "reflector", "w", "update", "partials", "panels", "r_and_q"]
    out = {k: float(ph[i]) for i, k in enumerate(names)}
    out["columns"] = int(ph[8])
    return a, r, out


def batch_step(integrators, states, coeff: complex = -1j, threads: int = 0):
    """Advance independent instances (integrator k with state k) by one step each,
    concurrently from ``threads`` host threads (0: all hardware threads)."""
    n = len(integrators)
    if len(states) != n:
        raise ValueError("one state per integrator")
    its = (C.c_void_p * max(n, 1))(*[it.h for it in integrators])
    sts = (C.c_void_p * max(n, 1))(*[st.h for st in states])
    failed = C.c_int(-1)
    _check(lib().ttn_batch_step(its, sts, n, coeff.real, coeff.imag, int(threads), C.byref(failed)))

