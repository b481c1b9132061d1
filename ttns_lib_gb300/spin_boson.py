"""Spin-boson workloads for the sweep.

H = (eps/2) sz + (Delta/2) sx + sz * sum_k c_k (b_k + b_k^dag) + sum_k w_k b_k^dag b_k

with an ohmic, exponentially cut-off bath discretised by

    w_k = -wc * ln(1 - k/(N+1)),     c_k = sqrt(alpha * wc / (N+1)) * w_k,   k = 1..N.

Finite temperature uses thermofield doubling: each mode k becomes the pair
(w_k, c_k cosh th_k) and (-w_k, c_k sinh th_k) with tanh th_k = exp(-beta w_k / 2);
both members of a pair start in their vacuum and sit on sibling leaves.

The operator layout follows the reference driver (src/spin_boson.cpp:499-543):
term 0 is the system Hamiltonian on mode 0; for bath mode i (tree mode i+1) term
1+2i is the diagonal w_i n on mode i+1 and term 2+2i is sz on mode 0 times the
coupling c_i (b + b^dag) on mode i+1.  The tree follows src/spin_boson.cpp:448-489:
root(1) -> [spin leaf, bath top (rank 2) -> balanced binary bath tree].
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from .model import SOPOperator, Topology, spin_bath_topology

SZ = np.array([[1, 0], [0, -1]], dtype=np.complex128)
SX = np.array([[0, 1], [1, 0]], dtype=np.complex128)
SY = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)


@dataclass
class SpinBosonModel:
    topology: Topology
    sop: SOPOperator
    omega: np.ndarray       # per bath mode (tree modes 1..M)
    coupling: np.ndarray    # per bath mode
    eps: float
    delta: float
    local_dim: int
    chi: int
    description: str


def ohmic_modes(N: int, alpha: float, wc: float):
    k = np.arange(1, N + 1, dtype=np.float64)
    w = -wc * np.log(1.0 - k / (N + 1.0))
    c = np.sqrt(alpha * wc / (N + 1.0)) * w
    return w, c


def thermofield(w: np.ndarray, c: np.ndarray, beta: float):
    th = np.arctanh(np.exp(-beta * w / 2.0))
    wt = np.empty(2 * len(w))
    ct = np.empty(2 * len(w))
    wt[0::2], wt[1::2] = w, -w
    ct[0::2], ct[1::2] = c * np.cosh(th), c * np.sinh(th)
    return wt, ct


def boson_ops(d: int):
    n = np.arange(d, dtype=np.float64)
    b = np.diag(np.sqrt(n[1:]), 1).astype(np.complex128)
    return n, b + b.conj().T


def build(N: int, alpha: float, wc: float, d: int, chi: int, eps: float = 0.0, delta: float = 1.0,
          beta: Optional[float] = None) -> SpinBosonModel:
    w, c = ohmic_modes(N, alpha, wc)
    if beta is not None:
        w, c = thermofield(w, c, beta)
    desc = f"spin-boson N={N}{' (thermofield x2)' if beta is not None else ''} alpha={alpha} wc={wc} d={d} chi={chi}"
    return build_from_modes(w, c, d, chi, eps, delta, desc)


def build_from_modes(w, c, d: int, chi: int, eps: float = 0.0, delta: float = 1.0,
                     description: str = "") -> SpinBosonModel:
    """The spin-boson operator and tree for explicit bath frequencies ``w`` and couplings
    ``c`` (one leaf per entry).  Operator binding order: 0 the system operator
    (eps/2) sz + (Delta/2) sx, 1 sz, then per bath mode i: 2+2i w_i n, 3+2i c_i (b + b^dag)."""
    w = np.asarray(w, dtype=np.float64)
    c = np.asarray(c, dtype=np.float64)
    M = len(w)
    topo = spin_bath_topology(2, [d] * M, chi)
    mode_dims = [2] + [d] * M
    H = SOPOperator(1 + 2 * M, mode_dims)
    H.bind_dense(0.5 * eps * SZ + 0.5 * delta * SX, [0], 0)
    H.bind_dense(SZ, [2 + 2 * i for i in range(M)], 0)
    n, x = boson_ops(d)
    for i in range(M):
        H.bind_diag(w[i] * n, [1 + 2 * i], i + 1)
        H.bind_dense(c[i] * x, [2 + 2 * i], i + 1)
    desc = description or f"spin-boson with {M} bath modes d={d} chi={chi}"
    return SpinBosonModel(topo, H, w, c, eps, delta, d, chi, desc)


def parameter_gradient(model: SpinBosonModel, op_cotangents) -> dict:
    """dJ/d(eps, Delta, c_k, w_k) from the cotangents of the operator matrices (binding
    order of ``build_from_modes``) returned by an adjoint sweep: for an operator
    O = p B, dJ/dp = Re sum conj(O_bar) * B."""
    G = op_cotangents
    d = model.local_dim
    n, x = boson_ops(d)
    M = len(model.omega)

    def proj(Gk, B):
        return float(np.real(np.sum(np.conj(Gk) * B)))

    return dict(eps=proj(G[0], 0.5 * SZ), delta=proj(G[0], 0.5 * SX),
                coupling=np.array([proj(G[3 + 2 * i], x) for i in range(M)]),
                omega=np.array([proj(G[2 + 2 * i], np.diag(n)) for i in range(M)]))


# The five workloads of the benchmark suite (synthetic, formula-generated).
def config(name: str) -> dict:
    cfgs = {
        # zero temperature, plain complex128, runs on the CPU oracle in seconds
        "c1": dict(N=16, alpha=0.5, wc=5.0, d=8, chi=8, eps=0.0, delta=1.0, beta=None,
                   dt=0.05, steps=200, krylov_dim=12),
        # thermofield beta=1, 2x256 modes, chi=32 (subspace expansion in the reference)
        "c2": dict(N=256, alpha=0.3, wc=5.0, d=16, chi=32, eps=0.0, delta=1.0, beta=1.0,
                   dt=0.02, steps=500, krylov_dim=16),
        # thermofield beta=10, 2x512 = 1024 modes, chi=64: the headline workload
        "c3": dict(N=512, alpha=0.2, wc=2.0, d=16, chi=64, eps=0.5, delta=1.0, beta=10.0,
                   dt=0.02, steps=1000, krylov_dim=16),
        # adjoint workload
        "c5": dict(N=128, alpha=0.4, wc=5.0, d=12, chi=24, eps=0.0, delta=1.0, beta=None,
                   dt=0.05, steps=400, krylov_dim=12),
    }
    return dict(cfgs[name])


def build_config(name: str, **override) -> tuple:
    cfg = config(name)
    cfg.update(override)
    m = build(cfg["N"], cfg["alpha"], cfg["wc"], cfg["d"], cfg["chi"], cfg["eps"], cfg["delta"], cfg["beta"])
    return m, cfg


def initial_state_numpy(topo: Topology, seed: int = 0, psi0: Optional[np.ndarray] = None) -> List[np.ndarray]:
    """Spin up / bath vacuum in SPF 0, random orthonormal unoccupied SPFs at the leaves,
    identity interior nodes and e_0 at the root (src/spin_boson.cpp:584-649), drawn
    from numpy's generator.  ``api.initial_state`` draws the same structure with
    std::mt19937 as the reference driver does."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(topo.nnodes):
        dimen, r = topo.node_shape(i)
        if topo.is_leaf(i):
            cols = np.zeros((r, dimen), dtype=np.complex128)
            if topo.leaf_mode[i] == 0 and psi0 is not None:
                cols[0] = psi0
            else:
                cols[0, 0] = 1.0
            for j in range(1, r):
                while True:
                    v = rng.normal(size=dimen) * np.exp(1j * rng.uniform(0, 2 * np.pi, size=dimen))
                    v /= np.linalg.norm(v)
                    for q in range(j):
                        v -= np.vdot(cols[q], v) * cols[q]
                    nv = np.linalg.norm(v)
                    if nv > 1e-12:
                        cols[j] = v / nv
                        break
            out.append(np.ascontiguousarray(cols.T))
        elif i != 0:
            out.append(np.eye(dimen, r, dtype=np.complex128))
        else:
            a = np.zeros((dimen, r), dtype=np.complex128)
            a[0, 0] = 1.0
            out.append(a)
    return out
