"""Host-side description of a tree tensor network state and a sum-of-product operator.

These mirror the reference's construction API so that a caller ports line by line:

* ``Topology`` plays the part of ``ntree<size_t>`` + ``ntree_builder`` +
  ``httensor(topology, capacity)`` (include/ttns_lib/httensor.hpp:51,
  include/ttns_lib/tree/ntree_builder.hpp:59-139, 215-261).  Nodes are numbered in
  pre-order, children ordered by id, exactly the contiguous node order of the
  reference's ``tree<T>`` (include/ttns_lib/tree/tree.hpp:187-192).
* ``SOPOperator`` plays the part of ``sop_operator<T>(nterms, mode_dims)`` with
  ``bind(op, r_indices, mode)`` and ``coeff(r)`` (include/ttns_lib/operators/
  sop_operator.hpp:262, 323-392, 471-473).  Primitive operators may be dense,
  diagonal or CSR, like ``dense_matrix_operator`` / ``diagonal_matrix_operator`` /
  ``sparse_matrix_operator`` (include/ttns_lib/operators/matrix_operators.hpp:14-79,
  151-209, 411-474); they are stored dense because every leaf operator of the
  sweep is at most a few dozen states wide.

Only numpy is used here; the device path lives behind the C-ABI (``api.py``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np


@dataclass
class Topology:
    """Pre-order tree: ``parent[0] == -1``; leaves carry (leaf_mode, leaf_dim)."""

    parent: np.ndarray
    hrank: np.ndarray
    leaf_mode: np.ndarray
    leaf_dim: np.ndarray

    def __post_init__(self):
        self.parent = np.ascontiguousarray(self.parent, dtype=np.int32)
        self.hrank = np.ascontiguousarray(self.hrank, dtype=np.int32)
        self.leaf_mode = np.ascontiguousarray(self.leaf_mode, dtype=np.int32)
        self.leaf_dim = np.ascontiguousarray(self.leaf_dim, dtype=np.int32)
        n = len(self.parent)
        self.children: List[List[int]] = [[] for _ in range(n)]
        for i in range(1, n):
            if not (0 <= self.parent[i] < i):
                raise ValueError("nodes must be numbered in pre-order (0 <= parent[i] < i)")
            self.children[self.parent[i]].append(i)
        self.dims: List[List[int]] = []
        for i in range(n):
            if self.children[i]:
                self.dims.append([int(self.hrank[c]) for c in self.children[i]])
            else:
                self.dims.append([int(self.leaf_dim[i])])

    @property
    def nnodes(self) -> int:
        return len(self.parent)

    @property
    def nmodes(self) -> int:
        return int(np.sum(self.leaf_mode >= 0))

    def is_leaf(self, i: int) -> bool:
        return not self.children[i]

    def dimen(self, i: int) -> int:
        return int(np.prod(self.dims[i]))

    def node_shape(self, i: int):
        return (self.dimen(i), int(self.hrank[i]))

    def node_size(self, i: int) -> int:
        return self.dimen(i) * int(self.hrank[i])

    def state_size(self) -> int:
        return sum(self.node_size(i) for i in range(self.nnodes))

    def offsets(self) -> np.ndarray:
        off = np.zeros(self.nnodes + 1, dtype=np.int64)
        for i in range(self.nnodes):
            off[i + 1] = off[i] + self.node_size(i)
        return off

    def mode_dims(self) -> List[int]:
        md = [0] * self.nmodes
        for i in range(self.nnodes):
            if self.leaf_mode[i] >= 0:
                md[int(self.leaf_mode[i])] = int(self.leaf_dim[i])
        return md


class _NTree:
    """Small builder used to lay out a topology the way ntree_builder does."""

    def __init__(self, value: int, phys: Optional[int] = None, mode: int = -1):
        self.value = value
        self.phys = phys
        self.mode = mode
        self.kids: List["_NTree"] = []

    def add(self, t: "_NTree") -> "_NTree":
        self.kids.append(t)
        return t


def _balanced(node: _NTree, leaves: Sequence[tuple], chi_of_level, level: int = 0):
    """Balanced binary subtree below ``node`` (ntree_builder.hpp:59-139, degree 2)."""
    n = len(leaves)
    if n == 1:
        d, mode = leaves[0]
        node.kids.append(_NTree(chi_of_level(level), phys=d, mode=mode))
        return
    r = n % 2
    start = 0
    for i in range(2):
        nchild = n // 2 + (1 if i < r else 0)
        sub = leaves[start:start + nchild]
        start += nchild
        if nchild == 1:
            d, mode = sub[0]
            node.kids.append(_NTree(chi_of_level(level), phys=d, mode=mode))
        else:
            child = node.add(_NTree(chi_of_level(level)))
            _balanced_internal(child, sub, chi_of_level, level + 1)


def _balanced_internal(node: _NTree, leaves, chi_of_level, level):
    n = len(leaves)
    r = n % 2
    start = 0
    for i in range(2):
        nchild = n // 2 + (1 if i < r else 0)
        sub = leaves[start:start + nchild]
        start += nchild
        if nchild == 1:
            d, mode = sub[0]
            node.kids.append(_NTree(chi_of_level(level), phys=d, mode=mode))
        else:
            child = node.add(_NTree(chi_of_level(level)))
            _balanced_internal(child, sub, chi_of_level, level + 1)


def _flatten(root: _NTree) -> Topology:
    parent, hrank, lm, ld = [], [], [], []
    vals = []

    def sanitise(t: _NTree) -> int:
        # post-order cap: hrank <= product of the children's values (ntree_builder.hpp:215-233)
        if t.phys is not None:
            t.value = min(t.value, t.phys)
            return t.value
        prod = 1
        for k in t.kids:
            prod *= sanitise(k)
        t.value = min(t.value, prod)
        return t.value

    sanitise(root)

    def walk(t: _NTree, par: int):
        idx = len(parent)
        parent.append(par)
        hrank.append(t.value)
        lm.append(t.mode if t.phys is not None else -1)
        ld.append(t.phys if t.phys is not None else 0)
        for k in t.kids:
            walk(k, idx)

    walk(root, -1)
    del vals
    return Topology(np.array(parent), np.array(hrank), np.array(lm), np.array(ld))


def spin_bath_topology(spin_dim: int, bath_dims: Sequence[int], chi: int) -> Topology:
    """root(1) -> [spin leaf (spin_dim), bath top (spin_dim) -> balanced binary bath].

    Same shape as the spin-boson driver (src/spin_boson.cpp:448-489) with a uniform
    bath bond dimension ``chi``; sanitising caps leaves at their local dimension.
    Mode 0 is the spin; bath modes are 1..len(bath_dims) in leaf order.
    """
    root = _NTree(1)
    root.add(_NTree(spin_dim, phys=spin_dim, mode=0))
    top = root.add(_NTree(spin_dim))
    leaves = [(int(d), k + 1) for k, d in enumerate(bath_dims)]
    if len(leaves) == 1:
        top.add(_NTree(chi, phys=leaves[0][0], mode=1))
    else:
        _balanced(top, leaves, lambda level: chi)
    return _flatten(root)


def balanced_topology(leaf_dims: Sequence[int], chi: int, root_rank: int = 1) -> Topology:
    """A balanced binary tree over ``leaf_dims`` with a root of rank ``root_rank``."""
    root = _NTree(root_rank)
    leaves = [(int(d), k) for k, d in enumerate(leaf_dims)]
    if len(leaves) == 1:
        root.add(_NTree(chi, phys=leaves[0][0], mode=0))
    else:
        _balanced_internal(root, leaves, lambda level: chi, 0)
    return _flatten(root)


@dataclass
class _Bound:
    mode: int
    matrix: np.ndarray
    terms: List[int]
    # ("diag", d) or ("csr", indptr, indices, data) when bound in that form; valid while
    # ``sparse_of`` is ``matrix`` (replacing the matrix drops back to the dense form)
    sparse: Optional[tuple] = None
    sparse_of: Optional[np.ndarray] = None

    def sparse_form(self):
        return self.sparse if self.sparse is not None and self.sparse_of is self.matrix else None


class SOPOperator:
    """H = sum_r c_r prod_nu O_{r,nu} with operators bound to (terms, mode)."""

    def __init__(self, nterms: int, mode_dims: Sequence[int]):
        self.nterms = int(nterms)
        self.mode_dims = [int(d) for d in mode_dims]
        self.coeffs = np.ones(self.nterms, dtype=np.complex128)
        self.ops: List[_Bound] = []
        self._taken = set()

    def _bind(self, mat: np.ndarray, terms, mode: int, sparse: Optional[tuple] = None):
        d = self.mode_dims[mode]
        mat = np.ascontiguousarray(mat, dtype=np.complex128)
        if mat.shape != (d, d):
            raise ValueError(f"operator on mode {mode} must be {d}x{d}")
        terms = [int(r) for r in terms]
        for r in terms:
            if not 0 <= r < self.nterms:
                raise ValueError("term index out of range")
            if (r, mode) in self._taken:
                raise ValueError(f"term {r} already has an operator on mode {mode}")
            self._taken.add((r, mode))
        self.ops.append(_Bound(mode, mat, terms, sparse, mat if sparse is not None else None))

    def bind_dense(self, mat, terms, mode: int):
        self._bind(np.asarray(mat), terms, mode)

    def bind_diag(self, diag, terms, mode: int):
        dg = np.ascontiguousarray(diag, dtype=np.complex128)
        self._bind(np.diag(dg), terms, mode, ("diag", dg))

    def bind_csr(self, indptr, indices, data, terms, mode: int):
        d = self.mode_dims[mode]
        indptr = np.asarray(indptr, dtype=np.int64)
        rows = np.repeat(np.arange(d), np.diff(indptr[:d + 1]))
        m = np.zeros((d, d), dtype=np.complex128)
        ind = np.asarray(indices, dtype=np.int64)[:len(rows)]
        dat = np.asarray(data, dtype=np.complex128)[:len(rows)]
        np.add.at(m, (rows, ind), dat)
        self._bind(m, terms, mode, ("csr", indptr[:d + 1].copy(), ind.copy(), dat.copy()))

    def set_coeff(self, r: int, c: complex):
        self.coeffs[r] = c

    # flat arrays shared by the C-ABI and the oracle
    def flat(self):
        op_mode = np.array([b.mode for b in self.ops], dtype=np.int32)
        op_data = np.concatenate([b.matrix.ravel() for b in self.ops]) if self.ops else np.zeros(0, np.complex128)
        bind_ptr = np.zeros(len(self.ops) + 1, dtype=np.int32)
        for k, b in enumerate(self.ops):
            bind_ptr[k + 1] = bind_ptr[k] + len(b.terms)
        bind_r = np.array([r for b in self.ops for r in b.terms], dtype=np.int32)
        return op_mode, np.ascontiguousarray(op_data), bind_ptr, bind_r

    def dense(self) -> np.ndarray:
        """Full Hilbert-space matrix (small systems only; used by known-answer tests)."""
        dims = self.mode_dims
        total = int(np.prod(dims))
        if total > 1 << 14:
            raise ValueError("system too large for a dense matrix")
        per_term = [[np.eye(d, dtype=np.complex128) for d in dims] for _ in range(self.nterms)]
        for b in self.ops:
            for r in b.terms:
                per_term[r][b.mode] = b.matrix
        H = np.zeros((total, total), dtype=np.complex128)
        for r in range(self.nterms):
            t = np.array([[1.0 + 0j]])
            for m in per_term[r]:
                t = np.kron(t, m)
            H += self.coeffs[r] * t
        return H


def full_state(topo: Topology, tensors: Sequence[np.ndarray]) -> np.ndarray:
    """Contract a tree state into the full vector, modes ordered 0..nmodes-1."""
    n = topo.nnodes

    def sub(i):
        # returns (array with shape (*leaf_dims_in_subtree, hrank), list of modes)
        A = np.asarray(tensors[i]).reshape(topo.node_shape(i))
        if topo.is_leaf(i):
            return A, [int(topo.leaf_mode[i])]
        parts = [sub(c) for c in topo.children[i]]
        T = A.reshape(*topo.dims[i], int(topo.hrank[i]))
        modes = []
        for k, (P, pm) in enumerate(parts):
            # contract child rank index with axis k of T (axes before k already expanded)
            ax = sum(len(parts[j][1]) for j in range(k))
            T = np.tensordot(P, T, axes=([P.ndim - 1], [ax]))
            # move the newly added child axes into position ax..
            nnew = P.ndim - 1
            order = list(range(nnew, nnew + ax)) + list(range(nnew)) + list(range(nnew + ax, T.ndim))
            T = np.transpose(T, order)
            modes += pm
        return T, modes

    T, modes = sub(0)
    T = T.reshape(*T.shape[:-1]) if T.shape[-1] == 1 else T
    perm = np.argsort(modes)
    T = np.transpose(T, list(perm) + ([] if T.ndim == len(modes) else [T.ndim - 1]))
    return T.reshape(-1) if T.ndim == len(modes) else T.reshape(-1, T.shape[-1])
