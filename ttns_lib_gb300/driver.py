"""The spin-boson driver: the reference's input files, run end to end on the device.

Restates src/spin_boson.cpp (main, :156-679) and src/mode_data.hpp on the host and
steps the state with this package's device integrator (``api.py``):

1. read the input file (JSON; keys matched with whitespace removed and lower-cased,
   complex numbers written as "a+bj"), spin_boson.cpp:176-306;
2. discretise the bath (``bath.py``), spin_boson.cpp:310-381;
3. partition the modes into blocks whose combined harmonic basis stays below a target
   dimension (``partition_modes``, mode_data.hpp:818-886) and build each block's basis
   (``harmonic_mode_combination::construct_basis_topology``, mode_data.hpp:120-229);
4. lay out the tree -- a root over a system leaf and a balanced binary bath tree whose
   bond dimension falls from ``nspf`` at the top to ``nspf lower`` at the leaves -- and
   the same tree of capacities (spin_boson.cpp:444-491);
5. bind the sum-of-product Hamiltonian H = Hsys + sum_b (H0_b + Scoup Hc_b)
   (spin_boson.cpp:497-545);
6. start from psi0 on the system and the vacuum on every block, with random unoccupied
   single-particle functions (spin_boson.cpp:584-649);
7. step with the subspace-expanding integrator and print one row per step: t, the
   expectation values of the observables on the system, the one-site and two-site
   expansion counts, the H applications per node and, optionally, every bond dimension
   (``run``, spin_boson.cpp:41-101).
"""
from __future__ import annotations

import json
import math
import sys
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, TextIO, Tuple

import numpy as np

from . import bath as _bath
from .model import SOPOperator, Topology, _flatten, _NTree

ECUT = 3000.0          # energy cutoff of a combined block basis (spin_boson.cpp:242)
NMAX_HIGH_TARGET = 250  # target block dimension above twice the high-frequency bound (:418)
MAX_BOND = 256          # widest bond of the device library (kMaxBond, csrc/ttn_kernels.cuh)


# --------------------------------------------------------------------------------------
# input
# --------------------------------------------------------------------------------------

def _complex(v) -> complex:
    if isinstance(v, str):
        return complex("".join(v.split()))
    return complex(v)


def _matrix(v) -> np.ndarray:
    a = np.array([[_complex(x) for x in row] for row in v], dtype=np.complex128)
    if a.ndim != 2:
        raise ValueError("expected a matrix")
    return a


def _vector(v) -> np.ndarray:
    return np.array([_complex(x) for x in v], dtype=np.complex128)


@dataclass
class DriverInput:
    """The driver's inputs with the reference's defaults (spin_boson.cpp:176-306)."""

    tmax: float
    dt: float
    nspf: int
    nspf_lower: int
    nmax_dim: int
    ntarget: int
    nmodes: int
    bath: _bath.SpectralDensity
    hsys: np.ndarray
    psi0: np.ndarray
    scoup: np.ndarray
    ops: List[np.ndarray]
    seed: int = 0
    nmax_high: Optional[int] = None
    high_frequency_bound: float = 10.0
    max_frequency_cutoff: Optional[float] = None
    negative_frequency_cutoff: Optional[float] = None
    bath_tol: float = 1e-5
    moment_scaling: float = 2.0
    krylov_tolerance: float = 1e-12
    krylov_dim: int = 6
    spawning_parameter: float = 1e-12
    unoccupied_threshold: float = 1e-12
    jacobi_alpha: float = 1.0
    jacobi_beta: float = 0.0
    nspf_capacity: Optional[int] = None
    nspf_lower_capacity: Optional[int] = None
    minimum_unoccupied: Optional[int] = None
    print_bond_dimension: bool = False
    output_file: Optional[str] = None
    check_bath_discretisation: bool = False
    nthreads: int = 1

    def __post_init__(self):
        if self.nmax_high is None:
            self.nmax_high = self.nmax_dim
        cap = self.nspf if self.nspf_capacity is None else max(self.nspf_capacity, self.nspf)
        self.nspf_capacity = cap
        low = self.nspf_lower if self.nspf_lower_capacity is None else max(self.nspf_lower_capacity, self.nspf_lower)
        self.nspf_lower_capacity = low
        if self.minimum_unoccupied is None:
            self.minimum_unoccupied = self.nspf_capacity


def parse_input(doc: Dict) -> DriverInput:
    """``DriverInput`` from a parsed input document; raises ValueError naming a missing or
    inconsistent entry, as the reference's ASSERT / CALL_AND_HANDLE messages do."""
    d = _bath.normalise_keys(doc)

    def req(k, conv):
        if k not in d:
            raise ValueError(f"input: missing required entry {k!r}")
        return conv(d[k])

    def opt(k, conv, default=None):
        return conv(d[k]) if k in d else default

    if "bath" not in d:
        raise ValueError("Spectral density not found.")
    hsys = req("hsys", _matrix)
    if hsys.shape[0] != hsys.shape[1]:
        raise ValueError("The system hamiltonian is not square.")
    n = hsys.shape[0]
    psi0 = req("psi0", _vector)
    if psi0.shape[0] != n:
        raise ValueError("The system wavefunction is not the correct size.")
    scoup = req("scoup", _matrix)
    if scoup.shape != (n, n):
        raise ValueError("The system contribution to the system-bath coupling operator must be a square matrix.")
    if "ops" not in d:
        raise ValueError("Unable to find observable operators.")
    raw = d["ops"]
    if raw and isinstance(raw[0], list) and raw[0] and isinstance(raw[0][0], list):
        ops = [_matrix(m) for m in raw]
    else:
        ops = [_matrix(raw)]
    for m in ops:
        if m.shape != (n, n):
            raise ValueError("The size of the observable operator matrix is not the same as the system Hilbert space "
                             "dimension.")
    return DriverInput(
        tmax=req("tmax", float), dt=req("dt", float), nspf=req("nspf", int), nspf_lower=req("nspflower", int),
        nmax_dim=req("maximumdimension", int), ntarget=req("targetdimension", int), nmodes=req("nmodes", int),
        bath=_bath.load_bath(d["bath"]), hsys=hsys, psi0=psi0, scoup=scoup, ops=ops,
        seed=opt("seed", int, 0), nmax_high=opt("maximumdimensionhighfrequency", int),
        high_frequency_bound=opt("highfrequencybound", float, 10.0),
        max_frequency_cutoff=opt("maxfrequencycutoff", float),
        negative_frequency_cutoff=opt("negativefrequencycutoff", float),
        bath_tol=opt("bathintegrationerrortolerance", float, 1e-5), moment_scaling=opt("momentscaling", float, 2.0),
        krylov_tolerance=opt("krylovtolerance", float, 1e-12), krylov_dim=opt("krylovdimension", int, 6),
        spawning_parameter=opt("spawningparameter", float, 1e-12),
        unoccupied_threshold=opt("unoccupiedthreshold", float, 1e-12), jacobi_alpha=opt("jacobialpha", float, 1.0),
        jacobi_beta=opt("jacobibeta", float, 0.0), nspf_capacity=opt("nspfcapacity", int),
        nspf_lower_capacity=opt("nspflowercapacity", int), minimum_unoccupied=opt("minimumunoccupied", int),
        print_bond_dimension=opt("printbonddimension", bool, False), output_file=opt("outputfile", str),
        check_bath_discretisation=opt("checkbathdiscretisation", bool, False), nthreads=opt("nthreads", int, 1))


def load_input(path: str) -> DriverInput:
    with open(path) as f:
        return parse_input(json.load(f))


# --------------------------------------------------------------------------------------
# bath modes, blocks and their operators
# --------------------------------------------------------------------------------------

def frequency_window(inp: DriverInput) -> Tuple[float, float]:
    """[w_min, w_max] of the discretisation (spin_boson.cpp:317-356): a user cutoff gives
    [-cut, cut], else the bath's own bounds; at finite temperature a user negative cutoff
    replaces w_min; at zero temperature w_min = 0."""
    b = inp.bath
    if inp.max_frequency_cutoff is not None:
        lo, hi = -inp.max_frequency_cutoff, inp.max_frequency_cutoff
    else:
        lo, hi = b.frequency_bounds(inp.bath_tol, thermofield=True)
    if b.nonzero_temperature:
        if inp.negative_frequency_cutoff is not None:
            lo = inp.negative_frequency_cutoff
        return float(lo), float(hi)
    return 0.0, float(hi)


def bath_modes(inp: DriverInput) -> Tuple[np.ndarray, np.ndarray]:
    """Frequencies (sorted by |w|) and couplings of the discretised bath."""
    lo, hi = frequency_window(inp)
    return _bath.discretise(inp.bath, inp.nmodes, lo, hi)


def _nper(w: float, ecut: float, nmax: int) -> int:
    """States kept for one mode: min(nmax, floor(ecut / |w|)) (mode_data.hpp:133, :788)."""
    return min(int(nmax), int(ecut / abs(w)))


def block_nstates(wk: Sequence[float], ecut: float, nmax: int) -> int:
    """Dimension of a block: every mode gets the first mode's count (the lowest
    frequency of the block), so the block holds nper(w_0)^n states
    (``compute_nstates`` / ``get_nstates_in_cut``, mode_data.hpp:230-235, 786-795)."""
    return _nper(wk[0], ecut, nmax) ** len(wk)


def partition_modes(wk: np.ndarray, ecut: float, wc: float, nmax: int, nmax4: int, nmax2: int,
                    nmax3: int) -> List[int]:
    """Block sizes, lowest frequencies first (mode_data.hpp:818-886): a block starting at
    mode ``count`` grows while its dimension stays <= nmax (nmax4 when w_count > wc), the
    per-mode limit being nmax2 (nmax3 when w_count > wc); a lone mode that already exceeds
    the target still forms a block."""
    N = len(wk)
    if N == 0:
        raise ValueError("Failed to partition modes.  We cannot have zero modes.")
    if np.any(np.abs(wk[1:]) < np.abs(wk[:-1])):
        raise ValueError("Failed to partition modes.  The frequency array must be sorted from smallest to largest.")
    parts = []
    count = 0
    remaining = N
    while remaining:
        high = wk[count] > wc
        nmaxt = nmax3 if high else nmax2
        nmaxp = nmax4 if high else nmax
        ntoadd = 1
        while True:
            nt = block_nstates(wk[count:count + ntoadd], ecut, nmaxt)
            if nt > nmaxp:
                if ntoadd > 1:
                    ntoadd -= 1
                break
            if remaining > ntoadd:
                ntoadd += 1
            else:
                break
        parts.append(ntoadd)
        remaining -= ntoadd
        count += ntoadd
    return parts


@dataclass
class Block:
    """One combined bath mode: its harmonic modes, basis and operators."""

    wk: np.ndarray
    gk: np.ndarray
    nmax: int
    nstates: int
    occupations: np.ndarray          # (populated rows, nmodes), lexicographic
    h0: np.ndarray = field(repr=False)  # diagonal, length nstates
    hc_indptr: np.ndarray = field(repr=False)
    hc_indices: np.ndarray = field(repr=False)
    hc_data: np.ndarray = field(repr=False)

    def hc_dense(self) -> np.ndarray:
        m = np.zeros((self.nstates, self.nstates), dtype=np.complex128)
        for i in range(self.nstates):
            for q in range(self.hc_indptr[i], self.hc_indptr[i + 1]):
                m[i, self.hc_indices[q]] += self.hc_data[q]
        return m


def make_block(wk: np.ndarray, gk: np.ndarray, ecut: float, nmax: int) -> Block:
    """The block's basis and operators (``construct_basis_topology``, ``H0``, ``Hc``;
    mode_data.hpp:120-229, 237-313).

    The basis is the product of per-mode occupations n_j < min(nmax, floor(ecut/|w_j|)),
    listed lexicographically with the first mode slowest; H0 = sum_j w_j n_j (diagonal)
    and Hc = sum_j g_j (a_j + a_j^dagger), whose CSR row lists the lowering entries
    (mode order) before the raising ones (reverse mode order).

    The block's dimension is nper(w_0)^n (``block_nstates``).  When a later mode keeps
    fewer states than the first, the product basis is shorter than that; the remaining
    rows are kept, with zero energy and no coupling, so that the block has the
    reference's dimension.  (The reference leaves their content to its matrix library's
    resize; they are never occupied from the vacuum start.)
    """
    wk = np.asarray(wk, dtype=np.float64)
    gk = np.asarray(gk, dtype=np.float64)
    n = len(wk)
    nstates = block_nstates(wk, ecut, nmax)
    if n == 1:
        per = [min(nstates, int(nmax))]
    else:
        per = [_nper(w, ecut, nmax) for w in wk]
    occ = np.array(np.unravel_index(np.arange(int(np.prod(per))), per)).T.astype(np.int64)
    if occ.shape[0] > nstates:
        raise AssertionError("block basis larger than its dimension")
    P = occ.shape[0]
    h0 = np.zeros(nstates, dtype=np.float64)
    h0[:P] = occ @ wk
    # index of an occupation vector in the lexicographic product basis
    stride = np.ones(n, dtype=np.int64)
    for j in range(n - 2, -1, -1):
        stride[j] = stride[j + 1] * per[j + 1]
    # entries (row, order within the row, column, value): lowering entries in mode order,
    # then raising entries in reverse mode order; row i of the product basis is i itself
    rows, keys, cols, vals = [], [], [], []
    idx = np.arange(P, dtype=np.int64)
    for j in range(n):
        lo = occ[:, j] > 0
        rows.append(idx[lo]); keys.append(np.full(int(lo.sum()), j)); cols.append(idx[lo] - stride[j])
        vals.append(np.sqrt(occ[lo, j].astype(np.float64)) * gk[j])
        up = occ[:, j] + 1 < per[j]
        rows.append(idx[up]); keys.append(np.full(int(up.sum()), 2 * n - 1 - j)); cols.append(idx[up] + stride[j])
        vals.append(np.sqrt(occ[up, j].astype(np.float64) + 1.0) * gk[j])
    rows, keys, cols, vals = (np.concatenate(a) for a in (rows, keys, cols, vals))
    order = np.lexsort((keys, rows))
    indptr = np.zeros(nstates + 1, dtype=np.int64)
    indptr[1:P + 1] = np.cumsum(np.bincount(rows, minlength=P))
    indptr[P + 1:] = indptr[P]
    return Block(wk, gk, int(nmax), int(nstates), occ, h0, indptr, cols[order].astype(np.int64),
                 vals[order].astype(np.float64))


def make_blocks(inp: DriverInput, wk: np.ndarray, gk: np.ndarray) -> List[Block]:
    """Partition and build every block (spin_boson.cpp:408-436)."""
    wc2 = 2.0 * inp.high_frequency_bound
    parts = partition_modes(wk, ECUT, wc2, inp.ntarget, NMAX_HIGH_TARGET, inp.nmax_dim, inp.nmax_high)
    blocks = []
    s = 0
    for p in parts:
        nmaxt = inp.nmax_high if wk[s] > wc2 else inp.nmax_dim
        blocks.append(make_block(wk[s:s + p], gk[s:s + p], ECUT, nmaxt))
        s += p
    return blocks


# --------------------------------------------------------------------------------------
# tree, Hamiltonian, observables
# --------------------------------------------------------------------------------------

def level_ranks(nspf: int, nspf_lower: int, nlevels: int):
    """Bond dimension of the bath tree by depth (spin_boson.cpp:452-466): nspf at the top
    (level 0), nspf_lower from level nlevels on, and in between the geometric
    interpolation 2^((nlevels - l)(log2 nspf - log2 nspf_lower) / nlevels + log2
    nspf_lower), truncated."""
    rmax = math.log2(nspf)
    rmin = math.log2(nspf_lower)

    def f(l: int) -> int:
        if l >= nlevels:
            return int(nspf_lower)
        if l == 0:
            return int(nspf)
        return int(math.pow(2.0, ((nlevels - l) * (rmax - rmin)) / nlevels + rmin))

    return f


def _subtree(node: _NTree, leaves: Sequence[Tuple[int, int]], fl, level: int):
    """A balanced binary subtree (ntree_builder::balanced_subtree, include/ttns_lib/tree/
    ntree_builder.hpp:59-131): children at ``level`` get fl(level); a child with one
    leaf is a tree leaf carrying the block."""
    n = len(leaves)
    if n < 2:
        for (d, mode) in leaves:
            node.add(_NTree(fl(level), phys=d, mode=mode))
        return
    r = n % 2
    start = 0
    for i in range(2):
        nchild = n // 2 + (1 if i < r else 0)
        sub = leaves[start:start + nchild]
        start += nchild
        if nchild == 1:
            node.add(_NTree(fl(level), phys=sub[0][0], mode=sub[0][1]))
        else:
            _subtree(node.add(_NTree(fl(level))), sub, fl, level + 1)


def driver_topology(nhilb: int, block_dims: Sequence[int], nspf: int, nspf_lower: int) -> Topology:
    """root(1) -> [system leaf (nhilb), bath top (nhilb) -> balanced binary tree over the
    blocks], sanitised so that no bond exceeds the product of its children's
    (spin_boson.cpp:444-467, ntree_builder::sanitise_tree)."""
    nlevels = int(math.log2(len(block_dims)))
    fl = level_ranks(nspf, nspf_lower, nlevels)
    root = _NTree(1)
    root.add(_NTree(nhilb, phys=nhilb, mode=0))
    top = root.add(_NTree(nhilb))
    _subtree(top, [(int(d), k + 1) for k, d in enumerate(block_dims)], fl, 0)
    return _flatten(root)


def build_hamiltonian(inp: DriverInput, blocks: Sequence[Block], dense: bool = True) -> SOPOperator:
    """H = Hsys + sum_b [H0_b + Scoup Hc_b] (spin_boson.cpp:497-545): term 0 is Hsys on
    the system, term 1 + 2b is H0 on block b, term 2 + 2b couples Scoup on the system to
    Hc on block b."""
    nb = len(blocks)
    dims = [inp.hsys.shape[0]] + [b.nstates for b in blocks]
    H = SOPOperator(1 + 2 * nb, dims)
    H.bind_dense(inp.hsys, [0], 0)
    H.bind_dense(inp.scoup, [2 + 2 * i for i in range(nb)], 0)
    for i, b in enumerate(blocks):
        H.bind_diag(b.h0, [1 + 2 * i], i + 1)
        H.bind_csr(b.hc_indptr, b.hc_indices, b.hc_data, [2 + 2 * i], i + 1)
    return H


class InteractionPictureCoupling:
    """The coupling of one block in the interaction picture of its H0, for the
    time-dependent operator hook (``set_op_update``): ``interaction_picture_sb_operator``
    (src/system_bath_coupling_interaction_picture_operator.hpp:10-207, built from a block
    by ``Hc_interact``, src/mode_data.hpp:315-320).

    Before a leaf evolution over [t, t + dt] the matrix becomes
    sum_j (gt_j a_j^dagger + conj(gt_j) a_j), where gt_j is g_j exp(i w_j s) averaged over
    s in [t, t + dt]: g_j e^{i w_j t} (e^{i w_j dt} - 1) / (i w_j dt).  When |w_j dt| < 1e-5
    the reference sums the 20-term series of e^x, x = i w_j dt, in place of (e^x - 1)/x, so
    it uses the value at the end of the interval, g_j e^{i w_j (t + dt)}; that is kept (it
    differs from the mean by less than 1e-5 |g_j| / 2).  The block's own H0 is left out of
    the Hamiltonian (``build_interaction_picture_hamiltonian``).
    """

    def __init__(self, block: Block):
        self.block = block
        b = block
        rows = np.repeat(np.arange(b.nstates), np.diff(b.hc_indptr))
        cols = b.hc_indices
        occ = b.occupations
        n = occ.shape[1]
        # classify every CSR entry: lowering (column = row - e_j, a^dagger element) or raising
        mode = np.zeros(len(cols), dtype=np.int64)
        up = np.zeros(len(cols), dtype=bool)
        amp = np.zeros(len(cols))
        stride = np.ones(n, dtype=np.int64)
        per = [int(occ[:, j].max()) + 1 for j in range(n)] if occ.shape[0] else [1] * n
        for j in range(n - 2, -1, -1):
            stride[j] = stride[j + 1] * per[j + 1]
        for q, (r, c) in enumerate(zip(rows, cols)):
            diff = int(c) - int(r)
            j = int(np.nonzero(stride == abs(diff))[0][0]) if n > 1 else 0
            mode[q] = j
            if diff < 0:            # <n|a_j^dagger|n - 1> = sqrt(n)
                amp[q] = math.sqrt(float(occ[r, j]))
            else:                   # <n|a_j|n + 1> = sqrt(n + 1)
                up[q] = True
                amp[q] = math.sqrt(float(occ[r, j] + 1))
        self._rows, self._cols, self._mode, self._up, self._amp = rows, cols, mode, up, amp

    def averaged_couplings(self, t: float, dt: float) -> np.ndarray:
        w = self.block.wk
        g = self.block.gk
        out = np.zeros(len(w), dtype=np.complex128)
        for i in range(len(w)):
            ukt = complex(math.cos(w[i] * t), math.sin(w[i] * t))
            x = 1j * w[i] * dt
            if abs(w[i] * dt) < 1e-5:
                s, f = 0.0 + 0.0j, 1.0 + 0.0j
                for k in range(20):
                    s += f
                    f *= x / (k + 1.0)
                out[i] = g[i] * ukt * s
            else:
                out[i] = g[i] * ukt * (complex(math.cos(w[i] * dt), math.sin(w[i] * dt)) - 1.0) / x
        return out

    def matrix(self, t: float, dt: float) -> np.ndarray:
        gt = self.averaged_couplings(t, dt)
        m = np.zeros((self.block.nstates, self.block.nstates), dtype=np.complex128)
        vals = np.where(self._up, np.conj(gt[self._mode]), gt[self._mode]) * self._amp
        m[self._rows, self._cols] = vals
        return m


def build_interaction_picture_hamiltonian(inp: DriverInput, blocks: Sequence[Block]):
    """H(t) = Hsys + sum_b Scoup Hc_b(t) in the interaction picture of the bath (term 0 is
    Hsys, term 1 + b couples block b) and the hook that updates every Hc_b(t); pass the
    hook to ``set_op_update`` of the integrator (or of the oracle)."""
    nb = len(blocks)
    dims = [inp.hsys.shape[0]] + [b.nstates for b in blocks]
    H = SOPOperator(1 + nb, dims)
    H.bind_dense(inp.hsys, [0], 0)
    H.bind_dense(inp.scoup, [1 + i for i in range(nb)], 0)
    ops = [InteractionPictureCoupling(b) for b in blocks]
    for i, op in enumerate(ops):
        H.bind_dense(op.matrix(0.0, 0.0), [1 + i], i + 1)

    def update(mode, op, t, dt, mat):
        if mode >= 1:
            mat[:] = ops[mode - 1].matrix(t, dt)

    return H, update


@dataclass
class DriverModel:
    inp: DriverInput
    wk: np.ndarray
    gk: np.ndarray
    blocks: List[Block]
    topology: Topology
    capacity: np.ndarray
    hamiltonian: SOPOperator


def build_model(inp: DriverInput) -> DriverModel:
    """Everything the driver sets up before stepping (spin_boson.cpp:310-545)."""
    wk, gk = bath_modes(inp)
    blocks = make_blocks(inp, wk, gk)
    dims = [b.nstates for b in blocks]
    n = inp.hsys.shape[0]
    topo = driver_topology(n, dims, inp.nspf, inp.nspf_lower)
    H = build_hamiltonian(inp, blocks)
    return DriverModel(inp, wk, gk, blocks, topo, capacity_tree(inp, dims, topo), H)


def capacity_tree(inp: DriverInput, dims: Sequence[int], topo: Topology, log: Optional[TextIO] = None) -> np.ndarray:
    """Largest bond above every node: the tree of ``nspf capacity`` / ``nspf lower
    capacity`` (spin_boson.cpp:469-489), never below the starting bonds, and capped at the
    device library's widest bond (``MAX_BOND``); a cap that bites is reported on ``log``."""
    cap = driver_topology(inp.hsys.shape[0], dims, inp.nspf_capacity, inp.nspf_lower_capacity).hrank
    cap = np.maximum(cap, topo.hrank)
    if np.any(topo.hrank > MAX_BOND):
        raise ValueError(f"starting bond dimensions above {MAX_BOND} are not supported by the device library")
    if np.any(cap > MAX_BOND):
        (log or sys.stderr).write(f"bond capacities above {MAX_BOND} (up to {int(cap.max())}) are capped at "
                                  f"{MAX_BOND}, the widest bond of the device library\n")
        cap = np.minimum(cap, MAX_BOND)
    return cap


# --------------------------------------------------------------------------------------
# stepping and output
# --------------------------------------------------------------------------------------

def _g(x: float) -> str:
    """A number as the reference prints it (std::setprecision(16), default format)."""
    return format(float(x), ".16g")


def format_row(t: float, values: Sequence[float], counts: Optional[Tuple[int, int]], nh_per_node: Optional[float],
               hrank: Optional[Sequence[int]]) -> str:
    """One output row (spin_boson.cpp:41-101): t, the observables, then "0 0 0" on the
    first row or Nonesite Ntwosite nh/nodes on the others, then the bond dimensions of
    every non-root node when requested."""
    s = _g(t) + " " + "".join(_g(v) + " " for v in values)
    if counts is None:
        s += " 0 0 0 "
    else:
        s += f"{int(counts[0])} {int(counts[1])} " + _g(nh_per_node) + " "
    if hrank is not None:
        s += "".join(f"{int(h)} " for h in hrank)
    return s + "\n"


def nsteps_for(tmax: float, dt: float) -> int:
    """Steps taken by ``while(tdvp.t() < tmax)`` with t = dt * nsteps."""
    n = 0
    while dt * n < tmax:
        n += 1
    return n


class SpinBosonRun:
    """The device state, Hamiltonian and subspace-expanding integrator of one input file
    (spin_boson.cpp:584-662), stepped one row at a time."""

    def __init__(self, inp: DriverInput, model: Optional[DriverModel] = None, device: int = 0, krylov_stop: int = 0):
        from . import api
        self.inp = inp
        self.model = model if model is not None else build_model(inp)
        m = self.model
        self.A = api.httensor(m.topology, device=device)
        self.A.init_product(inp.psi0, inp.seed)
        self.tdvp = api.subspace_expansion_projector_splitting_integrator(
            self.A, m.hamiltonian, m.capacity, krylov_dim=inp.krylov_dim, krylov_tolerance=inp.krylov_tolerance,
            spawning_threshold=inp.spawning_parameter, unoccupied_threshold=inp.unoccupied_threshold,
            minimum_unoccupied=int(inp.minimum_unoccupied), seed=0, device=device)
        if krylov_stop:
            self.tdvp.set_krylov_stop(krylov_stop)
        self.tdvp.dt = inp.dt
        self.mel = self.tdvp.mel()
        self.nnodes = m.topology.nnodes

    @property
    def t(self) -> float:
        return self.tdvp.t()

    def observables(self) -> List[float]:
        return [float(np.real(self.mel(op, 0, self.A))) for op in self.inp.ops]

    def hrank(self) -> np.ndarray:
        return self.A.hrank()[1:]

    def first_row(self) -> str:
        hr = self.hrank() if self.inp.print_bond_dimension else None
        return format_row(0.0, self.observables(), None, None, hr)

    def step(self) -> str:
        self.tdvp(self.A, coeff=-1j)
        hr = self.hrank() if self.inp.print_bond_dimension else None
        nh = self.tdvp.nh_applications() / float(self.nnodes)
        return format_row(self.t, self.observables(), self.tdvp.expansion_counts(), nh, hr)

    def last_line(self) -> str:
        return "nh_app: " + _g(self.tdvp.nh_applications() / float(self.nnodes)) + "\n"


def run(inp: DriverInput, out: TextIO, device: int = 0, max_steps: Optional[int] = None,
        model: Optional[DriverModel] = None, krylov_stop: int = 0) -> SpinBosonRun:
    """Step to tmax (or ``max_steps`` rows) writing the reference's columns to ``out``."""
    r = SpinBosonRun(inp, model, device, krylov_stop)
    out.write(r.first_row())
    n = 0
    while r.t < inp.tmax and (max_steps is None or n < max_steps):
        out.write(r.step())
        out.flush()
        n += 1
    out.write(r.last_line())
    return r


def check_discretisation(inp: DriverInput, wk: np.ndarray, gk: np.ndarray, out: TextIO, wmin: float, wmax: float,
                         nhist: int):
    """The ``check bath discretisation`` report (spin_boson.cpp:104-153): the modes, then
    a histogram of dw pi g_k^2 per bin against the spectral density (S + J at finite
    temperature)."""
    out.write("Discretised bath properties:\n")
    out.write("w_k g_k\n")
    for w, g in zip(wk, gk):
        out.write(f"( {w:g}, {g:g})\n")
    hist = np.zeros(nhist)
    dw = (wmax - wmin) / nhist
    for w, g in zip(wk, gk):
        if wmin <= w < wmax:
            hist[int((w - wmin) / dw)] += dw * g * g * math.pi
    out.write("Histogram: \n")
    out.write("w hist(w) S(w)\n")
    b = inp.bath
    for i in range(nhist):
        w = wmin + i * dw + dw / 2.0
        ref = float(b.S(w) + b.J(w)) if b.nonzero_temperature else float(b.J(w))
        out.write(f"{w:g} {hist[i]:g} {ref:g}\n")


def main(argv: Optional[Sequence[str]] = None) -> int:
    """``python -m ttns_lib_gb300.driver <input file> [--steps N] [--device D]
    [--output FILE]``: the reference's ``spin_boson <input filename>``."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m ttns_lib_gb300.driver")
    ap.add_argument("input")
    ap.add_argument("--steps", type=int, default=None, help="stop after this many rows")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--output", default=None, help="overrides the input's output file")
    ap.add_argument("--krylov-stop", default="full", choices=["full", "residual"],
                    help="how Krylov sub-steps end: the full space or, as the reference, the residual estimate")
    a = ap.parse_args(argv)
    try:
        with open(a.input) as f:
            doc = json.load(f)
        inp = parse_input(doc)
        wk, gk = bath_modes(inp)
        ofile = a.output if a.output is not None else inp.output_file
        out = open(ofile, "w") if ofile else sys.stdout
        try:
            if inp.check_bath_discretisation:
                d = _bath.normalise_keys(doc)
                lo, hi = frequency_window(inp)
                wmin = float(d.get("bathhistmin", lo))
                wmax = float(d.get("bathhistmax", hi))
                nhist = int(d.get("bathhistn", int(math.sqrt(inp.nmodes))))
                check_discretisation(inp, wk, gk, out, wmin, wmax, nhist)
                return 0
            blocks = make_blocks(inp, wk, gk)
            n = inp.hsys.shape[0]
            dims = [b.nstates for b in blocks]
            topo = driver_topology(n, dims, inp.nspf, inp.nspf_lower)
            model = DriverModel(inp, wk, gk, blocks, topo, capacity_tree(inp, dims, topo), build_hamiltonian(inp, blocks))
            sys.stdout.write(f"{len(blocks)}\n")
            run(inp, out, device=a.device, max_steps=a.steps, model=model,
                krylov_stop=1 if a.krylov_stop == "residual" else 0)
        finally:
            if out is not sys.stdout:
                out.close()
    except Exception as ex:  # the reference prints the message chain and returns 1
        sys.stderr.write(f"{ex}\n")
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
