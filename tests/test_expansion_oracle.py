"""Subspace expansion (adaptive bond dimension) of the oracle (oracle/ttn_expansion.hpp),
restating the reference's subspace_expansion_projector_splitting_engine, pinned by known
answers: an expansion changes the state's representation but not the state; with every
bond free to grow to full rank the expanding integrator follows exact dynamics
exp(-iHt) while the fixed-rank one does not; nothing grows when the spawning threshold
cannot be met; capacities are respected; the random one-site fallback adds orthonormal
unoccupied functions where the two-site search has no direction."""
import numpy as np
import pytest
import scipy.linalg as sla

from helpers import full_rank, generic_state
from oracle.oracle import Oracle
from ttns_lib_gb300 import spin_boson as sb
from ttns_lib_gb300.model import Topology, full_state


def _model(chi):
    w, c = sb.ohmic_modes(4, 0.5, 5.0)
    return sb.build_from_modes(w, c, 3, chi, 0.3, 1.0)


def _isometries(orc):
    st = orc.get_state()
    return max(np.max(np.abs(a.conj().T @ a - np.eye(a.shape[1]))) for a in st[1:])


def test_expansion_changes_the_representation_not_the_state():
    m = _model(2)
    topo = m.topology
    cap = full_rank(_model(27).topology).hrank
    st = generic_state(topo, np.random.default_rng(4))
    psi = full_state(topo, st)
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-12)
    assert orc.expand_prepare(0.05)
    hr = orc.hrank()
    assert np.all(hr >= topo.hrank) and np.any(hr > topo.hrank) and np.all(hr <= cap)
    assert np.linalg.norm(full_state(orc.current_topology(), orc.get_state()) - psi) < 1e-13
    assert _isometries(orc) < 1e-13


def test_expanding_integrator_follows_exact_dynamics():
    m = _model(2)
    topo = m.topology
    cap = full_rank(_model(27).topology).hrank
    st = generic_state(topo, np.random.default_rng(4))
    psi = full_state(topo, st)
    H = m.sop.dense()
    errs = {}
    for expand in (False, True):
        orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
        orc.set_state(st)
        if expand:
            orc.set_expansion(cap, spawning_threshold=1e-12)
        for k in range(20):
            orc.step(0.05)
        ex = sla.expm(-1j * H * 20 * 0.05) @ psi
        errs[expand] = np.linalg.norm(full_state(orc.current_topology(), orc.get_state()) - ex)
        if expand:
            assert np.array_equal(orc.hrank(), cap)
    assert errs[False] > 0.1
    assert errs[True] < 1e-6


def test_nothing_grows_below_the_spawning_threshold():
    m = _model(2)
    topo = m.topology
    cap = full_rank(_model(27).topology).hrank
    st = generic_state(topo, np.random.default_rng(6))
    a = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    b = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    a.set_state(st)
    b.set_state(st)
    b.set_expansion(cap, spawning_threshold=1e300, minimum_unoccupied=0)
    for _ in range(3):
        a.step(0.05)
        b.step(0.05)
    assert np.array_equal(b.hrank(), topo.hrank)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)


def test_capacity_bounds_the_growth():
    m = _model(2)
    topo = m.topology
    cap = np.minimum(full_rank(_model(27).topology).hrank, topo.hrank + 1)
    st = generic_state(topo, np.random.default_rng(7))
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-12)
    for _ in range(5):
        orc.step(0.05)
        hr = orc.hrank()
        assert np.all(hr <= cap) and np.all(hr >= topo.hrank)
    assert np.array_equal(orc.hrank(), cap)


def test_random_fallback_adds_orthonormal_unoccupied_functions():
    """A leaf of rank 1 between wider siblings: no two-site direction exists (rank 1), so
    with a minimum number of unoccupied functions random orthonormal ones are added."""
    topo = Topology(np.array([-1, 0, 0, 0]), np.array([1, 3, 1, 3]), np.array([-1, 0, 1, 2]), np.array([0, 3, 3, 3]))
    from ttns_lib_gb300.model import SOPOperator
    rng = np.random.default_rng(2)
    H = SOPOperator(3, [3, 3, 3])
    for r in range(3):
        a = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        H.bind_dense(a + a.conj().T, [r], r)
    st = generic_state(topo, rng)
    psi = full_state(topo, st)
    orc = Oracle(topo, H, krylov_dim=8, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(np.array([1, 3, 3, 3]), spawning_threshold=1e-12, minimum_unoccupied=2, seed=5)
    assert orc.expand_prepare(0.05)
    assert orc.hrank()[2] == 3
    assert np.linalg.norm(full_state(orc.current_topology(), orc.get_state()) - psi) < 1e-13
    assert _isometries(orc) < 1e-13


@pytest.mark.parametrize("g", [40, 150, 300])
def test_dominant_eigenpairs_dense_and_lanczos(g):
    """The top eigenpairs used to pick expansion directions: dense Jacobi for small Gram
    matrices, Lanczos for large ones (g > 96), both against numpy."""
    from oracle.oracle import top_eig
    rng = np.random.default_rng(g)
    M = rng.normal(size=(g, 60)) + 1j * rng.normal(size=(g, 60))
    M[:, 0] *= 20.0
    M[:, 1] *= 10.0
    G = M @ M.conj().T
    vals, vecs = top_eig(G, 2)
    ref_w, ref_v = np.linalg.eigh(G)
    assert np.allclose(vals, ref_w[::-1][:2], rtol=1e-10)
    for j in range(2):
        r = ref_v[:, -1 - j]
        assert abs(abs(np.vdot(r, vecs[j])) - 1.0) < 1e-8
