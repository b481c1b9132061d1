"""Subspace expansion on the device (ttn_integrator_set_expansion) against the oracle's
restatement.  The expansion itself is deterministic: after the expanding preparation the
bond dimensions and every node tensor equal the oracle's (to rounding); during time steps
the bond dimensions grow at the same steps.  Trajectories are compared with exact dynamics
rather than with the oracle's: directions added by an expansion start exactly unoccupied,
which makes the following steps ill-conditioned in the sense of the product-state start
(rounding-level differences between two exponentials grow to ~1e-5), while both the
oracle and the device follow exp(-iHt) to < 1e-6 once the bonds reach full rank."""
import numpy as np
import pytest
import scipy.linalg as sla

from helpers import full_rank, generic_state
from oracle.oracle import Oracle
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb
from ttns_lib_gb300.model import SOPOperator, Topology, full_state

pytestmark = pytest.mark.gpu


def _model(chi):
    w, c = sb.ohmic_modes(4, 0.5, 5.0)
    return sb.build_from_modes(w, c, 3, chi, 0.3, 1.0)


def test_expanding_preparation_matches_oracle():
    m = _model(2)
    topo = m.topology
    cap = full_rank(_model(27).topology).hrank
    st = generic_state(topo, np.random.default_rng(4))
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-7)
    orc.expand_prepare(0.05)
    A = api.httensor(topo)
    A.set(st)
    integ = api.subspace_expansion_projector_splitting_integrator(A, m.sop, cap, krylov_dim=10, spawning_threshold=1e-7)
    integ.dt = 0.05
    integ.prepare(A)
    assert np.array_equal(A.hrank(), orc.hrank())
    for a, b in zip(A.get(), orc.get_state()):
        assert np.max(np.abs(a - b)) < 1e-12
    assert np.linalg.norm(full_state(A.current_topology(), A.get()) - full_state(topo, st)) < 1e-13


def test_expanding_steps_follow_exact_dynamics():
    m = _model(2)
    topo = m.topology
    cap = full_rank(_model(27).topology).hrank
    st = generic_state(topo, np.random.default_rng(4))
    psi = full_state(topo, st)
    H = m.sop.dense()
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-12)
    A = api.httensor(topo)
    A.set(st)
    integ = api.subspace_expansion_projector_splitting_integrator(A, m.sop, cap, krylov_dim=10, spawning_threshold=1e-12)
    integ.dt = 0.05
    prev = topo.hrank.copy()
    for k in range(20):
        integ(A, m.sop, -1j)
        orc.step(0.05)
        hr = A.hrank()
        assert np.all(hr >= prev) and np.all(hr <= cap)
        prev = hr
    ex = sla.expm(-1j * H * 20 * 0.05) @ psi
    assert np.array_equal(A.hrank(), cap) and np.array_equal(orc.hrank(), cap)
    assert np.linalg.norm(full_state(A.current_topology(), A.get()) - ex) < 1e-6
    assert np.linalg.norm(full_state(orc.current_topology(), orc.get_state()) - ex) < 1e-6


def test_random_fallback_matches_oracle():
    topo = Topology(np.array([-1, 0, 0, 0]), np.array([1, 3, 1, 3]), np.array([-1, 0, 1, 2]), np.array([0, 3, 3, 3]))
    rng = np.random.default_rng(2)
    H = SOPOperator(3, [3, 3, 3])
    for r in range(3):
        a = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        H.bind_dense(a + a.conj().T, [r], r)
    st = generic_state(topo, rng)
    cap = np.array([1, 3, 3, 3])
    orc = Oracle(topo, H, krylov_dim=8, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-12, minimum_unoccupied=2, seed=5)
    A = api.httensor(topo)
    A.set(st)
    integ = api.subspace_expansion_projector_splitting_integrator(A, H, cap, krylov_dim=8, spawning_threshold=1e-12,
                                                                  minimum_unoccupied=2, seed=5)
    integ.dt = 0.05
    for _ in range(2):
        integ(A, H, -1j)
        orc.step(0.05)
    assert np.array_equal(A.hrank(), orc.hrank())
    d = full_state(A.current_topology(), A.get()) - full_state(orc.current_topology(), orc.get_state())
    assert np.max(np.abs(d)) < 1e-10


def test_expansion_validates_its_arguments():
    m = _model(2)
    A = api.httensor(m.topology)
    A.set(generic_state(m.topology, np.random.default_rng(1)))
    integ = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8)
    bad = m.topology.hrank.copy()
    bad[3] -= 1
    with pytest.raises(api.TTNError):
        integ.set_expansion(A, bad)
    mixed = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8, precision=api.PREC_MIXED)
    with pytest.raises(api.TTNError):
        mixed.set_expansion(A, m.topology.hrank)


def test_large_two_site_matrices_on_the_device():
    """Bonds whose two-site matrix has both sides above 96 (here 144 x 144): the dominant
    directions are found on the device (Gram matrix, Lanczos and the other side's vectors
    by GEMM).  The bond dimensions equal the oracle's, the state is unchanged and every
    non-root node stays an isometry (inside near-degenerate clusters of singular values
    the two may pick different directions at rounding level)."""
    from helpers import random_sop
    topo = Topology(np.array([-1, 0, 1, 1, 0, 0]), np.array([1, 4, 12, 12, 12, 12]), np.array([-1, -1, 0, 1, 2, 3]),
                    np.array([0, 0, 12, 12, 12, 12]))
    rng = np.random.default_rng(9)
    H = random_sop(rng, [12] * 4, nterms=8)
    st = generic_state(topo, rng)
    cap = np.array([1, 40, 12, 12, 12, 12])
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_expansion(cap, spawning_threshold=1e-7)
    orc.expand_prepare(0.05)
    A = api.httensor(topo)
    A.set(st)
    integ = api.subspace_expansion_projector_splitting_integrator(A, H, cap, krylov_dim=10, spawning_threshold=1e-7)
    integ.dt = 0.05
    integ.prepare(A)
    assert np.array_equal(A.hrank(), orc.hrank()) and A.hrank()[1] > 4
    assert np.linalg.norm(full_state(A.current_topology(), A.get()) - full_state(topo, st)) < 1e-12
    assert max(np.max(np.abs(a.conj().T @ a - np.eye(a.shape[1]))) for a in A.get()[1:]) < 1e-12
