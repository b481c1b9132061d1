"""The oracle pinned by known answers: dense exp(-iHt) on full-rank trees, the
uncoupled spin, conservation laws and the Householder conventions."""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import generic_state, random_case, random_sop, random_tree
from oracle.oracle import Oracle, qr
from ttns_lib_gb300 import spin_boson as sb
from ttns_lib_gb300.model import full_state


def test_full_rank_spin_boson_matches_dense_expm():
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=9, eps=0.3, delta=1.0)
    topo = m.topology
    st = sb.initial_state_numpy(topo, seed=1, psi0=np.array([1, 0]))
    psi = full_state(topo, st)
    H = m.sop.dense()
    orc = Oracle(topo, m.sop, krylov_dim=12, krylov_tol=1e-12)
    orc.set_state(st)
    dt = 0.05
    for k in range(12):
        orc.step(dt)
        ex = sla.expm(-1j * H * (k + 1) * dt) @ psi
        got = full_state(topo, orc.get_state())
        assert np.linalg.norm(got - ex) < 1e-11


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_tree_random_sop_matches_dense_expm(seed):
    rng = np.random.default_rng(100 + seed)
    dims = [int(x) for x in rng.integers(2, 4, size=5)]
    topo = random_tree(rng, dims)
    H = random_sop(rng, dims, nterms=10)
    st = generic_state(topo, rng)
    psi = full_state(topo, st)
    Hd = H.dense()
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    for k in range(5):
        orc.step(0.1)
        ex = sla.expm(-1j * Hd * (k + 1) * 0.1) @ psi
        got = full_state(topo, orc.get_state())
        assert np.linalg.norm(got - ex) < 1e-10


# random operator shapes, among them groups that mix terms acting below a node with terms
# that are the identity there (at a leaf: 310; at a branch node: 312, 338)
@pytest.mark.parametrize("seed", [300, 304, 310, 312, 320, 338])
def test_random_operator_shapes_match_dense_expm(seed):
    topo, H, st, _ = random_case(seed)
    psi = full_state(topo, st)
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    for k in range(3):
        orc.step(0.1)
        ex = sla.expm(-1j * H.dense() * (k + 1) * 0.1) @ psi
        assert np.linalg.norm(full_state(topo, orc.get_state()) - ex) < 1e-10


def test_uncoupled_spin_precesses():
    m = sb.build(N=4, alpha=0.0, wc=5.0, d=4, chi=4, eps=0.0, delta=1.0)
    orc = Oracle(m.topology, m.sop, krylov_dim=8)
    orc.set_state(sb.initial_state_numpy(m.topology, seed=0, psi0=np.array([1, 0])))
    for k in range(20):
        orc.step(0.05)
        t = (k + 1) * 0.05
        assert abs(orc.expect(0, sb.SZ).real - np.cos(t)) < 1e-11


def test_norm_and_energy_conserved_truncated():
    m, cfg = sb.build_config("c1")
    orc = Oracle(m.topology, m.sop, krylov_dim=cfg["krylov_dim"])
    st = sb.initial_state_numpy(m.topology, seed=0, psi0=np.array([1, 0]))
    orc.set_state(st)
    for _ in range(5):
        orc.step(cfg["dt"])
        assert abs(orc.norm2() - 1.0) < 1e-11


def test_householder_conventions():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(9, 4)) + 1j * rng.normal(size=(9, 4))
    q, r = qr(a)
    assert np.allclose(q @ r, a, atol=1e-13)
    assert np.allclose(q.conj().T @ q, np.eye(4), atol=1e-13)
    assert np.allclose(np.tril(r, -1), 0)
    # exact zeros give tau = 0: Q columns are unit vectors, R keeps alpha
    z = np.zeros((6, 3), dtype=np.complex128)
    z[0, 0] = 1.0
    q, r = qr(z)
    assert np.array_equal(q, np.eye(6, 3))
    assert r[0, 0] == 1.0


def test_householder_tiny_columns_stay_finite():
    rng = np.random.default_rng(5)
    a = (rng.normal(size=(50, 6)) + 1j * rng.normal(size=(50, 6))) * 1e-170
    a[:, 0] *= 1e-140  # below the LAPACK safe minimum: exercises the rescaling loop
    q, r = qr(a)
    assert np.isfinite(q).all() and np.isfinite(r).all()
    assert np.allclose(q.conj().T @ q, np.eye(6), atol=1e-13)
    assert np.allclose(q @ r, a, rtol=0, atol=1e-13 * np.abs(a).max())

def test_oracle_matches_golden_trajectory():
    """The committed dense-expm trajectory (tests/golden/make_golden.py): full-rank tree,
    so the sweep is exact; 40 steps including the first-step sub-steps."""
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "spin_boson_fullrank_N4.json")))
    m = sb.build(**g["params"])
    orc = Oracle(m.topology, m.sop, krylov_dim=12, krylov_tol=1e-12)
    orc.set_state(sb.initial_state_numpy(m.topology, seed=g["seed"], psi0=np.array([1.0, 0.0])))
    for k in range(g["steps"]):
        orc.step(g["dt"])
        assert abs(orc.expect(0, sb.SZ).real - g["sz"][k]) < 1e-11, k
        assert abs(orc.expect(0, sb.SX).real - g["sx"][k]) < 1e-11, k
        assert abs(orc.norm2() - g["norm"][k]) < 1e-11, k


def test_time_dependent_operators_converge_to_driven_dynamics():
    """A driven spin-boson model (bias eps(t) = eps0 + A cos(W t) through the primitive
    operators' update hook, full-rank tree): the sweep converges at second order in dt to
    the time-ordered propagation of the dense Hamiltonian."""
    from helpers import full_rank
    w, c = sb.ohmic_modes(2, 0.5, 5.0)
    m = sb.build_from_modes(w, c, 3, 9, 0.3, 1.0)
    topo = full_rank(m.topology)
    eps0, amp, om, delta = 0.3, 0.8, 3.0, 1.0

    def sysop(t):
        return 0.5 * (eps0 + amp * np.cos(om * t)) * sb.SZ + 0.5 * delta * sb.SX

    def update(mode, op, t, dt, mat):
        if op == 0:
            mat[:] = sysop(t + dt / 2)

    st = generic_state(topo, np.random.default_rng(1))
    psi = full_state(topo, st)
    H0 = m.sop.dense()
    static = np.kron(0.5 * eps0 * sb.SZ + 0.5 * delta * sb.SX, np.eye(H0.shape[0] // 2))
    x = psi.copy()
    nf = 2000
    for k in range(nf):
        t = (k + 0.5) / nf
        x = sla.expm(-1j * (H0 - static + np.kron(sysop(t), np.eye(H0.shape[0] // 2))) / nf) @ x
    errs = []
    for dt in (0.02, 0.01):
        orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
        orc.set_state(st)
        orc.set_op_update(update)
        for _ in range(int(round(1.0 / dt))):
            orc.step(dt)
        errs.append(np.linalg.norm(full_state(topo, orc.get_state()) - x))
    assert errs[1] < 1e-6
    assert 3.0 < errs[0] / errs[1] < 5.0


def test_orthogonaliser_keeps_the_state_and_makes_isometries():
    """orthogonaliser (include/ttns_lib/decompositions/orthogonaliser.hpp:83-112) on an
    arbitrary state of a random tree: the full state vector is unchanged, every non-root
    node is an isometry, and a full-rank tree then follows exp(-iHt)."""
    from helpers import full_rank, generic_state, random_sop, random_tree
    from ttns_lib_gb300.model import full_state
    import scipy.linalg as sla
    rng = np.random.default_rng(31)
    topo = full_rank(random_tree(rng, [2, 3, 2, 2], max_children=3))
    H = random_sop(rng, topo.mode_dims())
    st = [rng.normal(size=t.shape) + 1j * rng.normal(size=t.shape) for t in generic_state(topo, rng)]
    psi = full_state(topo, st)
    orc = Oracle(topo, H, krylov_dim=12, krylov_tol=1e-13)
    orc.set_state(st)
    orc.orthogonalise()
    got = orc.get_state()
    assert np.linalg.norm(full_state(topo, got) - psi) < 1e-13 * np.linalg.norm(psi)
    for t in got[1:]:
        assert np.max(np.abs(t.conj().T @ t - np.eye(t.shape[1]))) < 1e-14
    for _ in range(4):
        orc.step(0.05)
    ex = sla.expm(-1j * H.dense() * 0.2) @ psi
    assert np.linalg.norm(full_state(topo, orc.get_state()) - ex) < 1e-9 * np.linalg.norm(psi)
