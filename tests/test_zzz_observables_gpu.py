"""General observables of the boundary (matrix_element's overloads) on the device against
dense contractions of the full state vectors: <bra|ket>, <bra|O_a O_b|ket> for a product of
one-mode operators, and <bra|H|ket> of a sum-of-product operator; bra = ket included."""
import numpy as np
import pytest

from helpers import generic_state, rand_herm
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb
from ttns_lib_gb300.model import full_state

pytestmark = pytest.mark.gpu


def _kron_ops(dims, ops_by_mode):
    M = np.array([[1.0 + 0j]])
    for m, d in enumerate(dims):
        M = np.kron(M, ops_by_mode.get(m, np.eye(d)))
    return M


def test_overlap_product_and_sop_expectations_match_dense():
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    topo = m.topology
    rng = np.random.default_rng(13)
    sa, sb_ = generic_state(topo, rng), generic_state(topo, rng)
    A, B = api.httensor(topo), api.httensor(topo)
    A.set(sa)
    B.set(sb_)
    integ = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8)
    mel = integ.mel()
    fa, fb = full_state(topo, sa), full_state(topo, sb_)
    assert abs(mel.overlap(A, B) - np.vdot(fa, fb)) < 1e-12
    assert abs(mel.overlap(B, B) - np.vdot(fb, fb)) < 1e-12
    dims = topo.mode_dims()
    ops = {0: sb.SZ, 2: rand_herm(rng, dims[2]), 3: rand_herm(rng, dims[3])}
    ref = np.vdot(fa, _kron_ops(dims, ops) @ fb)
    assert abs(mel.product(ops, A, B) - ref) < 1e-12
    ref_self = np.vdot(fa, _kron_ops(dims, ops) @ fa)
    assert abs(mel.product(ops, A) - ref_self) < 1e-12
    H = m.sop.dense()
    assert abs(mel.sop(m.sop, A, B) - np.vdot(fa, H @ fb)) < 1e-11
    assert abs(mel.sop(m.sop, A) - np.vdot(fa, H @ fa)) < 1e-11


def test_orthogonaliser_on_the_device():
    """orthogonaliser(A) for an arbitrary (non-orthogonal) state: the state is unchanged,
    every non-root node becomes an isometry, the tensors equal the oracle's (same
    Householder gauge), and stepping afterwards follows the oracle."""
    from oracle.oracle import Oracle
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    topo = m.topology
    rng = np.random.default_rng(21)
    st = [rng.normal(size=t.shape) + 1j * rng.normal(size=t.shape) for t in generic_state(topo, rng)]
    st[0] = st[0] / np.linalg.norm(full_state(topo, st))
    psi = full_state(topo, st)
    A = api.httensor(topo)
    A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=10, krylov_tolerance=1e-13)
    integ.orthogonalise(A)
    got = A.get()
    assert np.linalg.norm(full_state(topo, got) - psi) < 1e-12 * np.linalg.norm(psi)
    for t in got[1:]:
        assert np.max(np.abs(t.conj().T @ t - np.eye(t.shape[1]))) < 1e-13
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-13)
    orc.set_state(st)
    orc.orthogonalise()
    assert max(np.max(np.abs(a - b)) for a, b in zip(got, orc.get_state())) < 1e-12
    integ.dt = 0.05
    for _ in range(3):
        integ(A)
        orc.step(0.05)
    assert max(np.max(np.abs(a - b)) for a, b in zip(A.get(), orc.get_state())) < 1e-10
