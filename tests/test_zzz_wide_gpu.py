"""Bonds wider than 64 (64 < n <= 256), which subspace expansion grows: the gauge moves'
QR kernels in their wide instantiations (ttns_lib_gb300/csrc/ttn_qr_rows.cu with the rows in
shared memory; ttn_qr.cu, rows in global memory, for matrices too tall for that) against the
oracle's Householder QR (the same LAPACK conventions, so the same gauge), and a sweep over a
tree whose bonds are 70 wide against the oracle.  No library QR is involved."""
import numpy as np
import pytest

from helpers import generic_state, random_sop
from oracle.oracle import Oracle, qr
from ttns_lib_gb300 import api
from ttns_lib_gb300.model import Topology

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n", [(300, 96), (160, 160), (2000, 256), (12000, 200)])
def test_wide_qr_matches_the_oracle(m, n):
    rng = np.random.default_rng(m + n)
    a = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
    a[:, 3] = 0.0  # an exactly zero column: tau = 0 and a deterministic completion of Q
    q, r = api.device_qr(a)
    qo, ro = qr(a)
    assert np.max(np.abs(r - ro)) < 1e-11 * np.max(np.abs(ro))
    assert np.max(np.abs(q - qo)) < 1e-10
    assert np.max(np.abs(q.conj().T @ q - np.eye(n))) < 1e-12
    assert np.max(np.abs(q @ r - a)) < 1e-12 * np.max(np.abs(a))
    assert np.all(np.abs(np.imag(np.diag(r))) == 0.0)


def test_sweep_with_bonds_wider_than_64_matches_the_oracle():
    topo = Topology(np.array([-1, 0, 1, 1, 0]), np.array([1, 70, 9, 9, 70]), np.array([-1, -1, 0, 1, 2]),
                    np.array([0, 0, 9, 9, 70]))
    rng = np.random.default_rng(41)
    H = random_sop(rng, topo.mode_dims(), nterms=6)
    st = generic_state(topo, rng)
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    A = api.httensor(topo)
    A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10)
    integ.dt = 0.05
    for _ in range(3):
        integ(A)
        orc.step(0.05)
    assert max(np.max(np.abs(a - b)) for a, b in zip(A.get(), orc.get_state())) < 1e-9
    with pytest.raises(api.TTNError):
        api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10, precision=api.PREC_MIXED)
