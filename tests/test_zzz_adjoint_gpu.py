"""The adjoint sweep on the device (ttn_adjoint_grad) against the oracle's adjoint sweep
on the same inputs: the objective J = sum_t w_t Re <O>(t), dJ/dc_r for every term
coefficient, the cotangent of every operator matrix and of the state.  The oracle's
adjoint is itself checked against central finite differences
(tests/test_adjoint_oracle.py).  Both differentiate the same discrete sweep; they differ
by rounding, by the Krylov step control of the two exponentials (agreeing to ~1e-11 in
the trajectories) and by converged quadratures, so the gradients agree to 1e-8 of the
largest component."""
import numpy as np
import pytest

from helpers import generic_state, rand_herm, random_sop, random_tree
from oracle.oracle import Oracle
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

pytestmark = pytest.mark.gpu

TOL = 1e-8


def _compare(topo, H, st, dt, wt, mode, O, ckpt):
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    Jo, gco, gopo, gso = orc.adjoint(dt, len(wt), wt, mode, O, checkpoint_every=ckpt, state_cotangent=True)
    A = api.httensor(topo, device=0)
    A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10, krylov_tolerance=1e-12)
    Jd, gcd, gopd, gsd = integ.adjoint(A, dt, len(wt), wt, mode, O, checkpoint_every=ckpt, state_cotangent=True)
    assert abs(Jd - Jo) <= 1e-10 * max(1.0, abs(Jo))
    scale = max(np.max(np.abs(gco)), max(np.max(np.abs(g)) for g in gopo))
    assert np.max(np.abs(gcd - gco)) <= TOL * scale
    for a, b in zip(gopd, gopo):
        assert np.max(np.abs(a - b)) <= TOL * scale
    gso_flat = np.asarray(gso)
    gsd_flat = np.concatenate([g.ravel() for g in gsd])
    assert np.max(np.abs(gsd_flat - gso_flat)) <= TOL * np.max(np.abs(gso_flat))
    # the state is left at the end of the trajectory, as the oracle's
    fin = np.concatenate([a.ravel() for a in A.get()])
    ref = np.concatenate([a.ravel() for a in orc.get_state()])
    assert np.max(np.abs(fin - ref)) <= 1e-9


def test_device_adjoint_matches_oracle_spin_boson():
    m = sb.build(N=4, alpha=0.4, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    rng = np.random.default_rng(5)
    st = generic_state(m.topology, rng)
    wt = rng.uniform(size=3)
    _compare(m.topology, m.sop, st, 0.05, wt, 0, sb.SZ, ckpt=2)


def test_device_adjoint_matches_oracle_random_operator():
    rng = np.random.default_rng(201)
    dims = [int(x) for x in rng.integers(2, 4, size=5)]
    topo = random_tree(rng, dims, chi=2)
    H = random_sop(rng, dims, nterms=10)
    st = generic_state(topo, rng)
    wt = rng.uniform(size=2)
    _compare(topo, H, st, 0.1, wt, 0, rand_herm(rng, dims[0]), ckpt=1)


def test_device_adjoint_rejects_mixed_precision_and_used_integrators():
    m = sb.build(N=2, alpha=0.4, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    rng = np.random.default_rng(1)
    st = generic_state(m.topology, rng)
    A = api.httensor(m.topology, device=0)
    A.set(st)
    mixed = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8, precision=api.PREC_MIXED)
    with pytest.raises(api.TTNError):
        mixed.adjoint(A, 0.05, 1, [1.0], 0, sb.SZ)
    plain = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8)
    plain.dt = 0.05
    plain(A)
    with pytest.raises(api.TTNError):
        plain.adjoint(A, 0.05, 1, [1.0], 0, sb.SZ)


def test_device_adjoint_through_torch_matches_plain_path_differences():
    """dJ/d(eps, Delta, c_k) from the device adjoint through the torch.autograd wrapper
    against central differences of J computed by the plain FP64 device path
    (ttn_integrator_step and <sz> after every step), within 1e-5 relative."""
    torch = pytest.importorskip("torch")
    N, d, chi, dt, h = 3, 3, 3, 0.05, 1e-4
    w0, c0 = sb.ohmic_modes(N, 0.4, 5.0)
    rng = np.random.default_rng(21)
    topo = sb.build_from_modes(w0, c0, d, chi, 0.3, 1.0).topology
    st = generic_state(topo, rng)
    wt = rng.uniform(size=3)
    f = api.torch_objective(api.spin_boson_adjoint(w0, d, chi, st, dt, wt, krylov_dim=10, krylov_tolerance=1e-12,
                                                   checkpoint_every=2))
    theta = torch.tensor(np.concatenate([[0.3, 1.0], c0]), dtype=torch.float64, requires_grad=True)
    (grad,) = torch.autograd.grad(f(theta), theta)

    def plain_J(th):
        m = sb.build_from_modes(w0, th[2:], d, chi, th[0], th[1])
        A = api.httensor(topo, device=0)
        A.set(st)
        integ = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=10, krylov_tolerance=1e-12)
        integ.dt = dt
        J = 0.0
        for k in range(len(wt)):
            integ(A, m.sop, -1j)
            J += wt[k] * integ.mel()(sb.SZ, 0, A).real
        return J

    th = theta.detach().numpy()
    fd = np.zeros_like(th)
    for i in range(th.size):
        e = np.zeros_like(th)
        e[i] = h
        fd[i] = (plain_J(th + e) - plain_J(th - e)) / (2 * h)
    assert np.max(np.abs(grad.numpy() - fd)) <= 1e-5 * np.max(np.abs(fd))


def test_device_adjoint_at_the_adjoint_workload_shapes():
    """The adjoint workload's model (zero temperature, N = 128 modes, alpha = 0.4, wc = 5,
    d = 12, chi = 24, dt = 0.05) over its first 4 steps from a generic state, with a
    checkpoint every 2 steps: dJ/deps and dJ/dDelta from the device adjoint against central
    differences (h = 1e-6) of the plain FP64 device path, within 1e-5 of the larger
    difference quotient (a run of 6 steps with three coupling derivatives as well passed the
    same check in 8 minutes; this keeps the suite's time)."""
    m, cfg = sb.build_config("c5")
    topo = m.topology
    rng = np.random.default_rng(55)
    st = generic_state(topo, rng)
    wt = rng.uniform(size=4)
    theta = np.concatenate([[m.eps, m.delta], m.coupling])
    J, grad = api.spin_boson_adjoint(m.omega, cfg["d"], cfg["chi"], st, cfg["dt"], wt, krylov_dim=cfg["krylov_dim"],
                                     krylov_tolerance=1e-12, checkpoint_every=2)(theta)

    def plain_J(th):
        mm = sb.build_from_modes(m.omega, th[2:], cfg["d"], cfg["chi"], th[0], th[1])
        A = api.httensor(topo, device=0)
        A.set(st)
        integ = api.fixed_step_projector_splitting_integrator(A, mm.sop, krylov_dim=cfg["krylov_dim"],
                                                             krylov_tolerance=1e-12)
        integ.dt = cfg["dt"]
        out = 0.0
        for k in range(len(wt)):
            integ(A, mm.sop, -1j)
            out += wt[k] * integ.mel()(sb.SZ, 0, A).real
        return out

    assert abs(plain_J(theta) - J) <= 1e-10 * max(1.0, abs(J))
    h = 1e-6
    idx = [0, 1]
    fd = []
    for i in idx:
        e = np.zeros_like(theta)
        e[i] = h
        fd.append((plain_J(theta + e) - plain_J(theta - e)) / (2 * h))
    fd = np.array(fd)
    assert np.max(np.abs(grad[idx] - fd)) <= 1e-5 * np.max(np.abs(fd)), (grad[idx], fd)
