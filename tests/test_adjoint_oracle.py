"""The adjoint sweep of the oracle (oracle/ttn_adjoint.hpp) against central finite
differences: J = sum_t w_t Re <O>(t) over integrator steps (the first one sub-stepped),
gradients with respect to the spin-boson parameters (bias, tunnelling, every bath
coupling and frequency), every SOP coefficient, every operator matrix and the state.
Random trees carry shared operators, duplicate and identity-only terms, so that every
term-group kind of the compressed operator (S, M, singletons, root mean fields) is
differentiated.  Starting states are generic (every bond populated): from a product
state the gauge factors are singular and the sweep is not differentiable."""
import copy

import numpy as np
import pytest

from helpers import generic_state, rand_herm, random_sop, random_tree
from oracle.oracle import Oracle
from ttns_lib_gb300 import spin_boson as sb

H_FD = 1e-5   # central differences; the Krylov tolerance keeps their noise near 1e-9


def _adjoint(topo, sop, st, dt, weights, mode, op, ckpt=2, **kw):
    o = Oracle(topo, sop, krylov_dim=10, krylov_tol=1e-14)
    o.set_state(st)
    return o.adjoint(dt, len(weights), weights, mode, op, checkpoint_every=ckpt, **kw)


def test_spin_boson_parameter_gradients_match_finite_differences():
    """The c5-shaped objective (zero-temperature spin-boson, J = sum_t w_t <sz>(t), w_t
    uniform in [0, 1]) on a small bath: dJ/d(eps, Delta, c_k, w_k) within 1e-5 relative."""
    N, d, chi, nsteps, dt = 4, 3, 3, 4, 0.05
    w0, c0 = sb.ohmic_modes(N, 0.4, 5.0)
    eps0, del0 = 0.3, 1.0
    base = sb.build_from_modes(w0, c0, d, chi, eps0, del0)
    rng = np.random.default_rng(5)
    st = generic_state(base.topology, rng)
    wt = rng.uniform(size=nsteps)

    def J(model):
        return _adjoint(model.topology, model.sop, st, dt, wt, 0, sb.SZ)[0]

    _, _, gops = _adjoint(base.topology, base.sop, st, dt, wt, 0, sb.SZ)
    g = sb.parameter_gradient(base, gops)
    adj, fd = [], []

    def central(make):
        return (J(make(H_FD)) - J(make(-H_FD))) / (2 * H_FD)

    adj.append(g["eps"]); fd.append(central(lambda e: sb.build_from_modes(w0, c0, d, chi, eps0 + e, del0)))
    adj.append(g["delta"]); fd.append(central(lambda e: sb.build_from_modes(w0, c0, d, chi, eps0, del0 + e)))
    for k in range(N):
        def fc(e, k=k):
            c = c0.copy(); c[k] += e
            return sb.build_from_modes(w0, c, d, chi, eps0, del0)

        def fw(e, k=k):
            w = w0.copy(); w[k] += e
            return sb.build_from_modes(w, c0, d, chi, eps0, del0)
        adj.append(g["coupling"][k]); fd.append(central(fc))
        adj.append(g["omega"][k]); fd.append(central(fw))
    adj, fd = np.array(adj), np.array(fd)
    assert np.linalg.norm(adj - fd) <= 1e-5 * np.linalg.norm(fd)
    assert np.max(np.abs(adj - fd)) <= 1e-5 * np.max(np.abs(fd))


@pytest.mark.parametrize("seed,chi", [(0, None), (1, 2)])
def test_random_sop_coefficient_and_operator_gradients(seed, chi):
    rng = np.random.default_rng(200 + seed)
    dims = [int(x) for x in rng.integers(2, 4, size=5)]
    topo = random_tree(rng, dims, chi=chi)
    H = random_sop(rng, dims, nterms=10)
    st = generic_state(topo, rng)
    wt = rng.uniform(size=3)
    O = rand_herm(rng, dims[0])
    _, gc, gops = _adjoint(topo, H, st, 0.1, wt, 0, O)

    def J(Hs):
        return _adjoint(topo, Hs, st, 0.1, wt, 0, O)[0]

    adj, fd = [], []
    for r in range(H.nterms):
        Hp, Hm = copy.deepcopy(H), copy.deepcopy(H)
        Hp.coeffs[r] += H_FD
        Hm.coeffs[r] -= H_FD
        adj.append(gc[r]); fd.append((J(Hp) - J(Hm)) / (2 * H_FD))
    for k in range(len(H.ops)):
        B = rand_herm(rng, H.ops[k].matrix.shape[0])
        Hp, Hm = copy.deepcopy(H), copy.deepcopy(H)
        Hp.ops[k].matrix = H.ops[k].matrix + H_FD * B
        Hm.ops[k].matrix = H.ops[k].matrix - H_FD * B
        adj.append(float(np.real(np.sum(np.conj(gops[k]) * B)))); fd.append((J(Hp) - J(Hm)) / (2 * H_FD))
    adj, fd = np.array(adj), np.array(fd)
    assert np.max(np.abs(adj - fd)) <= 1e-6 * np.max(np.abs(fd))


def test_state_cotangent_and_checkpoint_independence():
    """The cotangent of the starting state against a directional difference, and the
    gradients independent of the checkpoint interval (K = 1, 2, all steps)."""
    m = sb.build(N=3, alpha=0.4, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    topo = m.topology
    rng = np.random.default_rng(9)
    st = generic_state(topo, rng)
    wt = rng.uniform(size=3)
    outs = [_adjoint(topo, m.sop, st, 0.05, wt, 0, sb.SZ, ckpt=k, skip_prepare=True, state_cotangent=True)
            for k in (1, 2, 3)]
    for o in outs[1:]:
        assert o[0] == outs[0][0]
        assert np.array_equal(o[1], outs[0][1])
        assert all(np.array_equal(a, b) for a, b in zip(o[2], outs[0][2]))
        assert np.array_equal(o[3], outs[0][3])
    delta = [rng.normal(size=a.shape) + 1j * rng.normal(size=a.shape) for a in st]
    h = 1e-6
    Jp = _adjoint(topo, m.sop, [a + h * b for a, b in zip(st, delta)], 0.05, wt, 0, sb.SZ, skip_prepare=True)[0]
    Jm = _adjoint(topo, m.sop, [a - h * b for a, b in zip(st, delta)], 0.05, wt, 0, sb.SZ, skip_prepare=True)[0]
    fd = (Jp - Jm) / (2 * h)
    ad = float(np.real(np.vdot(outs[0][3], np.concatenate([b.ravel() for b in delta]))))
    assert abs(fd - ad) <= 1e-7 * abs(fd)


def test_adjoint_objective_equals_plain_steps():
    """The adjoint's forward pass is the integrator's own trajectory."""
    m = sb.build(N=3, alpha=0.4, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    topo = m.topology
    rng = np.random.default_rng(11)
    st = generic_state(topo, rng)
    wt = rng.uniform(size=3)
    J = _adjoint(topo, m.sop, st, 0.05, wt, 0, sb.SZ)[0]
    o = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-14)
    o.set_state(st)
    ref = 0.0
    for k in range(3):
        o.step(0.05)
        ref += wt[k] * o.expect(0, sb.SZ).real
    assert J == ref


def test_torch_objective_wrapper_returns_the_adjoint_gradient():
    """The torch.autograd.Function wrapper (a check harness) around an adjoint evaluator:
    autograd returns the adjoint gradient, which matches central differences of J."""
    torch = pytest.importorskip("torch")
    from ttns_lib_gb300 import api
    N, d, chi, dt = 3, 3, 3, 0.05
    w0, c0 = sb.ohmic_modes(N, 0.4, 5.0)
    rng = np.random.default_rng(21)
    topo = sb.build_from_modes(w0, c0, d, chi, 0.3, 1.0).topology
    st = generic_state(topo, rng)
    wt = rng.uniform(size=2)

    def evaluate(theta):
        m = sb.build_from_modes(w0, theta[2:], d, chi, theta[0], theta[1])
        J, _, gops = _adjoint(topo, m.sop, st, dt, wt, 0, sb.SZ)
        g = sb.parameter_gradient(m, gops)
        return J, np.concatenate([[g["eps"], g["delta"]], g["coupling"]])

    f = api.torch_objective(evaluate)
    theta = torch.tensor(np.concatenate([[0.3, 1.0], c0]), dtype=torch.float64, requires_grad=True)
    J = f(theta)
    (grad,) = torch.autograd.grad(J, theta)
    th = theta.detach().numpy()
    fd = np.zeros_like(th)
    for i in range(th.size):
        e = np.zeros_like(th); e[i] = H_FD
        fd[i] = (evaluate(th + e)[0] - evaluate(th - e)[0]) / (2 * H_FD)
    assert np.max(np.abs(grad.numpy() - fd)) <= 1e-5 * np.max(np.abs(fd))
