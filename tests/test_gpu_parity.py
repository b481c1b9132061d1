"""Device path vs the CPU oracle on the same inputs (GB300 only).

Tolerances: the plain form is complex128 throughout, so kernel-level results agree to
rounding (relative 1e-12) and sweeps from well-conditioned states agree to 1e-10.
Runs that start from the rank-1 product state are compared against the oracle's own
spread under rounding-level perturbations (see test_product_state_within_envelope)."""
import copy

import json
import os

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import generic_state, random_case, random_sop, random_tree
from oracle.oracle import Oracle, qr as oracle_qr
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb
from ttns_lib_gb300.model import full_state

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make_pair(topo, sop, state, m=12, tol=1e-12):
    orc = Oracle(topo, sop, krylov_dim=m, krylov_tol=tol)
    orc.set_state(state)
    A = api.httensor(topo)
    A.set(state)
    dev = api.fixed_step_projector_splitting_integrator(A, sop, krylov_dim=m, krylov_tolerance=tol)
    return orc, A, dev


@pytest.mark.parametrize("shape", [(9, 4), (64, 8), (256, 16), (4096, 64), (130, 33)])
def test_device_qr_matches_oracle(shape):
    rng = np.random.default_rng(shape[0])
    a = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    qd, rd = api.device_qr(a)
    qo, ro = oracle_qr(a)
    assert rel(qd, qo) < 1e-12 and rel(rd, ro) < 1e-12
    assert np.allclose(qd @ rd, a, atol=1e-12 * np.abs(a).max() * shape[0])


def test_device_qr_rank_deficient_exact_zeros():
    z = np.zeros((40, 6), dtype=np.complex128)
    z[7, 0] = 1.0
    z[3, 2] = -2.0 + 1j
    qd, rd = api.device_qr(z)
    qo, ro = oracle_qr(z)
    # same completion of the basis: identical zero pattern, values equal to rounding
    assert np.array_equal(qd == 0, qo == 0) and np.array_equal(rd == 0, ro == 0)
    assert np.allclose(qd, qo, rtol=1e-15, atol=1e-15) and np.allclose(rd, ro, rtol=1e-15, atol=1e-15)


def test_device_qr_tiny_columns_match_oracle():
    rng = np.random.default_rng(6)
    a = (rng.normal(size=(300, 16)) + 1j * rng.normal(size=(300, 16))) * 1e-170
    a[:, 0] *= 1e-140
    qd, rd = api.device_qr(a)
    qo, ro = oracle_qr(a)
    assert np.isfinite(qd).all() and np.isfinite(rd).all()
    assert rel(qd, qo) < 1e-12 and rel(rd, ro) < 1e-12


@pytest.mark.parametrize("seed", [310, 312, 338])
def test_random_operator_shapes_match_oracle_and_dense_expm(seed):
    """Operators whose groups mix terms acting below a node with terms that are the
    identity there: H_eff of every node against the oracle, then sweeps against exp(-iHt)."""
    topo, H, st, _ = random_case(seed)
    orc, A, dev = make_pair(topo, H, st, m=10)
    orc.refresh_env()
    dev.refresh_env(A)
    rng = np.random.default_rng(seed)
    for node in range(topo.nnodes):
        v = rng.normal(size=topo.node_shape(node)) + 1j * rng.normal(size=topo.node_shape(node))
        assert rel(dev.heff(node, v), orc.heff(node, v)) < 1e-12
        assert rel(dev.program_apply(node, v), orc.heff(node, v)) < 1e-12
    psi = full_state(topo, st)
    B = api.httensor(topo)
    B.set(st)
    integ = api.fixed_step_projector_splitting_integrator(B, H, krylov_dim=10)
    integ.dt = 0.1
    for k in range(3):
        integ(B, H, -1j)
        ex = sla.expm(-1j * H.dense() * (k + 1) * 0.1) @ psi
        assert np.linalg.norm(full_state(topo, B.get()) - ex) < 1e-10


def spin_boson_small():
    m, cfg = sb.build_config("c1")
    return m, cfg


def test_environments_and_heff_match_oracle():
    m, cfg = spin_boson_small()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(1))
    orc, A, dev = make_pair(topo, m.sop, st, m=cfg["krylov_dim"])
    orc.refresh_env()
    dev.refresh_env(A)
    rng = np.random.default_rng(2)
    for node in range(topo.nnodes):
        groups = orc.groups(node)
        assert dev.num_groups(node) == len(groups)
        for g, info in enumerate(groups):
            if node != 0 and not info["id_spf"]:
                assert rel(dev.env(node, g, "spf"), orc.env(node, g, "spf")) < 1e-12
            if node != 0 and not info["id_mf"]:
                assert rel(dev.env(node, g, "mf"), orc.env(node, g, "mf")) < 1e-12
        v = rng.normal(size=topo.node_shape(node)) + 1j * rng.normal(size=topo.node_shape(node))
        assert rel(dev.heff(node, v), orc.heff(node, v)) < 1e-12


def test_expm_node_matches_oracle():
    m, cfg = spin_boson_small()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(3))
    orc, A, dev = make_pair(topo, m.sop, st, m=cfg["krylov_dim"])
    orc.refresh_env()
    dev.refresh_env(A)
    for node in [0, 1, 2, 3, topo.nnodes - 1]:
        v = st[node]
        yo, no = orc.expm_node(node, v, 0.025)
        yd, nd = dev.expm_node(node, v, 0.025)
        assert rel(yd, yo) < 1e-11
        assert abs(nd - no) <= max(2, 0.05 * no)


def test_sweep_from_generic_state_matches_oracle():
    m, cfg = spin_boson_small()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(4))
    orc, A, dev = make_pair(topo, m.sop, st, m=cfg["krylov_dim"])
    dev.dt = cfg["dt"]
    for k in range(8):
        orc.step(cfg["dt"])
        dev(A, m.sop, -1j)
        szo = orc.expect(0, sb.SZ).real
        szd = dev.mel()(sb.SZ, 0, A).real
        assert abs(szo - szd) < 1e-10, (k, szo, szd)
    for a, b in zip(A.get(), orc.get_state()):
        assert rel(a, b) < 1e-9
    # the Krylov step-size rule rounds to two significant digits, so rounding-level
    # differences can flip an occasional sub-step: counts agree to a fraction of a percent
    assert abs(dev.nh_applications() - orc.nh_applications) <= 0.005 * orc.nh_applications
    assert abs(dev.mel()(A) - 1.0) < 1e-10


@pytest.mark.parametrize("seed", [0, 1])
def test_full_rank_random_tree_matches_dense_expm(seed):
    rng = np.random.default_rng(200 + seed)
    dims = [int(x) for x in rng.integers(2, 4, size=5)]
    topo = random_tree(rng, dims)
    H = random_sop(rng, dims, nterms=10)
    st = generic_state(topo, rng)
    psi = full_state(topo, st)
    Hd = H.dense()
    A = api.httensor(topo)
    A.set(st)
    dev = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10)
    dev.dt = 0.1
    for k in range(5):
        dev(A, H, -1j)
        ex = sla.expm(-1j * Hd * (k + 1) * 0.1) @ psi
        assert np.linalg.norm(full_state(topo, A.get()) - ex) < 1e-10


def test_bond_singular_values_match_oracle():
    m, cfg = spin_boson_small()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(8))
    orc, A, dev = make_pair(topo, m.sop, st, m=cfg["krylov_dim"])
    dev.dt = cfg["dt"]
    for k in range(3):
        for node in range(1, topo.nnodes):
            so = orc.bond_sv(node)
            sd = dev.bond_sv(A, node)
            assert sd.shape == so.shape
            assert np.abs(sd - so).max() < 1e-12 * max(1.0, so.max()), (k, node)
        orc.step(cfg["dt"])
        dev(A, m.sop, -1j)
    # a normalised state: the squared Schmidt values of every bond sum to 1
    for node in range(1, topo.nnodes):
        assert abs(np.sum(dev.bond_sv(A, node) ** 2) - 1.0) < 1e-12


def test_init_product_state_structure():
    m, cfg = spin_boson_small()
    topo = m.topology
    A = api.httensor(topo)
    A.init_product(np.array([1.0, 0.0]), seed=0)
    st = A.get()
    for i, a in enumerate(st):
        if i == 0:
            assert a[0, 0] == 1.0 and np.count_nonzero(a) == 1
            continue
        assert np.allclose(a.conj().T @ a, np.eye(a.shape[1]), atol=1e-12)
        if topo.is_leaf(i):
            assert a[0, 0] == 1.0 and np.all(a[1:, 0] == 0)


def test_product_state_within_envelope():
    """From spin-up x vacuum the truncated dynamics amplifies rounding; the device run
    must stay inside the spread of the oracle under 1e-15 coefficient perturbations."""
    m, cfg = spin_boson_small()
    topo = m.topology
    A = api.httensor(topo)
    A.init_product(np.array([1.0, 0.0]), seed=0)
    st = A.get()
    nsteps = 20
    dev = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=cfg["krylov_dim"])
    dev.dt = cfg["dt"]
    sd = []
    for _ in range(nsteps):
        dev(A, m.sop, -1j)
        sd.append(dev.mel()(sb.SZ, 0, A).real)

    def run(sop):
        o = Oracle(topo, sop, krylov_dim=cfg["krylov_dim"])
        o.set_state(st)
        out = []
        for _ in range(nsteps):
            o.step(cfg["dt"])
            out.append(o.expect(0, sb.SZ).real)
        return np.array(out)

    so = run(m.sop)
    spreads = []
    for seed in (1, 2, 3):
        s2 = copy.deepcopy(m.sop)
        s2.coeffs = s2.coeffs * (1 + 1e-15 * np.random.default_rng(seed).normal(size=s2.nterms))
        spreads.append(np.abs(run(s2) - so))
    env = np.max(spreads, axis=0)
    diff = np.abs(np.array(sd) - so)
    assert diff[0] < 1e-7
    assert np.all(diff <= 20 * np.maximum(env, 1e-8)), (diff, env)

def test_device_matches_golden_trajectory():
    """The committed dense-expm trajectory (tests/golden/make_golden.py) on the device:
    full-rank tree, so the sweep is exact; 40 steps including the first-step sub-steps."""
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "spin_boson_fullrank_N4.json")))
    m = sb.build(**g["params"])
    A = api.httensor(m.topology)
    A.set(sb.initial_state_numpy(m.topology, seed=g["seed"], psi0=np.array([1.0, 0.0])))
    dev = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=12, krylov_tolerance=1e-12)
    dev.dt = g["dt"]
    for k in range(g["steps"]):
        dev(A, m.sop, -1j)
        assert abs(dev.mel()(sb.SZ, 0, A).real - g["sz"][k]) < 1e-11, k
        assert abs(dev.mel()(sb.SX, 0, A).real - g["sx"][k]) < 1e-11, k


def test_residual_krylov_stop_matches_oracle():
    """Krylov stop rule 1 (the Lanczos recurrence ends on the residual estimate for the
    remaining interval): the device follows the oracle with the same rule to 1e-10 over
    six steps from a generic state, applies H far less often than the full-space rule, and
    stays within 1e-9 of the full-space trajectory."""
    w, c = sb.ohmic_modes(8, 0.5, 5.0)
    m = sb.build_from_modes(w, c, 6, 6, 0.3, 1.0)
    st = generic_state(m.topology, np.random.default_rng(17))
    orc = Oracle(m.topology, m.sop, krylov_dim=12, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_krylov_stop(1)
    A, B = api.httensor(m.topology), api.httensor(m.topology)
    A.set(st)
    B.set(st)
    ia = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=12, krylov_tolerance=1e-12)
    ib = api.fixed_step_projector_splitting_integrator(B, m.sop, krylov_dim=12, krylov_tolerance=1e-12)
    ia.set_krylov_stop(1)
    ia.dt = ib.dt = 0.05
    for _ in range(6):
        ia(A)
        ib(B)
        orc.step(0.05)
    assert max(np.max(np.abs(a - b)) for a, b in zip(A.get(), orc.get_state())) < 1e-10
    assert abs(ia.nh_applications() - orc.nh_applications) <= 0.02 * orc.nh_applications
    assert ia.nh_applications() < 0.8 * ib.nh_applications()
    assert abs(ia.mel()(sb.SZ, 0, A).real - ib.mel()(sb.SZ, 0, B).real) < 1e-9
