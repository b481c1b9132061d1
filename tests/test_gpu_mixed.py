"""Mixed precision (tcgen05 tensor-core contractions on exact integer slices) against the
oracle and the FP64 path.

The mixed form runs the rank-64 mode and mean-field contractions of the Krylov matvec and
of the environment updates on the tensor cores: every FP64 operand row is scaled by a
power of two and cut into six 7-bit integer slices, the slice products are accumulated
exactly in FP32 level by level, and the levels are combined in integers, so a contraction
is accurate to about 1e-13 relative to sum |a||b|.  Tolerances: one H_eff application
within 1e-10 relative of the oracle, one node exponential within 1e-9, and <sigma_z> after
several sweeps within 1e-8 of the FP64 device path (the mixed form is measured against
max |d<sigma_z>| <= 1e-6).
"""
import numpy as np
import pytest

from helpers import generic_state
from oracle.oracle import Oracle
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def rank64_tree():
    # thermofield spin-boson, 2 x 8 bath modes of dimension 16, bonds of 64: the
    # headline workload's node shapes (16 x 16 x 64 and 64 x 64 x 64) on a small tree
    return sb.build_config("c3", N=8)


def integrators(topo, sop, state, m):
    out = {}
    for name, prec in (("fp64", api.PREC_FP64), ("mixed", api.PREC_MIXED)):
        A = api.httensor(topo)
        A.set(state)
        out[name] = (A, api.fixed_step_projector_splitting_integrator(A, sop, krylov_dim=m, krylov_tolerance=1e-12,
                                                                     precision=prec))
    return out


def test_mixed_program_apply_matches_oracle():
    m, cfg = rank64_tree()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(11))
    orc = Oracle(topo, m.sop, krylov_dim=cfg["krylov_dim"])
    orc.set_state(st)
    orc.refresh_env()
    its = integrators(topo, m.sop, st, cfg["krylov_dim"])
    for A, it in its.values():
        it.refresh_env(A)
    rng = np.random.default_rng(12)
    n_tc = 0
    for node in range(topo.nnodes):
        v = rng.normal(size=topo.node_shape(node)) + 1j * rng.normal(size=topo.node_shape(node))
        ref = orc.heff(node, v)
        y64 = its["fp64"][1].program_apply(node, v)
        ymx = its["mixed"][1].program_apply(node, v)
        assert rel(y64, ref) < 1e-12, node
        e = rel(ymx, ref)
        assert e < 1e-10, (node, e)
        if not np.array_equal(ymx, y64):
            n_tc += 1
    # every interior node of bond dimension 64 ran contractions on the tensor cores (its
    # result differs in the last bits from the FP64 contractions)
    rank64 = sum(1 for i in range(topo.nnodes) if not topo.is_leaf(i) and topo.hrank[i] == 64)
    assert rank64 > 0 and n_tc >= rank64


def test_mixed_expm_node_matches_oracle():
    m, cfg = rank64_tree()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(13))
    orc = Oracle(topo, m.sop, krylov_dim=cfg["krylov_dim"])
    orc.set_state(st)
    orc.refresh_env()
    its = integrators(topo, m.sop, st, cfg["krylov_dim"])
    A, it = its["mixed"]
    it.refresh_env(A)
    for node in range(2, topo.nnodes, 3):
        yo, _ = orc.expm_node(node, st[node], cfg["dt"])
        yd, _ = it.expm_node(node, st[node], cfg["dt"])
        assert rel(yd, yo) < 1e-9, node


def test_mixed_sweeps_track_fp64():
    m, cfg = rank64_tree()
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(14))
    its = integrators(topo, m.sop, st, cfg["krylov_dim"])
    worst = 0.0
    for A, it in its.values():
        it.dt = cfg["dt"]
    for k in range(6):
        sz = {}
        for name, (A, it) in its.items():
            it(A, m.sop, -1j)
            sz[name] = it.mel()(sb.SZ, 0, A).real
        worst = max(worst, abs(sz["mixed"] - sz["fp64"]))
    assert worst <= 1e-8, worst
    A, it = its["mixed"]
    assert abs(it.mel()(A) - 1.0) < 1e-10


def test_mixed_residual_stop_tracks_the_oracle():
    """Krylov stop rule 1 (the Lanczos recurrence ends on the residual estimate, the
    reference's rule) in mixed precision: four sweeps of a 17-node tree with the headline
    workload's node shapes (4096 x 64 nodes on the tensor cores) from a generic state
    follow the oracle with the same rule to 1e-8 in <sigma_z> and 1e-7 in every node
    tensor, with the oracle's count of H applications to 2 %."""
    m, cfg = sb.build_config("c3", N=4)
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(15))
    orc = Oracle(topo, m.sop, krylov_dim=cfg["krylov_dim"], krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_krylov_stop(1)
    A = api.httensor(topo)
    A.set(st)
    it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=cfg["krylov_dim"], krylov_tolerance=1e-12,
                                                      precision=api.PREC_MIXED)
    it.set_krylov_stop(1)
    it.dt = cfg["dt"]
    for _ in range(4):
        it(A, m.sop, -1j)
        orc.step(cfg["dt"])
    assert abs(it.mel()(sb.SZ, 0, A).real - orc.expect(0, sb.SZ).real) < 1e-8
    assert max(np.max(np.abs(a - b)) for a, b in zip(A.get(), orc.get_state())) < 1e-7
    assert abs(it.nh_applications() - orc.nh_applications) <= 0.02 * orc.nh_applications
