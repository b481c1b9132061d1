"""Time-dependent primitive operators (ttn_integrator_set_op_update) on the device against
the oracle with the same update hook: a driven spin-boson model on a truncated tree."""
import numpy as np
import pytest

from helpers import generic_state
from oracle.oracle import Oracle
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

pytestmark = pytest.mark.gpu


def test_driven_sweep_matches_oracle():
    w, c = sb.ohmic_modes(4, 0.5, 5.0)
    m = sb.build_from_modes(w, c, 3, 3, 0.3, 1.0)
    topo = m.topology

    def update(mode, op, t, dt, mat):
        if op == 0:
            mat[:] = 0.5 * (0.3 + 0.8 * np.cos(3.0 * (t + dt / 2))) * sb.SZ + 0.5 * sb.SX

    st = generic_state(topo, np.random.default_rng(2))
    orc = Oracle(topo, m.sop, krylov_dim=10, krylov_tol=1e-12)
    orc.set_state(st)
    orc.set_op_update(update)
    A = api.httensor(topo)
    A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=10)
    integ.set_op_update(update)
    integ.dt = 0.05
    for _ in range(6):
        integ(A, m.sop, -1j)
        orc.step(0.05)
    assert abs(integ.mel()(sb.SZ, 0, A).real - orc.expect(0, sb.SZ).real) < 1e-10
    for a, b in zip(A.get(), orc.get_state()):
        assert np.max(np.abs(a - b)) < 1e-9


def test_interaction_picture_coupling_matches_oracle():
    """The driver's interaction-picture coupling (interaction_picture_sb_operator) through
    the device hook: a four-block spin-boson model stepped on the device and by the oracle
    with the same hook."""
    from helpers import full_rank
    from ttns_lib_gb300 import driver as D
    doc = {"Hsys": [[0, 1], [1, 0]], "Scoup": [[1, 0], [0, -1]], "psi0": [1, 0],
           "bath": {"type": "exponential", "wc": 2.0, "alpha": 0.2, "s": 1},
           "max frequency cutoff": 6.0, "tmax": 1.0, "dt": 0.05, "nspf": 2, "nspf lower": 2,
           "nmodes": 4, "maximum dimension": 5, "target dimension": 5, "ops": [[1, 0], [0, -1]]}
    inp = D.parse_input(doc)
    wk, gk = D.bath_modes(inp)
    blocks = D.make_blocks(inp, wk, gk)
    topo = full_rank(D.driver_topology(2, [b.nstates for b in blocks], 2, 2))
    H, upd = D.build_interaction_picture_hamiltonian(inp, blocks)
    st = generic_state(topo, np.random.default_rng(3))
    orc = Oracle(topo, H, krylov_dim=12, krylov_tol=1e-13)
    orc.set_state(st)
    orc.set_op_update(upd)
    A = api.httensor(topo)
    A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=12, krylov_tolerance=1e-13)
    integ.set_op_update(upd)
    integ.dt = 0.05
    for _ in range(8):
        integ(A, H, -1j)
        orc.step(0.05)
    assert abs(integ.mel()(sb.SZ, 0, A).real - orc.expect(0, sb.SZ).real) < 1e-10
    for a, b in zip(A.get(), orc.get_state()):
        assert np.max(np.abs(a - b)) < 1e-9
