"""Batched form: ttn_batch_step on independent instances against stepping each instance
on its own, through the C-ABI.

Instances share nothing (each integrator owns its stream and workspaces), so the batched
results must equal the one-at-a-time results exactly, whatever the thread count.
"""
import numpy as np
import pytest

from helpers import generic_state
from oracle.oracle import Oracle
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

pytestmark = pytest.mark.gpu

# small instances of the batched workload: different bath sizes, cut-offs, couplings and
# bond dimensions (the per-instance parameters vary as in the batched configuration)
SPECS = [
    dict(N=4, alpha=0.2, wc=2.0, d=4, chi=4, eps=0.0, delta=1.0, beta=None),
    dict(N=6, alpha=0.5, wc=5.0, d=6, chi=6, eps=0.3, delta=1.0, beta=None),
    dict(N=8, alpha=0.1, wc=3.0, d=8, chi=8, eps=-0.5, delta=1.0, beta=None),
    dict(N=4, alpha=0.8, wc=1.5, d=8, chi=8, eps=0.0, delta=1.0, beta=2.0),
    dict(N=5, alpha=0.3, wc=8.0, d=4, chi=8, eps=0.1, delta=1.0, beta=None),
]


def make(spec):
    m = sb.build(spec["N"], spec["alpha"], spec["wc"], spec["d"], spec["chi"], spec["eps"], spec["delta"],
                 spec["beta"])
    A = api.httensor(m.topology)
    A.init_product(psi0=[1.0, 0.0], seed=0)
    it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=10, krylov_tolerance=1e-12)
    it.dt = 0.05
    return m, A, it


@pytest.mark.parametrize("threads", [1, 3, 0])
def test_batch_step_equals_sequential_steps(threads):
    seq = [make(s) for s in SPECS]
    bat = [make(s) for s in SPECS]
    for _ in range(3):
        for m, A, it in seq:
            it(A, m.sop, -1j)
        api.batch_step([it for _, _, it in bat], [A for _, A, _ in bat], -1j, threads=threads)
    for (m, A, it), (mb, Ab, itb) in zip(seq, bat):
        assert itb.t() == it.t()
        assert itb.nh_applications() == it.nh_applications()
        for x, y in zip(A.get(), Ab.get()):
            assert np.array_equal(x, y)
        assert it.mel()(sb.SZ, 0, A) == itb.mel()(sb.SZ, 0, Ab)


def test_batch_step_reports_the_failing_instance():
    good = [make(s) for s in SPECS[:2]]
    m, A, it = make(SPECS[2])
    other = api.httensor(good[0][0].topology)  # a state of another tree
    other.init_product(psi0=[1.0, 0.0], seed=0)
    with pytest.raises(api.TTNError, match="instance 2"):
        api.batch_step([good[0][2], good[1][2], it], [good[0][1], good[1][1], other], -1j, threads=2)


def test_batch_instances_match_the_oracle():
    """Uneven instances stepped together by ttn_batch_step from generic states, each against
    the oracle stepping the same instance: <sz> to 1e-10 after every step and the node
    tensors to 1e-9 after three."""
    rng = np.random.default_rng(9)
    inst = []
    for spec in SPECS[:4]:
        m = sb.build(spec["N"], spec["alpha"], spec["wc"], spec["d"], spec["chi"], spec["eps"], spec["delta"],
                     spec["beta"])
        st = generic_state(m.topology, rng)
        orc = Oracle(m.topology, m.sop, krylov_dim=10, krylov_tol=1e-12)
        orc.set_state(st)
        A = api.httensor(m.topology)
        A.set(st)
        it = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=10, krylov_tolerance=1e-12)
        it.dt = 0.05
        inst.append((m, orc, A, it))
    for k in range(3):
        api.batch_step([it for _, _, _, it in inst], [A for _, _, A, _ in inst], -1j, threads=0)
        for i, (m, orc, A, it) in enumerate(inst):
            orc.step(0.05)
            szo = orc.expect(0, sb.SZ).real
            szd = it.mel()(sb.SZ, 0, A).real
            assert abs(szo - szd) < 1e-10, (i, k, szo, szd)
    for i, (m, orc, A, it) in enumerate(inst):
        for a, b in zip(A.get(), orc.get_state()):
            assert np.linalg.norm(a - b) <= 1e-9 * max(np.linalg.norm(b), 1e-300), i
