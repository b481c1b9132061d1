"""Checkpoint and resume (ttn_integrator_save / ttn_integrator_load): a run saved after
some steps and resumed in a fresh integrator and state continues exactly like the
uninterrupted run; a checkpoint of another tree is refused."""
import os

import numpy as np
import pytest

from helpers import generic_state
from ttns_lib_gb300 import api
from ttns_lib_gb300 import spin_boson as sb

pytestmark = pytest.mark.gpu


def test_resume_continues_the_uninterrupted_run(tmp_path):
    m = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    topo = m.topology
    st = generic_state(topo, np.random.default_rng(3))
    A = api.httensor(topo)
    A.set(st)
    ref = api.fixed_step_projector_splitting_integrator(A, m.sop, krylov_dim=8)
    ref.dt = 0.05
    path = os.path.join(str(tmp_path), "run.ckpt")
    for k in range(5):
        ref(A, m.sop, -1j)
        if k == 2:
            ref.save(A, path)
    B = api.httensor(topo)
    res = api.fixed_step_projector_splitting_integrator(B, m.sop, krylov_dim=8)
    res.load(B, path)
    assert abs(res.t() - 3 * 0.05) < 1e-15
    for _ in range(2):
        res(B, m.sop, -1j)
    for a, b in zip(A.get(), B.get()):
        assert np.max(np.abs(a - b)) < 1e-13
    assert res.nh_applications() == ref.nh_applications()
    other = sb.build(N=3, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    C = api.httensor(other.topology)
    oi = api.fixed_step_projector_splitting_integrator(C, other.sop, krylov_dim=8)
    with pytest.raises(api.TTNError):
        oi.load(C, path)
