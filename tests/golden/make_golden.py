"""Writes the golden fixtures of tests/golden/ (run from the repository root:
`python tests/golden/make_golden.py`).

spin_boson_fullrank_N4.json: a spin-boson model (4 bath modes, local dimension 3, bond
dimension 9: every bond at full rank, where the projector-splitting sweep is exact) started
from the product state of `spin_boson.initial_state_numpy(seed=1)` with the spin up,
propagated by the dense matrix exponential exp(-i H t) of the full Hamiltonian (numpy /
scipy, independent of the oracle and of the GPU code); <sigma_z>, <sigma_x> of the spin and
the norm at t = 0.05 k, k = 1..40.
"""
import json
import os
import sys

import numpy as np
import scipy.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ttns_lib_gb300 import spin_boson as sb  # noqa: E402
from ttns_lib_gb300.model import full_state  # noqa: E402

PARAMS = dict(N=4, alpha=0.5, wc=5.0, d=3, chi=9, eps=0.3, delta=1.0)
DT, STEPS, SEED = 0.05, 40, 1


def spin_expectation(psi, op):
    """<psi| op (x) 1 |psi> with the spin as the slowest index of the full state."""
    d0 = op.shape[0]
    M = psi.reshape(d0, -1)
    return complex(np.vdot(M, op @ M))


def main():
    m = sb.build(**PARAMS)
    topo = m.topology
    st = sb.initial_state_numpy(topo, seed=SEED, psi0=np.array([1.0, 0.0]))
    psi0 = full_state(topo, st)
    H = m.sop.dense()
    U = sla.expm(-1j * H * DT)
    psi = psi0.copy()
    t, sz, sx, norm = [], [], [], []
    for k in range(1, STEPS + 1):
        psi = U @ psi
        t.append(DT * k)
        sz.append(spin_expectation(psi, sb.SZ).real)
        sx.append(spin_expectation(psi, sb.SX).real)
        norm.append(float(np.vdot(psi, psi).real))
    out = dict(description=__doc__.split("\n\n")[1].replace("\n", " "), params=PARAMS, dt=DT, steps=STEPS,
               seed=SEED, t=t, sz=sz, sx=sx, norm=norm)
    with open(os.path.join(HERE, "spin_boson_fullrank_N4.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
