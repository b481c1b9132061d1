"""The host orchestration of the CUDA library (ttns_lib_gb300/csrc/ttn_host.cpp, with the
adjoint sweep of ttn_adjoint.hpp) run on the CPU against a test double of the CUDA
runtime and of the kernel wrappers (tests/host_double/mock_cuda.cpp), and compared with
the oracle: the plain sweep, and the adjoint sweep's objective and gradients.  This checks
what the GPU tests cannot isolate -- the sequence of operations, their operands, the
tape, the environment snapshots and the host-side cotangent algebra -- while the kernels
themselves are checked on the GB300 by the gpu-marked tests.  The double is built here
with g++ and loaded in a child process only."""
import json
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.join(ROOT, "tests", "host_double")
OUT = os.path.join(HERE, "_build", "libttn_host_double.so")
CUDA_INC = "/usr/local/cuda/include"


def _build():
    if shutil.which("g++") is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime_api.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    srcs = [os.path.join(ROOT, "ttns_lib_gb300", "csrc", "ttn_host.cpp"),
            os.path.join(ROOT, "ttns_lib_gb300", "csrc", "ttn_noalloc.cu"), os.path.join(HERE, "mock_cuda.cpp")]
    deps = srcs + [os.path.join(ROOT, "ttns_lib_gb300", "csrc", f) for f in os.listdir(os.path.join(ROOT, "ttns_lib_gb300", "csrc"))
                   if f.endswith((".cuh", ".hpp"))]
    deps += [os.path.join(ROOT, "include", "ttn_gb300.h"), os.path.join(ROOT, "include", "ttn_gb300_testing.h"),
             os.path.join(ROOT, "oracle", "ttn_oracle.cpp"),
             os.path.join(ROOT, "oracle", "ttn_adjoint.hpp")]
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC, "-o", OUT]
    for s in srcs:
        cmd += ["-x", "c++", s]
    subprocess.check_call(cmd)
    return OUT


CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from ttns_lib_gb300 import api
api.LIB_PATH = {lib!r}
from ttns_lib_gb300 import spin_boson as sb
from oracle.oracle import Oracle
from helpers import generic_state, rand_herm, random_case, random_sop, random_tree

out = {{}}

def flat(ts):
    return np.concatenate([np.asarray(t).ravel() for t in ts])

def plain(name, topo, H, st, dt, steps):
    A = api.httensor(topo, device=0); A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10, krylov_tolerance=1e-13)
    integ.dt = dt
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-13); orc.set_state(st)
    for _ in range(steps):
        integ(A); orc.step(dt)
    out[name] = float(np.max(np.abs(flat(A.get()) - flat(orc.get_state()))))

def adjoint(name, topo, H, st, dt, wt, mode, O, ckpt):
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-13); orc.set_state(st)
    Jo, gco, gopo, gso = orc.adjoint(dt, len(wt), wt, mode, O, checkpoint_every=ckpt, state_cotangent=True)
    A = api.httensor(topo, device=0); A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10, krylov_tolerance=1e-13)
    Jd, gcd, gopd, gsd = integ.adjoint(A, dt, len(wt), wt, mode, O, checkpoint_every=ckpt, state_cotangent=True)
    scale = max(np.max(np.abs(gco)), max(np.max(np.abs(g)) for g in gopo))
    out[name] = dict(J=abs(Jd - Jo) / max(1.0, abs(Jo)),
                     coeff=float(np.max(np.abs(gcd - gco)) / scale),
                     ops=float(max(np.max(np.abs(a - b)) for a, b in zip(gopd, gopo)) / scale),
                     state=float(np.max(np.abs(flat(gsd) - gso)) / np.max(np.abs(gso))),
                     final=float(np.max(np.abs(flat(A.get()) - flat(orc.get_state())))))

m = sb.build(N=4, alpha=0.4, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
rng = np.random.default_rng(5)
st = generic_state(m.topology, rng)
plain("plain_spin_boson", m.topology, m.sop, st, 0.05, 3)
adjoint("adjoint_spin_boson", m.topology, m.sop, st, 0.05, rng.uniform(size=3), 0, sb.SZ, 2)
for seed, chi in ((201, 2), (202, None)):
    rng = np.random.default_rng(seed)
    dims = [int(x) for x in rng.integers(2, 4, size=5)]
    topo = random_tree(rng, dims, chi=chi)
    H = random_sop(rng, dims, nterms=10)
    st = generic_state(topo, rng)
    plain(f"plain_random_{{seed}}", topo, H, st, 0.1, 2)
    adjoint(f"adjoint_random_{{seed}}", topo, H, st, 0.1, rng.uniform(size=2), 0, rand_herm(rng, dims[0]), 1)
def heff(name, topo, H, st):
    A = api.httensor(topo, device=0); A.set(st)
    integ = api.fixed_step_projector_splitting_integrator(A, H, krylov_dim=10, krylov_tolerance=1e-13)
    integ.refresh_env(A)
    orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-13); orc.set_state(st); orc.refresh_env()
    rng = np.random.default_rng(1)
    worst = 0.0
    for nd in range(topo.nnodes):
        v = rng.normal(size=topo.node_shape(nd)) + 1j * rng.normal(size=topo.node_shape(nd))
        ho = orc.heff(nd, v)
        for got in (integ.heff(nd, v), integ.program_apply(nd, v)):
            worst = max(worst, float(np.max(np.abs(got - ho)) / max(1.0, np.max(np.abs(ho)))))
    out[name] = worst

for seed in (310, 312, 338):
    topo, H, st, dims = random_case(seed)
    heff(f"plain_heff_{{seed}}", topo, H, st)
    plain(f"plain_case_{{seed}}", topo, H, st, 0.1, 2)
    adjoint(f"adjoint_case_{{seed}}", topo, H, st, 0.1, np.random.default_rng(seed).uniform(size=2), 0,
            rand_herm(np.random.default_rng(seed), dims[0]), 1)
# subspace expansion: preparation (deterministic) equal to the oracle's, the random
# fallback equal to the oracle's, and steps at full capacity following exact dynamics
import scipy.linalg as sla
from helpers import full_rank
from ttns_lib_gb300.model import full_state, SOPOperator, Topology
w0, c0 = sb.ohmic_modes(4, 0.5, 5.0)
m2 = sb.build_from_modes(w0, c0, 3, 2, 0.3, 1.0)
cap = full_rank(sb.build_from_modes(w0, c0, 3, 27, 0.3, 1.0).topology).hrank
st = generic_state(m2.topology, np.random.default_rng(4))
orc = Oracle(m2.topology, m2.sop, krylov_dim=10, krylov_tol=1e-12); orc.set_state(st)
orc.set_expansion(cap, spawning_threshold=1e-7)
orc.expand_prepare(0.05)
A = api.httensor(m2.topology, device=0); A.set(st)
integ = api.subspace_expansion_projector_splitting_integrator(A, m2.sop, cap, krylov_dim=10, spawning_threshold=1e-7)
integ.dt = 0.05
integ.prepare(A)
out["expansion_prepare_ranks"] = float(np.max(np.abs(A.hrank() - orc.hrank())))
out["expansion_prepare_tensors"] = float(max(np.max(np.abs(a - b)) for a, b in zip(A.get(), orc.get_state())))
B = api.httensor(m2.topology, device=0); B.set(st)
i2 = api.subspace_expansion_projector_splitting_integrator(B, m2.sop, cap, krylov_dim=10, spawning_threshold=1e-12)
i2.dt = 0.05
for _ in range(20):
    i2(B)
ex = sla.expm(-1j * m2.sop.dense() * 1.0) @ full_state(m2.topology, st)
out["expansion_exact_dynamics"] = float(np.linalg.norm(full_state(B.current_topology(), B.get()) - ex))
out["expansion_full_capacity"] = float(np.max(np.abs(B.hrank() - cap)))
topo = Topology(np.array([-1, 0, 0, 0]), np.array([1, 3, 1, 3]), np.array([-1, 0, 1, 2]), np.array([0, 3, 3, 3]))
rng = np.random.default_rng(2)
H = SOPOperator(3, [3, 3, 3])
for r in range(3):
    a = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
    H.bind_dense(a + a.conj().T, [r], r)
st = generic_state(topo, rng)
orc = Oracle(topo, H, krylov_dim=8, krylov_tol=1e-12); orc.set_state(st)
orc.set_expansion(np.array([1, 3, 3, 3]), spawning_threshold=1e-12, minimum_unoccupied=2, seed=5)
C2 = api.httensor(topo, device=0); C2.set(st)
i3 = api.subspace_expansion_projector_splitting_integrator(C2, H, np.array([1, 3, 3, 3]), krylov_dim=8,
                                                           spawning_threshold=1e-12, minimum_unoccupied=2, seed=5)
i3.dt = 0.05
for _ in range(2):
    i3(C2); orc.step(0.05)
out["expansion_random_fallback"] = float(np.max(np.abs(full_state(C2.current_topology(), C2.get())
                                                       - full_state(orc.current_topology(), orc.get_state()))))
# Gram matrices above 96 (formed by one GEMM, Lanczos eigenpairs): bond dimensions equal to
# the oracle's, the state unchanged, every non-root node an isometry (the directions chosen
# inside near-degenerate singular-value clusters may differ between the two at rounding)
topo = Topology(np.array([-1, 0, 1, 1, 0, 0]), np.array([1, 4, 12, 12, 12, 12]), np.array([-1, -1, 0, 1, 2, 3]),
                np.array([0, 0, 12, 12, 12, 12]))
rng = np.random.default_rng(9)
H = random_sop(rng, [12] * 4, nterms=8)
st = generic_state(topo, rng)
capb = np.array([1, 40, 12, 12, 12, 12])
orc = Oracle(topo, H, krylov_dim=10, krylov_tol=1e-12); orc.set_state(st)
orc.set_expansion(capb, spawning_threshold=1e-7)
orc.expand_prepare(0.05)
D = api.httensor(topo, device=0); D.set(st)
i4 = api.subspace_expansion_projector_splitting_integrator(D, H, capb, krylov_dim=10, spawning_threshold=1e-7)
i4.dt = 0.05
i4.prepare(D)
out["expansion_large_gram_ranks"] = float(np.max(np.abs(D.hrank() - orc.hrank())))
out["expansion_large_gram_state"] = float(np.linalg.norm(full_state(D.current_topology(), D.get()) - full_state(topo, st)))
out["expansion_large_gram_isometries"] = float(max(np.max(np.abs(a.conj().T @ a - np.eye(a.shape[1]))) for a in D.get()[1:]))
# general observables against dense contractions of the full state vectors
mo = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
rng = np.random.default_rng(13)
sa, sb_ = generic_state(mo.topology, rng), generic_state(mo.topology, rng)
Ao, Bo = api.httensor(mo.topology, device=0), api.httensor(mo.topology, device=0)
Ao.set(sa); Bo.set(sb_)
mel = api.fixed_step_projector_splitting_integrator(Ao, mo.sop, krylov_dim=8).mel()
fa, fb = full_state(mo.topology, sa), full_state(mo.topology, sb_)
dims = mo.topology.mode_dims()
ops = {{0: sb.SZ, 2: rand_herm(rng, dims[2])}}
K = np.array([[1.0 + 0j]])
for mm, dd in enumerate(dims):
    K = np.kron(K, ops.get(mm, np.eye(dd)))
out["plain_obs_overlap"] = abs(mel.overlap(Ao, Bo) - np.vdot(fa, fb))
out["plain_obs_product"] = abs(mel.product(ops, Ao, Bo) - np.vdot(fa, K @ fb))
out["plain_obs_sop"] = abs(mel.sop(mo.sop, Ao, Bo) - np.vdot(fa, mo.sop.dense() @ fb))
# checkpoint and resume: identical continuation
import tempfile
with tempfile.TemporaryDirectory() as td:
    path = td + "/run.ckpt"
    mo = sb.build(N=4, alpha=0.5, wc=5.0, d=3, chi=3, eps=0.3, delta=1.0)
    st = generic_state(mo.topology, np.random.default_rng(3))
    Ac = api.httensor(mo.topology, device=0); Ac.set(st)
    ref = api.fixed_step_projector_splitting_integrator(Ac, mo.sop, krylov_dim=8)
    ref.dt = 0.05
    for k in range(5):
        ref(Ac)
        if k == 2:
            ref.save(Ac, path)
    Bc = api.httensor(mo.topology, device=0)
    res = api.fixed_step_projector_splitting_integrator(Bc, mo.sop, krylov_dim=8)
    res.load(Bc, path)
    for _ in range(2):
        res(Bc)
    out["plain_checkpoint_resume"] = float(max(np.max(np.abs(a - b)) for a, b in zip(Ac.get(), Bc.get())))
# time-dependent primitive operators through the update hook, against the oracle
def upd(mode, op, t, dt, mat):
    if op == 0:
        mat[:] = 0.5 * (0.3 + 0.8 * np.cos(3.0 * (t + dt / 2))) * sb.SZ + 0.5 * sb.SX
w0, c0 = sb.ohmic_modes(4, 0.5, 5.0)
mt = sb.build_from_modes(w0, c0, 3, 3, 0.3, 1.0)
st = generic_state(mt.topology, np.random.default_rng(2))
orc = Oracle(mt.topology, mt.sop, krylov_dim=10, krylov_tol=1e-12); orc.set_state(st); orc.set_op_update(upd)
At = api.httensor(mt.topology, device=0); At.set(st)
it_ = api.fixed_step_projector_splitting_integrator(At, mt.sop, krylov_dim=10)
it_.set_op_update(upd)
it_.dt = 0.05
for _ in range(6):
    it_(At); orc.step(0.05)
out["plain_time_dependent"] = float(max(np.max(np.abs(a - b)) for a, b in zip(At.get(), orc.get_state())))
# the orthogonaliser on an arbitrary state, then steps, against the oracle
rng = np.random.default_rng(21)
st = [rng.normal(size=t.shape) + 1j * rng.normal(size=t.shape) for t in generic_state(mt.topology, rng)]
from ttns_lib_gb300.model import full_state
st[0] = st[0] / np.linalg.norm(full_state(mt.topology, st))
orc = Oracle(mt.topology, mt.sop, krylov_dim=10, krylov_tol=1e-12); orc.set_state(st); orc.orthogonalise()
Ao = api.httensor(mt.topology, device=0); Ao.set(st)
io = api.fixed_step_projector_splitting_integrator(Ao, mt.sop, krylov_dim=10)
io.orthogonalise(Ao)
out["plain_orthogonalise"] = float(max(np.max(np.abs(a - b)) for a, b in zip(Ao.get(), orc.get_state())))
io.dt = 0.05
for _ in range(3):
    io(Ao); orc.step(0.05)
io.orthogonalise(Ao); orc.orthogonalise()
for _ in range(2):
    io(Ao); orc.step(0.05)
out["plain_orthogonalise_steps"] = float(max(np.max(np.abs(a - b)) for a, b in zip(Ao.get(), orc.get_state())))
# the residual stop rule reaches the device library (the double's exponential is exact, the
# oracle's within the Krylov tolerance)
sk = generic_state(mt.topology, np.random.default_rng(5))
orc = Oracle(mt.topology, mt.sop, krylov_dim=10, krylov_tol=1e-13); orc.set_state(sk); orc.set_krylov_stop(1)
Ak = api.httensor(mt.topology, device=0); Ak.set(sk)
ik = api.fixed_step_projector_splitting_integrator(Ak, mt.sop, krylov_dim=10, krylov_tolerance=1e-13)
ik.set_krylov_stop(1)
ik.dt = 0.05
for _ in range(3):
    ik(Ak); orc.step(0.05)
out["plain_krylov_stop"] = float(max(np.max(np.abs(a - b)) for a, b in zip(Ak.get(), orc.get_state())))
# bonds wider than 64 (70): the wide instantiations of the QR kernels in both gauge moves
import ctypes
from ttns_lib_gb300.model import Topology
tw = Topology(np.array([-1, 0, 1, 1, 0]), np.array([1, 70, 9, 9, 70]), np.array([-1, -1, 0, 1, 2]),
              np.array([0, 0, 9, 9, 70]))
rng = np.random.default_rng(41)
Hw = random_sop(rng, tw.mode_dims(), nterms=6)
sw = generic_state(tw, rng)
orc = Oracle(tw, Hw, krylov_dim=10, krylov_tol=1e-12); orc.set_state(sw)
Aw = api.httensor(tw, device=0); Aw.set(sw)
iw = api.fixed_step_projector_splitting_integrator(Aw, Hw, krylov_dim=10)
iw.dt = 0.05
count = ctypes.CDLL({lib!r}).mock_wide_qr_count
count.restype = ctypes.c_ulonglong
before = count()
for _ in range(2):
    iw(Aw); orc.step(0.05)
if count() - before < 6:
    raise SystemExit("no QR wider than 64 columns ran")
out["plain_wide_bonds"] = float(max(np.max(np.abs(a - b)) for a, b in zip(Aw.get(), orc.get_state())))
print(json.dumps(out))
"""


def test_host_orchestration_matches_oracle():
    lib = _build()
    code = CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), lib=lib)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for k, v in res.items():
        if k.startswith("expansion"):
            # ranks equal and tensors after the deterministic preparation equal to rounding;
            # at full capacity the expanding integrator follows exp(-iHt)
            assert v < (1e-6 if k == "expansion_exact_dynamics" else 1e-11), (k, v)
        elif k.startswith("plain"):
            assert v < 1e-11, (k, v)
        else:
            assert v["J"] < 1e-12, (k, v)
            assert v["coeff"] < 1e-10 and v["ops"] < 1e-10 and v["state"] < 1e-10, (k, v)
            assert v["final"] < 1e-11, (k, v)


DRIVER_CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, {root!r})
from ttns_lib_gb300 import api
api.LIB_PATH = {lib!r}
from ttns_lib_gb300 import driver as D
from oracle.oracle import Oracle
g = json.load(open({golden!r}))
doc = dict(g["beta_10/ohmic/spin_boson_sudden"]["input"]); doc["nmodes"] = 16
inp = D.parse_input(doc)
m = D.build_model(inp)
r = D.SpinBosonRun(inp, m, device=0)
orc = Oracle(m.topology, m.hamiltonian, krylov_dim=inp.krylov_dim, krylov_tol=inp.krylov_tolerance)
orc.init_product(inp.psi0, inp.seed)
orc.set_expansion(m.capacity, spawning_threshold=inp.spawning_parameter, unoccupied_threshold=inp.unoccupied_threshold,
                  minimum_unoccupied=inp.minimum_unoccupied, seed=0)
out = dict(first=r.first_row(), start=float(max(np.max(np.abs(a - b)) for a, b in zip(r.A.get(), orc.get_state()))),
           steps=[])
import ctypes
csr = ctypes.CDLL({lib!r}).mock_csr_op_count
csr.restype = ctypes.c_ulonglong
for k in range(2):
    r.step(); orc.step(inp.dt)
    out["csr_ops"] = int(csr())
    out["steps"].append(dict(values=float(max(abs(a - orc.expect(0, op).real) for a, op in zip(r.observables(), inp.ops))),
                             counts=[list(r.tdvp.expansion_counts()), list(orc.expansion_counts())],
                             hrank=bool(np.array_equal(r.hrank(), orc.hrank()[1:]))))
# with a time-dependent update hook the programs use the dense copies (kept current by the hook)
def keep(mode, op, t, dt, mat):
    pass
r.tdvp.set_op_update(keep); orc.set_op_update(keep)
before = int(csr())
r.step(); orc.step(inp.dt)
out["csr_with_hook"] = int(csr()) - before
out["hook_values"] = float(max(abs(a - orc.expect(0, op).real) for a, op in zip(r.observables(), inp.ops)))
# the command-line entry: input file in, the reference's columns out
import os, tempfile
tmp = tempfile.mkdtemp()
doc["output file"] = os.path.join(tmp, "sb.out")
with open(os.path.join(tmp, "sb.in"), "w") as f:
    json.dump(doc, f)
out["cli_rc"] = D.main([os.path.join(tmp, "sb.in"), "--steps", "1"])
out["cli_lines"] = open(doc["output file"]).read().splitlines()
doc.pop("Hsys")
with open(os.path.join(tmp, "bad.in"), "w") as f:
    json.dump(doc, f)
out["cli_bad_rc"] = D.main([os.path.join(tmp, "bad.in")])
print(json.dumps(out))
"""


def test_driver_device_path_matches_oracle():
    """The spin-boson driver's device path (start state, expansion set-up, steps, leaf
    observables, expansion counters, sparse leaf operators in the matvec programs) on the
    test double against the oracle, on a 16-mode version of the reference's sudden-cutoff
    example: the same start state bit for bit, the same bond dimensions and counts,
    observables to rounding."""
    lib = _build()
    code = DRIVER_CHILD.format(root=ROOT, lib=lib, golden=os.path.join(ROOT, "tests", "golden", "driver_examples.json"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["first"].startswith("0 0 0 1 1  0 0 0 2 2 ")
    assert res["start"] == 0.0
    assert res["csr_ops"] > 0  # the blocks' sparse operators went through the CSR contractions
    assert res["csr_with_hook"] == 0 and res["hook_values"] < 1e-10
    lines = res["cli_lines"]
    assert res["cli_rc"] == 0 and res["cli_bad_rc"] == 1
    assert len(lines) == 3 and lines[0].startswith("0 0 0 1 1  0 0 0 2 2 ") and lines[2].startswith("nh_app: ")
    f = lines[1].split()
    assert float(f[0]) == 0.005 and len(f) == len(lines[0].split())
    for s in res["steps"]:
        assert s["values"] < 1e-11 and s["hrank"], s
        assert s["counts"][0] == s["counts"][1], s


NOALLOC_CHILD = r"""
import ctypes as C, json
import numpy as np
lib = C.CDLL({lib!r})
lib.ttn_qr_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
lib.mock_alloc_calls.restype = C.c_ulonglong
rng = np.random.default_rng(5)
out = {{}}
before = lib.mock_alloc_calls()
for call, (m, n) in enumerate([(96, 20), (64, 64)]):
    a = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
    q = a.copy()
    r = np.full((n, n), np.nan, dtype=np.complex128)
    rc = lib.ttn_qr_noalloc(m, n, q.ctypes.data, r.ctypes.data, None, 0)
    out["rc%d" % call] = rc
    out["qr%d" % call] = float(np.abs(q @ r - a).max())
    out["orth%d" % call] = float(np.abs(q.conj().T @ q - np.eye(n)).max())
out["alloc_calls"] = int(lib.mock_alloc_calls() - before)
wide = np.zeros((128, 65), dtype=np.complex128)
rw = np.zeros((65, 65), dtype=np.complex128)
out["rc_wide"] = lib.ttn_qr_noalloc(128, 65, wide.ctypes.data, rw.ctypes.data, None, 0)
print(json.dumps(out))
"""


def test_noalloc_entry_point_allocates_nothing():
    """ttn_qr_noalloc, built into the CPU test double, makes no cudaMalloc, cudaFree,
    cudaMallocHost or cudaFreeHost call on its first (set-up) call or on the next one,
    factorises correctly, and rejects more than 64 columns with TTN_ECAPACITY."""
    lib = _build()
    r = subprocess.run([sys.executable, "-c", NOALLOC_CHILD.format(lib=lib)], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["alloc_calls"] == 0, res
    for call in range(2):
        assert res["rc%d" % call] == 0, res
        assert res["qr%d" % call] < 1e-12 and res["orth%d" % call] < 1e-12, res
    assert res["rc_wide"] == 2, res  # TTN_ECAPACITY
