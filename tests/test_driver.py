"""The spin-boson driver (ttns_lib_gb300/driver.py, bath.py) against the reference's own
example outputs (tests/golden/driver_examples.json, made by make_driver_fixtures.py from
the reference's inputs/ and example_outputs/): the tree each input lays out, the output
format, and -- through the oracle -- the first step of the dynamics; plus known answers
for the bath discretisation and the block operators."""
import json
import math
import os

import numpy as np
import pytest

from ttns_lib_gb300 import bath as B
from ttns_lib_gb300 import driver as D

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "driver_examples.json")
WITH_BONDS = ["beta_10/ohmic/spin_boson_debye", "beta_10/ohmic/spin_boson_exponential",
              "beta_10/ohmic/spin_boson_sudden"]


def _golden():
    with open(GOLDEN) as f:
        return json.load(f)


def test_inputs_parse_with_the_reference_key_rules():
    g = _golden()
    for case, v in g.items():
        inp = D.parse_input(v["input"])
        assert inp.nmodes == 512 and inp.dt == 5e-3
        assert len(inp.ops) == 4
        assert np.allclose(inp.ops[1], [[0, -1j], [1j, 0]])
        assert inp.minimum_unoccupied == 2 and inp.krylov_dim == 12
        assert inp.bath.nonzero_temperature == case.startswith("beta")
    d = dict(g[WITH_BONDS[0]]["input"])
    d["  Max   Frequency Cutoff "] = d.pop("max frequency cutoff")
    assert D.parse_input(d).max_frequency_cutoff == 500
    bad = dict(g[WITH_BONDS[0]]["input"])
    bad["psi0"] = [1, 0, 0]
    with pytest.raises(ValueError, match="wavefunction"):
        D.parse_input(bad)
    bad = dict(g[WITH_BONDS[0]]["input"])
    bad["bath"] = {"type": "lorentzian", "wc": 1.0}
    with pytest.raises(ValueError, match="unknown bath"):
        D.parse_input(bad)


@pytest.mark.parametrize("case", WITH_BONDS)
def test_tree_matches_the_reference_example(case):
    """The bond dimension of every node on the first output row: pins the frequency
    window, the Gauss nodes (they decide how many modes share a block), the partition
    and the tree builder with its level-dependent bond dimensions."""
    v = _golden()[case]
    inp = D.parse_input(v["input"])
    wk, gk = D.bath_modes(inp)
    blocks = D.make_blocks(inp, wk, gk)
    topo = D.driver_topology(inp.hsys.shape[0], [b.nstates for b in blocks], inp.nspf, inp.nspf_lower)
    assert np.array_equal(topo.hrank[1:], np.array(v["rows"][0]["hrank"]))


@pytest.mark.parametrize("case", sorted(json.load(open(GOLDEN))))
def test_output_rows_are_formatted_like_the_reference(case):
    v = _golden()[case]
    r0, r1 = v["rows"][0], v["rows"][1]
    assert D.format_row(r0["t"], r0["values"], None, None, r0["hrank"] or None) == v["text"][0]
    assert D.format_row(r1["t"], r1["values"], r1["counts"], r1["nh_per_node"], r1["hrank"] or None) == v["text"][1]
    assert D.nsteps_for(5.0, 5e-3) == 1000 and D.nsteps_for(0.0105, 5e-3) == 3


def test_first_step_matches_the_reference_example():
    """The oracle stepping the driver's model of beta_10/ohmic/spin_boson_debye (343
    blocks, 687 nodes) from the driver's start state: after one step the observables
    agree with the reference's printed values to 1e-8; the two-site expansion count (which
    includes the start-up expansion sweeps) to 2 %; and almost every bond dimension.  The
    reference finds the dominant two-site directions with a 12-vector Krylov eigensolver
    and the oracle with an exact eigensolver, so the bonds that sit at the spawning
    threshold can differ by one."""
    from oracle.oracle import Oracle
    v = _golden()[WITH_BONDS[0]]
    inp = D.parse_input(v["input"])
    m = D.build_model(inp)
    orc = Oracle(m.topology, m.hamiltonian, krylov_dim=inp.krylov_dim, krylov_tol=inp.krylov_tolerance)
    orc.init_product(inp.psi0, inp.seed)
    for (r0, x) in zip(v["rows"][0]["values"], [orc.expect(0, op).real for op in inp.ops]):
        assert abs(r0 - x) < 1e-14
    orc.set_expansion(m.capacity, spawning_threshold=inp.spawning_parameter,
                      unoccupied_threshold=inp.unoccupied_threshold, minimum_unoccupied=inp.minimum_unoccupied, seed=0)
    orc.step(inp.dt)
    row = v["rows"][1]
    vals = [orc.expect(0, op).real for op in inp.ops]
    assert np.max(np.abs(np.array(vals) - row["values"])) < 1e-8
    one, two = orc.expansion_counts()
    assert one == row["counts"][0]
    assert abs(two - row["counts"][1]) <= 0.02 * row["counts"][1]
    hr = orc.hrank()[1:]
    ref = np.array(row["hrank"])
    assert np.mean(hr == ref) > 0.95 and np.max(np.abs(hr - ref)) <= 2


# ---- bath discretisation ------------------------------------------------------------

def test_gauss_rule_of_a_jacobi_measure_is_gauss_jacobi():
    """J(w) = c (w/wc)^s (1 - w/wc)^q on [0, wc] is a Jacobi weight: its Gauss rule is the
    Gauss-Jacobi rule (both endpoints singular, exercising the Gauss-Jacobi panels)."""
    from scipy.special import roots_jacobi
    b = B.JacobiCutoff(alpha=0.7, wc=3.0, s=0.5, q=1.5)
    N = 40
    w, W = B.gauss_rule(b, 0.0, 3.0, N)
    t, tw = roots_jacobi(N, 1.5, 0.5)   # weight (1 - t)^1.5 (1 + t)^0.5
    x = 1.5 * (1.0 + t)
    c = b._pref() * b.wc / b.wc ** b.s / b.wc ** b.q   # J = c w^s (wc - w)^q
    Wx = c * tw * 1.5 ** (1.0 + b.s + b.q)
    assert np.allclose(np.sort(w), np.sort(x), rtol=0, atol=1e-12)
    assert np.allclose(W[np.argsort(w)], Wx[np.argsort(x)], rtol=1e-11)


@pytest.mark.parametrize("bath,lo,hi", [
    (B.Exponential(2.0, 25.0, 1.0), 0.0, 500.0),
    (B.Exponential(2.0, 25.0, 0.5), 0.0, 172.7),
    (B.Debye(2.0, 25.0, beta=10.0), -2.0, 500.0),
    (B.Sudden(2.0, 25.0, 1.0, beta=10.0), -1.0, 25.0),
])
def test_gauss_rule_integrates_polynomials_exactly(bath, lo, hi):
    """sum_k W_k p(w_k) = int p dmu for p = Chebyshev polynomials of the window up to
    degree 2N - 1 (mu = J, or J / (1 - exp(-beta w)) at finite temperature)."""
    from scipy.integrate import quad
    N = 64
    w, W = B.gauss_rule(bath, lo, hi, N)
    assert np.all(W > 0) and np.all(np.diff(w) > 0) and lo < w[0] and w[-1] < hi
    y = (2.0 * w - (hi + lo)) / (hi - lo)
    pts = sorted({p for p, *_ in bath.breakpoints() if lo < p < hi} | ({0.0} if lo < 0 < hi else set()))
    for k in (0, 1, 7, 40, 2 * N - 1):
        f = lambda x: float(bath.measure(np.float64(x))) * math.cos(k * math.acos(max(-1.0, min(1.0, (2 * x - hi - lo) / (hi - lo)))))
        exact = quad(f, lo, hi, points=pts or None, limit=2000, epsabs=0, epsrel=1e-13)[0]
        got = float(np.sum(W * np.cos(k * np.arccos(np.clip(y, -1, 1)))))
        assert abs(got - exact) <= 1e-10 * float(np.sum(W)), k


def test_frequency_window_and_couplings():
    b = B.Exponential(2.0, 25.0, 1.0, beta=10.0)
    lo, hi = b.frequency_bounds(1e-3)
    assert hi == pytest.approx(25.0 * math.log(1000.0), rel=1e-15)
    # the negative bound keeps 1 - tol of the Boltzmann-weighted density
    from scipy.integrate import quad
    rho = lambda x: float(b.density(np.float64(x))) * math.exp(-10.0 * x)
    tot = quad(rho, 0, hi, epsrel=1e-13)[0]
    assert quad(rho, 0, -lo, epsrel=1e-13)[0] == pytest.approx((1 - 1e-3) * tot, rel=1e-10)
    w, g = B.discretise(b, 32, lo, hi)
    assert lo < 0 and np.all(np.diff(np.abs(w)) >= 0) and w.min() >= lo
    assert np.sum(math.pi * g ** 2) == pytest.approx(quad(lambda x: float(b.measure(np.float64(x))), lo, hi, points=[0.0],
                                                          epsrel=1e-13)[0], rel=1e-10)
    d = B.Debye(alpha=0.0, wc=4.0)
    assert B.load_bath({"type": "Debye", "wc": 4.0, "lambda": 2.0}).alpha == pytest.approx(1.0)
    assert B.load_bath({"type": "exponential", "wc": 1, "alpha": 1, "s": 1, "T": 0}).beta is None
    assert B.load_bath({"type": "exponential", "wc": 1, "alpha": 1, "s": 1, "T": 0.5}).beta == 2.0
    assert d.upper_bound(0.08) == pytest.approx(4.0 * math.tan(0.92 * math.pi / 2))


# ---- blocks ---------------------------------------------------------------------------

def test_block_operators_are_the_harmonic_ones():
    """A two-mode block: H0 = sum w_j n_j and Hc = sum g_j (a_j + a_j^dagger) in the
    product basis, first mode slowest, against Kronecker products."""
    wk = np.array([10.0, 11.0])
    gk = np.array([0.3, 0.7])
    blk = D.make_block(wk, gk, 3000.0, 5)
    assert blk.nstates == 25
    a = np.diag(np.sqrt(np.arange(1, 5)), 1)
    n = np.diag(np.arange(5.0))
    I = np.eye(5)
    H0 = wk[0] * np.kron(n, I) + wk[1] * np.kron(I, n)
    Hc = gk[0] * np.kron(a + a.T, I) + gk[1] * np.kron(I, a + a.T)
    assert np.allclose(np.diag(blk.h0), H0)
    assert np.allclose(blk.hc_dense(), Hc)
    # the first row's entries: lowering in mode order, then raising in reverse mode order
    assert list(blk.hc_indices[blk.hc_indptr[6]:blk.hc_indptr[7]]) == [1, 5, 7, 11]


def test_block_dimension_follows_its_lowest_frequency():
    """Every mode of a block keeps the first (lowest) mode's count, so the block holds
    nper(w_0)^n states; when a later mode keeps fewer, the rows past the product basis
    have no energy and no coupling."""
    wk = np.array([300.0, 340.0])          # floor(3000/w) = 10, 8
    blk = D.make_block(wk, np.array([0.1, 0.2]), 3000.0, 10)
    assert blk.nstates == 100 and blk.occupations.shape[0] == 80
    H = blk.hc_dense()
    assert np.allclose(H, H.T) and not np.any(H[80:]) and not np.any(blk.h0[80:])


def test_partition_groups_modes_under_the_target_dimension():
    """Blocks grow from the lowest frequency while nper(w_first)^n stays under the target:
    low modes keep 30 states (900 <= 1000 < 27000: pairs), modes above wc = 50 keep
    min(10, floor(3000 / w)) (pairs of 10 or 9, triples of 6 for w >= 430)."""
    wk = np.array([0.5, 1.0, 2.0, 60.0, 300.0, 310.0, 320.0, 430.0, 440.0, 450.0])
    assert D.partition_modes(wk, 3000.0, 50.0, 1000, 250, 30, 10) == [2, 2, 2, 2, 2]
    assert D.partition_modes(np.array([430.0, 440.0, 450.0, 460.0]), 3000.0, 50.0, 1000, 250, 30, 10) == [3, 1]
    # a lone mode above the target still forms a block
    assert D.partition_modes(np.array([0.1, 0.2]), 3000.0, 50.0, 20, 250, 30, 10) == [1, 1]
    with pytest.raises(ValueError):
        D.partition_modes(wk[::-1], 3000.0, 50.0, 1000, 250, 30, 10)


def test_level_ranks_interpolate_geometrically():
    f = D.level_ranks(8, 4, 8)
    assert [f(l) for l in range(10)] == [8, 7, 6, 6, 5, 5, 4, 4, 4, 4]
    g = D.level_ranks(4, 4, 3)
    assert [g(l) for l in range(5)] == [4, 4, 4, 4, 4]


def _small_driver_model():
    from helpers import full_rank
    doc = {"Hsys": [[0, 1], [1, 0]], "Scoup": [[1, 0], [0, -1]], "psi0": [1, 0],
           "bath": {"type": "exponential", "wc": 2.0, "alpha": 0.2, "s": 1},
           "max frequency cutoff": 6.0, "tmax": 1.0, "dt": 0.05, "nspf": 2, "nspf lower": 2,
           "nmodes": 4, "maximum dimension": 5, "target dimension": 5, "ops": [[1, 0], [0, -1]]}
    inp = D.parse_input(doc)
    wk, gk = D.bath_modes(inp)
    blocks = D.make_blocks(inp, wk, gk)
    topo = full_rank(D.driver_topology(2, [b.nstates for b in blocks], 2, 2))
    return inp, blocks, topo


def test_interaction_picture_coupling_converges_to_the_schroedinger_picture():
    """interaction_picture_sb_operator through the time-dependent operator hook: without
    the bath's H0 and with each block's coupling averaged over every evolution interval,
    <sz>(t) converges at second order or better to exact dense Schroedinger-picture
    dynamics (full-rank tree, so the only error is the time dependence), and the averaged
    couplings are the interval means of g exp(i w s) (the end-point value below
    |w dt| = 1e-5, as the reference computes them)."""
    import scipy.linalg as sla
    from scipy.integrate import quad
    from oracle.oracle import Oracle
    from ttns_lib_gb300.model import full_state
    inp, blocks, topo = _small_driver_model()
    ip = D.InteractionPictureCoupling(blocks[1])
    w, g = blocks[1].wk[0], blocks[1].gk[0]
    mean = (quad(lambda s: math.cos(w * s), 0.3, 0.4)[0] + 1j * quad(lambda s: math.sin(w * s), 0.3, 0.4)[0]) / 0.1
    assert abs(ip.averaged_couplings(0.3, 0.1)[0] - g * mean) < 1e-14
    te = 0.3 + 1e-7  # below |w dt| = 1e-5 the reference's series gives the end-point value
    assert abs(ip.averaged_couplings(0.3, 1e-7)[0] - g * complex(math.cos(w * te), math.sin(w * te))) < 1e-15
    assert np.allclose(ip.matrix(0.0, 0.0), blocks[1].hc_dense())
    HS = D.build_hamiltonian(inp, blocks)
    HI, upd = D.build_interaction_picture_hamiltonian(inp, blocks)
    o = Oracle(topo, HS, krylov_dim=12, krylov_tol=1e-13)
    o.init_product(inp.psi0, 0)
    st = o.get_state()
    psi = full_state(topo, st)
    ex = sla.expm(-1j * HS.dense() * 1.0) @ psi
    sz = np.kron(np.diag([1.0, -1.0]), np.eye(len(psi) // 2))
    ref = np.vdot(ex, sz @ ex).real
    errs = []
    for dt in (0.05, 0.025, 0.0125):
        oi = Oracle(topo, HI, krylov_dim=12, krylov_tol=1e-13)
        oi.set_state(st)
        oi.set_op_update(upd)
        for _ in range(int(round(1.0 / dt))):
            oi.step(dt)
        errs.append(abs(oi.expect(0, np.diag([1.0, -1.0])).real - ref))
    assert errs[0] < 2e-4 and errs[2] < 5e-6
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5


def test_sudden_cutoff_example_step_by_step():
    """beta_10/ohmic/spin_boson_sudden (512 one-mode blocks of 100 states): through the
    oracle, the first three printed rows of the reference -- observables to 1e-10, the
    expansion counts (start-up expansion sweeps included) exactly for two steps and to one
    bond decision in the third (9200 against 9201: one bond at the spawning threshold,
    where the reference's Krylov estimate and the exact eigensolver part)."""
    from oracle.oracle import Oracle
    v = _golden()["beta_10/ohmic/spin_boson_sudden"]
    inp = D.parse_input(v["input"])
    m = D.build_model(inp)
    orc = Oracle(m.topology, m.hamiltonian, krylov_dim=inp.krylov_dim, krylov_tol=inp.krylov_tolerance)
    orc.init_product(inp.psi0, inp.seed)
    orc.set_expansion(m.capacity, spawning_threshold=inp.spawning_parameter,
                      unoccupied_threshold=inp.unoccupied_threshold, minimum_unoccupied=inp.minimum_unoccupied, seed=0)
    for k in (1, 2, 3):
        orc.step(inp.dt)
        row = v["rows"][k]
        vals = np.array([orc.expect(0, op).real for op in inp.ops])
        assert np.max(np.abs(vals - row["values"])) < 1e-10, (k, vals, row["values"])
        one, two = orc.expansion_counts()
        assert one == row["counts"][0] and abs(two - row["counts"][1]) <= (0 if k < 3 else 2), (k, two, row["counts"])


def test_other_baths_and_input_forms():
    """Gaussian and Jacobi-cutoff baths, a temperature given as T, a single observable
    matrix, and the defaults of the optional entries: the model builds, the window and the
    couplings follow the bath (sum pi g^2 = integral of the measure over the window)."""
    from scipy.integrate import quad
    base = {"Hsys": [[0, 1], [1, 0]], "Scoup": [[1, 0], [0, -1]], "psi0": [1, 0], "tmax": 0.1, "dt": 0.01,
            "nspf": 4, "nspf lower": 2, "nmodes": 24, "maximum dimension": 6, "target dimension": 40,
            "ops": [[1, 0], [0, -1]]}
    cases = [
        ({"type": "gaussian", "wc": 3.0, "alpha": 0.5, "T": 0.5}, 1e-4),
        ({"type": "jacobi", "wc": 4.0, "alpha": 0.3, "s": 1.5, "q": 2.0}, 1e-4),
        ({"type": "sudden", "wc": 4.0, "alpha": 0.3, "s": 0.5}, 1e-4),
    ]
    for b, tol in cases:
        doc = dict(base, bath=b)
        doc["bath integration error tolerance"] = tol
        inp = D.parse_input(doc)
        assert len(inp.ops) == 1 and inp.seed == 0 and inp.krylov_dim == 6 and inp.nmax_high == 6
        assert inp.nspf_capacity == 4 and inp.minimum_unoccupied == 4
        lo, hi = D.frequency_window(inp)
        m = D.build_model(inp)
        assert sum(len(bl.wk) for bl in m.blocks) == 24 and m.topology.nmodes == len(m.blocks) + 1
        pts = [0.0] if lo < 0 else None
        total = quad(lambda x: float(inp.bath.measure(np.float64(x))), lo, hi, points=pts, limit=400, epsrel=1e-12)[0]
        assert np.sum(math.pi * m.gk ** 2) == pytest.approx(total, rel=1e-9)
        if inp.bath.nonzero_temperature:
            assert lo < 0 and np.any(m.wk < 0)
        else:
            assert lo == 0.0 and np.all(m.wk > 0)


def test_residual_stop_reproduces_the_reference_work_counter():
    """With the Lanczos recurrence ended on the residual estimate (Krylov stop rule 1) the
    oracle's H applications per node on the sudden-cutoff example follow the reference's
    printed counter (55.7, 70.5, 85.4 after three steps) to 5 %, where the full-space
    Expokit scheme counts 156, 182 and 208, and the observables still match the
    reference's to 1e-10."""
    from oracle.oracle import Oracle
    v = _golden()["beta_10/ohmic/spin_boson_sudden"]
    inp = D.parse_input(v["input"])
    m = D.build_model(inp)
    orc = Oracle(m.topology, m.hamiltonian, krylov_dim=inp.krylov_dim, krylov_tol=inp.krylov_tolerance)
    orc.set_krylov_stop(1)
    orc.init_product(inp.psi0, inp.seed)
    orc.set_expansion(m.capacity, spawning_threshold=inp.spawning_parameter,
                      unoccupied_threshold=inp.unoccupied_threshold, minimum_unoccupied=inp.minimum_unoccupied, seed=0)
    for k in (1, 2, 3):
        orc.step(inp.dt)
        row = v["rows"][k]
        vals = np.array([orc.expect(0, op).real for op in inp.ops])
        assert np.max(np.abs(vals - row["values"])) < 1e-10, (k, vals, row["values"])
        nh = orc.nh_applications / m.topology.nnodes
        assert abs(nh - row["nh_per_node"]) < 0.05 * row["nh_per_node"], (k, nh, row["nh_per_node"])
        assert abs(orc.expansion_counts()[1] - row["counts"][1]) <= 3
    with pytest.raises(RuntimeError):
        orc.set_krylov_stop(2)
