"""The spin-boson driver on the device against the reference's own example outputs
(tests/golden/driver_examples.json): the first rows of beta_10/ohmic/spin_boson_debye
(343 blocks of up to 216 states, 687 nodes, bonds growing from 8 towards 64) and of
zero_temperature/subohmic/spin_boson_exponential (256 blocks of up to 900 states, the
reference's own capacities 64 / 16), and the command-line entry writing the reference's
columns.

Tolerances are those the oracle meets on the same inputs on the CPU
(tests/test_driver.py): the reference picks expansion directions with a 12-vector Krylov
eigensolver and the device library an exact one, so the states drift apart slowly -- by
3e-9 / 5e-8 / 3e-7 over the first three steps of the Debye case and by 3e-11 / 3e-10 over
the first two of the sub-ohmic one; the sudden-cutoff case agrees to 1e-11 with identical
expansion counts."""
import json
import os

import numpy as np
import pytest

from ttns_lib_gb300 import driver as D

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "driver_examples.json")


def _case(name):
    with open(GOLDEN) as f:
        return json.load(f)[name]


def _check_rows(r, g, tols, count_tol):
    for k, tol in enumerate(tols):
        line = r.step()
        row = g["rows"][k + 1]
        assert abs(r.t - row["t"]) < 1e-12  # printed with 16 digits
        vals = np.array(r.observables())
        assert np.max(np.abs(vals - np.array(row["values"]))) < tol, (k, vals, row["values"])
        one, two = r.tdvp.expansion_counts()
        assert one == row["counts"][0]
        assert abs(two - row["counts"][1]) <= count_tol * row["counts"][1], (k, two, row["counts"])
        f = line.split()
        assert abs(float(f[0]) - row["t"]) < 1e-12 and len(f) == len(g["text"][1].split())
        if row["hrank"] and k == 0:
            # after the first step 96 % of the oracle's bonds equal the reference's; later
            # steps drift further apart (83 % after the second), so only the first is checked
            hr = r.hrank()
            ref = np.array(row["hrank"])
            assert np.mean(hr == ref) > 0.9 and np.max(np.abs(hr - ref)) <= 3, k


def test_debye_finite_temperature_example():
    g = _case("beta_10/ohmic/spin_boson_debye")
    inp = D.parse_input(g["input"])
    r = D.SpinBosonRun(inp, device=0)
    assert r.first_row() == g["text"][0]
    _check_rows(r, g, [1e-8, 2e-7, 1e-6], 0.05)


def test_subohmic_zero_temperature_example():
    g = _case("zero_temperature/subohmic/spin_boson_exponential")
    inp = D.parse_input(g["input"])
    m = D.build_model(inp)
    assert np.all(m.capacity <= D.MAX_BOND)
    r = D.SpinBosonRun(inp, m, device=0)
    assert r.first_row() == g["text"][0]
    _check_rows(r, g, [1e-9, 1e-8], 0.01)


def test_command_line_writes_the_reference_columns(tmp_path):
    g = _case("beta_10/ohmic/spin_boson_sudden")
    path = tmp_path / "sb.in"
    out = tmp_path / "sb.out"
    doc = dict(g["input"])
    doc["output file"] = str(out)
    path.write_text(json.dumps(doc))
    assert D.main([str(path), "--steps", "2"]) == 0
    lines = out.read_text().splitlines()
    assert lines[0] + "\n" == g["text"][0]
    assert len(lines) == 4 and lines[-1].startswith("nh_app: ")
    for k in (1, 2):
        f = lines[k].split()
        row = g["rows"][k]
        assert abs(float(f[0]) - row["t"]) < 1e-12
        assert np.max(np.abs(np.array([float(x) for x in f[1:5]]) - row["values"])) < 1e-9
        assert abs(int(f[6]) - row["counts"][1]) <= 0.01 * row["counts"][1]
        assert len(f) == len(g["text"][1].split())
    bad = tmp_path / "bad.in"
    doc.pop("Hsys")
    bad.write_text(json.dumps(doc))
    assert D.main([str(bad)]) == 1


def test_sparse_block_operators_match_the_oracle():
    """A 16-mode version of the sudden-cutoff example (blocks of 100 states, whose H0 and
    coupling go through the device's CSR contractions) against the oracle (dense)."""
    from oracle.oracle import Oracle
    g = _case("beta_10/ohmic/spin_boson_sudden")
    doc = dict(g["input"])
    doc["nmodes"] = 16
    inp = D.parse_input(doc)
    m = D.build_model(inp)
    r = D.SpinBosonRun(inp, m, device=0)
    orc = Oracle(m.topology, m.hamiltonian, krylov_dim=inp.krylov_dim, krylov_tol=inp.krylov_tolerance)
    orc.init_product(inp.psi0, inp.seed)
    orc.set_expansion(m.capacity, spawning_threshold=inp.spawning_parameter,
                      unoccupied_threshold=inp.unoccupied_threshold, minimum_unoccupied=inp.minimum_unoccupied, seed=0)
    for _ in range(2):
        r.step()
        orc.step(inp.dt)
        vals = np.array(r.observables())
        ref = np.array([orc.expect(0, op).real for op in inp.ops])
        assert np.max(np.abs(vals - ref)) < 1e-10
        assert np.array_equal(r.hrank(), orc.hrank()[1:])


def test_residual_stop_follows_the_reference_work_counter():
    """Krylov stop rule 1 on the device: the sudden-cutoff example's H applications per node
    follow the reference's printed counter to 8 % (the oracle with the same rule sits 4-5 %
    above it, the full-space rule about three times as high) while the observables keep
    their 1e-10 agreement."""
    g = _case("beta_10/ohmic/spin_boson_sudden")
    inp = D.parse_input(g["input"])
    r = D.SpinBosonRun(inp, device=0, krylov_stop=1)
    for k in (1, 2, 3):
        r.step()
        row = g["rows"][k]
        assert np.max(np.abs(np.array(r.observables()) - row["values"])) < 1e-10, k
        nh = r.tdvp.nh_applications() / r.nnodes
        assert abs(nh - row["nh_per_node"]) < 0.08 * row["nh_per_node"], (k, nh, row["nh_per_node"])


def test_whole_sudden_cutoff_run():
    """The reference's printed run of beta_10/ohmic/spin_boson_sudden on the device, its
    first 40 steps (to t = 0.2, bonds growing past 40; the whole 80 printed steps take 8
    minutes on GB300, more than the GPU suite can give one test): every row's observables
    within 1e-6 of the reference's.  The oracle, checked the same way on the CPU with the
    residual stop rule, stays within 8e-8 at every row of the whole run."""
    g = _case("beta_10/ohmic/spin_boson_sudden")
    traj = g["trajectory"]
    inp = D.parse_input(g["input"])
    r = D.SpinBosonRun(inp, device=0)
    worst = 0.0
    for k in range(1, min(len(traj), 41)):
        r.step()
        assert abs(r.t - traj[k][0]) < 1e-12  # printed with 16 digits
        worst = max(worst, float(np.max(np.abs(np.array(r.observables()) - traj[k][1:5]))))
    assert worst < 1e-6, worst


def test_debye_run_with_growing_bonds():
    """The first 10 printed steps of the reference's beta_10/ohmic/spin_boson_debye run (to
    t = 0.05; the whole printed run, 36 steps to t = 0.18 with the reference's top bond
    reaching 161, takes longer than the GPU suite can spend on one test): the bonds grow
    past 32 through the expansion's device eigensolver.  Every row's observables within
    1e-5 of the reference's (both runs are converged to the spawning threshold, and the
    two expansions choose their directions differently, so the trajectories part slowly:
    the oracle stays within 1.2e-6 over these steps).  Bonds wider than 64 are covered by
    tests/test_zzz_wide_gpu.py."""
    g = _case("beta_10/ohmic/spin_boson_debye")
    traj = g["trajectory"]
    inp = D.parse_input(g["input"])
    r = D.SpinBosonRun(inp, device=0)
    worst = 0.0
    for k in range(1, min(len(traj), 11)):
        r.step()
        assert abs(r.t - traj[k][0]) < 1e-12
        worst = max(worst, float(np.max(np.abs(np.array(r.observables()) - traj[k][1:5]))))
    assert worst < 1e-5, worst
    assert r.hrank().max() > 32
