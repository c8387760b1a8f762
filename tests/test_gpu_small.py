"""simulate of one small circuit in one round trip (bs_run_small): the whole state vector in one CTA,
then the library's sampler.  Its state and probabilities must match the FP64 oracle to 1e-12 and equal
the usual path's (reinit + evolve + probabilities) to the same bar; its samples must be the ones the
usual path's samples(seed) draws."""
import numpy as np
import pytest

import oracle
from conftest import bs, random_circuit, rel_err

pytestmark = pytest.mark.gpu


def ghz(n):
    return [bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, n)]


def test_ghz10_run_matches_oracle_and_usual_path():
    ops = ghz(10)
    sim = bs.StateVectorSimulator(10, 1000)
    p, s = sim.run(ops, 1000, seed=7)
    ref = oracle.OracleSV(10).evolve(ops).psi
    assert rel_err(sim.state_vector, ref) < 1e-12
    assert np.max(np.abs(p - np.abs(ref) ** 2)) < 1e-15
    assert set(np.unique(s)) <= {0, 1023} and 350 < np.sum(s == 0) < 650
    usual = bs.StateVectorSimulator(10, 1000)
    usual.evolve(ops)
    assert np.array_equal(usual.probabilities(), p)
    assert np.array_equal(usual.samples(7), s)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 11, 12])
@pytest.mark.parametrize("pows", [False, True])
def test_run_random_circuits(n, pows):
    """Every gate family (1-4 target dense, controlled, diagonal, monomial, swaps, powers)."""
    rng = np.random.default_rng(300 + 10 * n + pows)
    ops = random_circuit(n, 50, rng, pows=pows)
    sim = bs.StateVectorSimulator(n, 500)
    p, s = sim.run(ops, 500, seed=3)
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(sim.state_vector, ref) < 1e-12
    assert np.max(np.abs(p - np.abs(ref) ** 2)) < 1e-13
    usual = bs.StateVectorSimulator(n, 500).evolve(ops)
    assert rel_err(usual.probabilities(), p) < 1e-12
    assert np.all(np.abs(ref[s]) ** 2 > 1e-14)


@pytest.mark.parametrize("n", [4, 9, 12])
def test_run_permutation_heavy_circuits(n):
    """Long runs of permutation gates (CNOT chains, SWAPs, X, Y, CCNOT, controlled Y and their mixes)
    after a dense layer: the state must be the usual path's, since such gates only move and negate
    values, and the oracle's to 1e-12."""
    rng = np.random.default_rng(40 + n)
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)] + [bs.Instruction(bs.Ry(0.3 + 0.1 * q), [q]) for q in range(n)]
    for _ in range(60):
        qs = [int(x) for x in rng.choice(n, min(3, n), replace=False)]
        r = int(rng.integers(7))
        if r == 0:
            ops.append(bs.Instruction(bs.CNot(), qs[:2]))
        elif r == 1:
            ops.append(bs.Instruction(bs.Swap(), qs[:2]))
        elif r == 2:
            ops.append(bs.Instruction(bs.X(), qs[:1]))
        elif r == 3:
            ops.append(bs.Instruction(bs.Y(), qs[:1]))
        elif r == 4 and n >= 3:
            ops.append(bs.Instruction(bs.CCNot(), qs[:3]))
        elif r == 5:
            ops.append(bs.Instruction(bs.CY(), qs[:2]))
        else:
            ops.append(bs.Instruction(bs.CNot(), [qs[0], (qs[0] + 1) % n]))
    sim = bs.StateVectorSimulator(n, 400)
    p, s = sim.run(ops, 400, seed=4)
    usual = bs.StateVectorSimulator(n, 400).evolve(ops)
    assert rel_err(sim.state_vector, usual.state_vector) < 1e-15
    assert rel_err(p, usual.probabilities()) < 1e-15
    assert np.array_equal(sim.samples(4), s)     # the same draws from the state the run left
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(sim.state_vector, ref) < 1e-12
    assert np.all(np.abs(ref[s]) ** 2 > 1e-14)


def test_run_reuses_the_plan_only_for_the_same_list():
    """The plan of the last list is reused when the next list has the same op structs and matrix
    values; a changed angle, target or length is planned afresh.  Every result against the oracle."""
    sim = bs.StateVectorSimulator(8, 300)
    base = ghz(8)
    lists = [base + [bs.Instruction(bs.Ry(0.3), [2])], base + [bs.Instruction(bs.Ry(0.3), [2])],
             base + [bs.Instruction(bs.Ry(0.7), [2])], base + [bs.Instruction(bs.Ry(0.7), [5])],
             base, base + [bs.Instruction(bs.Ry(0.3), [2])]]
    first = None
    for i, ops in enumerate(lists):
        p, s = sim.run(ops, 300, seed=5)
        ref = oracle.OracleSV(8).evolve(ops).psi
        assert rel_err(sim.state_vector, ref) < 1e-12
        assert np.max(np.abs(p - np.abs(ref) ** 2)) < 1e-14
        assert np.array_equal(sim.samples(5), s)
        if i == 0:
            first = (p, s)
        if i in (1, 5):
            assert np.array_equal(p, first[0]) and np.array_equal(s, first[1])
        st = sim.last_stats()
        assert st["kernel_launches"] == 1 and st["gates"] >= 1 and st["gpu_ms"] > 0


def test_run_repeats_and_resets():
    """Each call starts from |0...0> whatever the handle held; the same seed gives the same shots."""
    ops = ghz(6) + [bs.Instruction(bs.Ry(0.4), [3])]
    sim = bs.StateVectorSimulator(6, 200)
    sim.evolve([bs.Instruction(bs.X(), [q]) for q in range(6)])
    p1, s1 = sim.run(ops, 200, seed=11)
    p2, s2 = sim.run(ops, 200, seed=11)
    assert np.array_equal(p1, p2) and np.array_equal(s1, s2)
    ref = oracle.OracleSV(6).evolve(ops).psi
    assert np.max(np.abs(p1 - np.abs(ref) ** 2)) < 1e-14


def test_run_falls_back_for_wide_gates_and_complex64():
    """A 5-target dense gate has no in-tile kernel, and complex64 states take the usual kernels:
    the results are still exact and the samples are samples(seed)'s."""
    rng = np.random.default_rng(9)
    a = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    u, _ = np.linalg.qr(a)
    ops = ghz(7) + [bs.Instruction(bs.Unitary(u), [0, 2, 3, 5, 6])]
    sim = bs.StateVectorSimulator(7, 300)
    p, s = sim.run(ops, 300, seed=2)
    ref = oracle.OracleSV(7).evolve(ops).psi
    assert np.max(np.abs(p - np.abs(ref) ** 2)) < 1e-13
    usual = bs.StateVectorSimulator(7, 300).evolve(ops)
    assert np.array_equal(usual.samples(2), s)
    p2, s2 = sim.run(ops, 300, seed=2)          # the same list again: the usual path again
    assert np.array_equal(p2, p) and np.array_equal(s2, s)
    s64 = bs.StateVectorSimulator(7, 300, precision="c64")
    p64, q64 = s64.run(ops, 300, seed=2)
    assert np.max(np.abs(p64 - np.abs(ref) ** 2)) < 1e-6


def test_simulate_uses_the_small_path_with_the_same_measurements():
    prog = bs.Program(ghz(5), [])
    r = bs.simulate(bs.StateVectorSimulator(5, 0), prog, 400, seed=5)
    m = r["measurements"]
    assert m.shape == (400, 5)
    assert np.all((m == 0).all(axis=1) | (m == 1).all(axis=1))
