"""complex64 states: FP32 gate arithmetic (error against the FP64 oracle is reported and
bounded), and FP64-accurate reductions on the stored complex64 values."""
import numpy as np
import pytest

import oracle
from conftest import bs, random_circuit, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [3, 9, 14, 17])
def test_c64_random_circuits_within_fp32_error(n):
    rng = np.random.default_rng(500 + n)
    ops = random_circuit(n, 50, rng)
    sim = bs.StateVectorSimulator(n, 0, precision="c64").evolve(ops)
    ref = oracle.OracleSV(n).evolve(ops).psi
    err = rel_err(sim.state_vector, ref)
    # FP32 rounding per gate, accumulated over 50 gates
    assert err < 2e-5, err


def test_c64_dense_layers_and_fused_sweeps():
    n = 18
    rng = np.random.default_rng(9)
    ops = []
    for layer in range(8):
        for q in range(n):
            a = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
            ops.append(bs.Instruction(bs.Unitary(np.linalg.qr(a)[0]), [q]))
        for q in range(layer % 2, n - 1, 2):
            ops.append(bs.Instruction(bs.CZ(), [q, q + 1]))
    sim = bs.StateVectorSimulator(n, 0, precision="c64").evolve(ops)
    err = rel_err(sim.state_vector, oracle.OracleSV(n).evolve(ops).psi)
    assert err < 2e-5, err


@pytest.mark.parametrize("mode", ["reference", "physical"])
def test_c64_noisy_density_matrix(mode):
    n = 5
    rng = np.random.default_rng(31)
    ops = []
    for ix in random_circuit(n, 25, rng):
        ops.append(ix)
        ops.append(bs.Instruction(bs.Depolarizing(0.05), [ix.target[0]]))
        ops.append(bs.Instruction(bs.AmplitudeDamping(0.02), [ix.target[-1]]))
    sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode, precision="c64").evolve(ops)
    ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops).matrix
    assert rel_err(sim.density_matrix, ref) < 2e-5


def test_c64_reductions_are_fp64_accurate_on_the_stored_values():
    n = 12
    rng = np.random.default_rng(4)
    ops = random_circuit(n, 40, rng)
    sim = bs.StateVectorSimulator(n, 0, precision="c64").evolve(ops)
    v = sim.state_vector                     # exact complex64 values, widened
    p = np.abs(v) ** 2
    assert rel_err(sim.probabilities(), p) < 1e-14
    for _ in range(6):
        x, z = int(rng.integers(0, 2 ** n)), int(rng.integers(0, 2 ** n))
        out = np.empty(1)
        sim._h.call("bs_expectation_pauli", 1, bs._abi.u64ptr(np.array([x], dtype=np.uint64)),
                    bs._abi.u64ptr(np.array([z], dtype=np.uint64)), bs._abi.dptr(np.ones(1)), bs._abi.dptr(out))
        assert abs(out[0] - oracle.expectation_pauli_sv(v.astype(np.complex128), n, x, z)) < 1e-13
    s = bs.StateVectorSimulator(n, 2000, precision="c64")
    s.state_vector = v
    u = rng.random(2000)
    got = s.samples_direct(u, wsum=float(np.sum(p)))
    assert np.sum(got != oracle.sample_direct(p, u, float(np.sum(p)))) <= 2


def test_c64_state_roundtrip_and_copy():
    v = (np.arange(256) + 1j * np.arange(256)[::-1]) / 3000.0
    s = bs.StateVectorSimulator(8, 0, precision="c64")
    s.state_vector = v
    assert np.allclose(s.state_vector, v.astype(np.complex64), rtol=0, atol=0)
    c = s.copy()
    assert np.array_equal(c.state_vector, s.state_vector)


def test_c64_runs_on_qubit_pairs_fold_into_two_bit_gates():
    """Complex64 sweeps fold runs of 1- and 2-qubit gates on the same two qubits (controls in the
    tile, or out of it) into dense 2-bit gates: same result as the oracle within FP32 error."""
    n = 16
    rng = np.random.default_rng(77)
    ops = []
    for _ in range(12):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        c = int(rng.integers(n))
        for ix in (bs.Instruction(bs.H(), [a]), bs.Instruction(bs.CNot(), [a, b]),
                   bs.Instruction(bs.Rz(float(rng.uniform(-3, 3))), [b]), bs.Instruction(bs.CZ(), [b, a]),
                   bs.Instruction(bs.Ry(float(rng.uniform(-3, 3))), [a]), bs.Instruction(bs.Swap(), [a, b]),
                   bs.Instruction(bs.Rx(float(rng.uniform(-3, 3))), [c])):
            ops.append(ix)
        if c not in (a, b):
            ops.append(bs.Instruction(bs.CCNot(), [c, a, b]))
    sim = bs.StateVectorSimulator(n, 0, precision="c64").evolve(ops)
    err = rel_err(sim.state_vector, oracle.OracleSV(n).evolve(ops).psi)
    assert err < 2e-5, err
