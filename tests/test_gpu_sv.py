"""State-vector parity: GB300 engine vs the reference's golden vectors and vs the
CPU oracle.  Amplitudes must agree within 1e-12 relative (norm-wise, Julia's
isapprox definition) with the FP64 oracle."""
import math

import numpy as np
import pytest

import oracle
from conftest import bs, make_op, random_circuit, rel_err
from golden import reference_kats as K

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("case", K.SV_KATS + K.CUSTOM_KATS, ids=lambda c: "+".join(s[0] for s in c[0]))
def test_sv_kats(case):
    ins, n, sv, probs = case
    ops = [make_op(s) for s in ins]
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    got = sim.state_vector
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(got, ref) < TOL
    assert rel_err(got, sv) < 1e-7
    if probs is not None:
        assert rel_err(sim.probabilities(), probs) < 1e-7


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 11, 13, 16])
@pytest.mark.parametrize("pows", [False, True])
def test_random_circuits(n, pows):
    rng = np.random.default_rng(1000 * n + pows)
    ops = random_circuit(n, 60 if n < 13 else 40, rng, pows=pows)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(sim.state_vector, ref) < TOL


@pytest.mark.parametrize("n", [14, 18, 20])
def test_deep_layers(n):
    """Dense SU(2) layers with CZ bricks (the 30-qubit benchmark's structure) at oracle size."""
    rng = np.random.default_rng(n)
    ops = []
    for layer in range(12):
        for q in range(n):
            a = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
            u, _ = np.linalg.qr(a)
            ops.append(bs.Instruction(bs.Unitary(u), [q]))
        for q in range(layer % 2, n - 1, 2):
            ops.append(bs.Instruction(bs.CZ(), [q, q + 1]))
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(sim.state_vector, ref) < TOL
    st = sim.last_stats()
    assert st["sweeps"] < len(ops)   # gates were fused into tiles


@pytest.mark.parametrize("n", [12, 16, 21])
def test_one_target_sweeps_with_controls_and_diagonals(n):
    """Sweeps whose non-diagonal gates are all 1-target: in-tile and out-of-tile controls, negated
    controls, monomials and diagonals on far qubits."""
    rng = np.random.default_rng(n + 100)
    ops = []
    for _ in range(80):
        q = int(rng.integers(n))
        r = int(rng.integers(6))
        if r == 0:
            a = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
            ops.append(bs.Instruction(bs.Unitary(np.linalg.qr(a)[0]), [q]))
        elif r == 1:
            ops.append(bs.Instruction([bs.H(), bs.Rx(0.3), bs.Ry(-1.2), bs.V(), bs.S(), bs.T()][rng.integers(6)], [q]))
        elif r == 2:
            c = int(rng.choice([x for x in range(n) if x != q]))
            ops.append(bs.Instruction(bs.CNot(), [c, q]))
        elif r == 3:
            c1, c2 = [int(x) for x in rng.choice([x for x in range(n) if x != q], 2, replace=False)]
            ops.append(bs.Instruction(bs.Control(bs.U(0.4, 0.2, -0.7), (0, 1)), [c1, c2, q]))
        elif r == 4:
            c = int(rng.choice([x for x in range(n) if x != q]))
            ops.append(bs.Instruction([bs.CZ(), bs.CPhaseShift(0.7), bs.ZZ(0.2)][rng.integers(3)], [c, q]))
        else:
            ops.append(bs.Instruction(bs.Rz(float(rng.normal())), [q]))
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    assert rel_err(sim.state_vector, oracle.OracleSV(n).evolve(ops).psi) < TOL


def test_ghz10():
    ops = [bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, 10)]
    sim = bs.StateVectorSimulator(10, 1000).evolve(ops)
    p = sim.probabilities()
    exp = np.zeros(1024)
    exp[0] = exp[-1] = 0.5
    assert np.allclose(p, exp, atol=1e-15)
    s = sim.samples(seed=3)
    assert s.shape == (1000,) and set(np.unique(s)) <= {0, 1023}
    assert 400 < np.sum(s == 0) < 600


@pytest.mark.parametrize("n", [4, 8, 12, 16, 20])
def test_qft_uniform(n):
    # test/test_sv_simulator.jl:360-384
    ops = []
    for t in range(n):
        ops.append(bs.Instruction(bs.H(), [t]))
        ang = math.pi / 2
        for c in range(t + 1, n):
            ops.append(bs.Instruction(bs.CPhaseShift(ang), [c, t]))
            ang /= 2
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    assert rel_err(sim.probabilities(), np.full(2 ** n, 1 / 2 ** n)) < 1e-12


@pytest.mark.parametrize("nq", [1, 2, 3, 4])
def test_gphase_and_control_gphase(nq):
    phi = 2.12
    hs = [bs.Instruction(bs.H(), [q]) for q in range(nq)]
    for g in (bs.GPhase(nq, phi), bs.Control(bs.GPhase(nq, phi), (0,) * nq), bs.MultiRZ(phi)):
        ops = hs + [bs.Instruction(g, list(range(nq)))]
        sim = bs.StateVectorSimulator(nq, 0).evolve(ops)
        assert rel_err(sim.state_vector, oracle.OracleSV(nq).evolve(ops).psi) < TOL


def test_controls_negctrl_and_unitary_big():
    rng = np.random.default_rng(5)
    n = 9
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    ops.append(bs.Instruction(bs.Control(bs.U(0.3, 0.2, 0.1), (0,)), [7, 2]))
    ops.append(bs.Instruction(bs.Control(bs.Ry(0.7), (1, 0)), [0, 8, 4]))
    ops.append(bs.Instruction(bs.Control(bs.Swap(), (1,)), [3, 1, 6]))
    q, _ = np.linalg.qr(rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32)))
    ops.append(bs.Instruction(bs.Unitary(q), [6, 0, 3, 8, 2]))       # 5 targets: sorted convention
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    assert rel_err(sim.state_vector, oracle.OracleSV(n).evolve(ops).psi) < TOL


def test_inverse_roundtrip():
    # test/test_gate_operations.jl: g then inv(g) is the identity on a superposition
    from conftest import GATES_1, GATES_A
    nq = 4
    hs = [bs.Instruction(bs.H(), [q]) for q in range(nq)]
    base = bs.StateVectorSimulator(nq, 0).evolve(hs).state_vector
    gates = [GATES_1[n]() for n in ["x", "y", "z", "h", "s", "si", "t", "ti", "v", "vi", "cnot", "cy", "cz", "cv", "swap", "iswap", "ecr"]]
    gates += [GATES_A[n](0.23) for n in ["rx", "ry", "rz", "phaseshift", "gpi", "gpi2", "xx", "yy", "zz", "xy", "pswap", "cphaseshift", "single_excitation"]]
    for g in gates:
        t = list(range(g.qubit_count()))
        sim = bs.StateVectorSimulator(nq, 0).evolve(hs + [bs.Instruction(g, t), bs.Instruction(g.inv(), t)])
        assert rel_err(sim.state_vector, base) < 1e-12, g


def test_errors_are_reported_not_faulted():
    sim = bs.StateVectorSimulator(3, 0)
    with pytest.raises(bs._abi.BraketGB300Error):
        sim.evolve([bs.Instruction(bs.H(), [5])])
    with pytest.raises(bs._abi.BraketGB300Error):
        sim.evolve([bs.Instruction(bs.CNot(), [1, 1])])
    # handle still usable
    sim.evolve([bs.Instruction(bs.X(), [0])])
    assert abs(sim.state_vector[4] - 1) < 1e-15


def test_zero_and_one_qubit():
    sim = bs.StateVectorSimulator(0, 10)
    assert np.allclose(sim.state_vector, [1.0])
    assert np.allclose(sim.probabilities(), [1.0])
    assert list(sim.samples(seed=1)) == [0] * 10
    sim.reinit(1, 0)
    sim.evolve([bs.Instruction(bs.Rx(0.15), [0])])
    assert rel_err(sim.state_vector, [0.99718882, -0.07492971j]) < 1e-7


def test_reinit_copy_copyto():
    # test/test_sv_simulator.jl: similar, copy and copyto!
    sim = bs.StateVectorSimulator(10, 0)
    v = np.exp(1j * np.arange(1024)) / 32
    sim.state_vector = v
    c = sim.copy()
    assert rel_err(c.state_vector, v) == 0
    d = bs.StateVectorSimulator(10, 0).copyto(sim)
    assert rel_err(d.state_vector, v) == 0
    sim.reinit(10, 5)
    assert sim.state_vector[0] == 1 and np.count_nonzero(sim.state_vector) == 1


@pytest.mark.parametrize("n,precision,tol", [(6, "c128", 1e-12), (13, "c128", 1e-12), (23, "c128", 1e-12),
                                             (13, "c64", 2e-5)])
def test_swaps_relabel_qubits(n, precision, tol):
    """SWAP gates move no data (the evolve relabels later gates and restores the order at the end):
    the state still matches the oracle, with swaps chained, repeated, and mixed with every gate kind."""
    rng = np.random.default_rng(200 + n)
    ops = []
    for _ in range(6 * n):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        ops.append(bs.Instruction(bs.Swap(), [a, b]))
        if rng.random() < 0.5:
            ops.append(bs.Instruction(bs.Swap(), [b, a]))
    mixed = random_circuit(n, 4 * n, rng)
    out = []
    for k, ix in enumerate(ops):
        out.append(ix)
        if k < len(mixed):
            out.append(mixed[k])
    sim = bs.StateVectorSimulator(n, 0, precision=precision)
    if n <= 13:
        ref = oracle.OracleSV(n).evolve(out).psi
        sim.evolve(out)
        assert rel_err(sim.state_vector, ref) < tol
    else:
        # at 23 qubits: evolve forward, then the inverse circuit, back to |0...0>
        sim.evolve(out + [bs.Instruction(ix.operator ** -1, list(ix.target)) for ix in reversed(out)])
        psi = sim.state_vector
        e0 = np.zeros_like(psi)
        e0[0] = 1.0
        assert rel_err(psi, e0) < tol


def test_swaps_in_density_matrix_with_reference_channels():
    """Relabeling on a density matrix, across a 3-target reference-mode channel (applied directly,
    so the order is restored first)."""
    n = 5
    rng = np.random.default_rng(17)
    ops = []
    for _ in range(12):
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        ops.append(bs.Instruction(bs.Swap(), [a, b]))
        ops.append(bs.Instruction(bs.Rx(float(rng.uniform(-3, 3))), [a]))
        ops.append(bs.Instruction(bs.CNot(), [b, a]))
    ks = [np.sqrt(0.9) * np.eye(8), np.sqrt(0.1) * np.kron(np.kron([[0, 1], [1, 0]], np.eye(2)), [[1, 0], [0, -1]])]
    ops.insert(10, bs.Instruction(bs.Kraus([k.astype(np.complex128) for k in ks]), [0, 2, 4]))
    for mode in ("reference", "physical"):
        sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode)
        sim.evolve(ops)
        ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops).matrix
        assert rel_err(sim.density_matrix, ref) < 1e-12


def test_bounded_wait_gives_up_and_the_handle_stays_usable():
    """Failure detection without a fault: a wait on a barrier that nothing completes gives up after
    its limit, the kernel raises the device flag and returns, the call reports BS_ERR_TIMEOUT, and the
    same handle then simulates correctly."""
    import oracle
    sim = bs.StateVectorSimulator(8, 0)
    with pytest.raises(bs._abi.BraketGB300Error) as e:
        sim._h.call("bs_selftest_wait_timeout", 0.01)
    assert e.value.code == bs._abi.BS_ERR_TIMEOUT
    ops = random_circuit(8, 30, np.random.default_rng(41))
    sim.evolve(ops)
    ref = oracle.OracleSV(8).evolve(ops).psi
    assert np.linalg.norm(sim.state_vector - ref) <= 1e-12 * np.linalg.norm(ref)
