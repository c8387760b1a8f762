"""Density-matrix parity: gates as fused superoperator sweeps, Kraus channels in the
reference's block-diagonal mode and in the full (physical) mode."""
import numpy as np
import pytest

import oracle
from conftest import bs, make_op, random_circuit, rel_err
from golden import reference_kats as K

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("case", K.DM_KATS, ids=lambda c: "+".join(s[0] for s in c[0]))
def test_dm_kats(case):
    ins, n, dm, probs = case
    ops = [make_op(s) for s in ins]
    sim = bs.DensityMatrixSimulator(n, 0).evolve(ops)
    ref = oracle.OracleDM(n).evolve(ops).matrix
    assert rel_err(sim.density_matrix, ref) < TOL
    assert rel_err(sim.density_matrix, dm) < 1e-7
    assert rel_err(sim.probabilities(), probs) < 1e-7


@pytest.mark.parametrize("case", K.SV_KATS, ids=lambda c: "+".join(s[0] for s in c[0]))
def test_dm_runs_sv_kats(case):
    ins, n, sv, probs = case
    ops = [make_op(s) for s in ins]
    sim = bs.DensityMatrixSimulator(n, 0).evolve(ops)
    assert rel_err(sim.density_matrix, oracle.OracleDM(n).evolve(ops).matrix) < TOL
    assert rel_err(sim.probabilities(), probs) < 1e-7


def _noisy(n, depth, rng):
    ops = []
    chans1 = [lambda: bs.Depolarizing(0.05), lambda: bs.AmplitudeDamping(0.1), lambda: bs.BitFlip(0.07),
              lambda: bs.PhaseFlip(0.2), lambda: bs.PhaseDamping(0.3), lambda: bs.GeneralizedAmplitudeDamping(0.2, 0.1),
              lambda: bs.PauliChannel(0.01, 0.02, 0.03)]
    chans2 = [lambda: bs.TwoQubitDepolarizing(0.05), lambda: bs.TwoQubitDephasing(0.1),
              lambda: bs.TwoQubitPauliChannel({"XY": 0.05, "ZZ": 0.1})]
    for ix in random_circuit(n, depth, rng):
        ops.append(ix)
        r = rng.random()
        if r < 0.5:
            ops.append(bs.Instruction(chans1[rng.integers(len(chans1))](), [ix.target[0]]))
        elif r < 0.7 and n >= 2:
            t = [int(x) for x in rng.choice(n, 2, replace=False)]
            ops.append(bs.Instruction(chans2[rng.integers(len(chans2))](), t))
    return ops


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7])
@pytest.mark.parametrize("mode", ["reference", "physical"])
def test_noisy_random(n, mode):
    rng = np.random.default_rng(77 + n)
    ops = _noisy(n, 30, rng)
    sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode).evolve(ops)
    ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops).matrix
    assert rel_err(sim.density_matrix, ref) < TOL


def test_modes_differ_exactly_where_the_reference_skips_coherences():
    # Bell state then BitFlip on q1: the reference leaves <YY> at -1, the full channel gives -0.8
    ops = [bs.Instruction(bs.H(), [0]), bs.Instruction(bs.CNot(), [0, 1]), bs.Instruction(bs.BitFlip(0.1), [1])]
    ref_mode = bs.DensityMatrixSimulator(2, 0, noise_mode="reference").evolve(ops)
    phys = bs.DensityMatrixSimulator(2, 0, noise_mode="physical").evolve(ops)
    yy = bs.observables.TensorProduct([bs.observables.Y(), bs.observables.Y()])
    assert abs(ref_mode.expectation(yy, 0, 1) - (-1.0)) < 1e-12
    assert abs(phys.expectation(yy, 0, 1) - (-0.8)) < 1e-12


def test_kraus_multi_target_and_unitary_conj_side():
    rng = np.random.default_rng(3)
    n = 4
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    q, _ = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))
    ops.append(bs.Instruction(bs.Unitary(q), [3, 0, 2]))
    k0 = np.sqrt(0.9) * np.eye(8)
    k1 = np.sqrt(0.1) * q
    ops.append(bs.Instruction(bs.Kraus([k0, k1]), [1, 3, 0]))
    for mode in ("reference", "physical"):
        sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode).evolve(ops)
        ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops).matrix
        assert rel_err(sim.density_matrix, ref) < TOL


@pytest.mark.parametrize("n", [8, 10])
def test_dm_config_shape(n):
    """Rx/Ry/Rz + CNOT ladder with depolarizing and amplitude damping after every gate
    (the 14-qubit benchmark's structure at oracle size)."""
    rng = np.random.default_rng(n)
    ops = []
    for d in range(3):
        for q in range(n):
            g = [bs.Rx, bs.Ry, bs.Rz][rng.integers(3)](float(rng.uniform(0, 2 * np.pi)))
            ops += [bs.Instruction(g, [q]), bs.Instruction(bs.Depolarizing(1e-3), [q]),
                    bs.Instruction(bs.AmplitudeDamping(5e-3), [q])]
        for q in range(n - 1):
            ops += [bs.Instruction(bs.CNot(), [q, q + 1]), bs.Instruction(bs.TwoQubitDepolarizing(1e-2), [q, q + 1]),
                    bs.Instruction(bs.AmplitudeDamping(5e-3), [q]), bs.Instruction(bs.AmplitudeDamping(5e-3), [q + 1])]
    for mode in ("reference", "physical") if n <= 8 else ("reference",):
        sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode).evolve(ops)
        ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops)
        assert rel_err(sim.density_matrix, ref.matrix) < TOL
        assert rel_err(sim.probabilities(), ref.probabilities()) < TOL
