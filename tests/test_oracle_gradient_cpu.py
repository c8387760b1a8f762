"""The oracle's gradient checker on its own (CPU): the one-pass Pauli expectation agrees with
the reference-style apply-then-dot form, and the FP64 parameter-shift rule agrees with closed
forms and with central finite differences."""
import math

import numpy as np
import pytest

import oracle
from conftest import bs


def test_one_pass_pauli_expectation_matches_apply_then_dot():
    rng = np.random.default_rng(1)
    for n in (1, 3, 9):
        psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        psi /= np.linalg.norm(psi)
        for _ in range(40):
            x, z = int(rng.integers(2 ** n)), int(rng.integers(2 ** n))
            assert abs(oracle.expectation_pauli_fast(psi, n, x, z) - oracle.expectation_pauli_sv(psi, n, x, z)) < 1e-14


def test_parameter_shift_closed_forms():
    # <Z> after Ry(t)|0> = cos t
    t = 0.73
    e, g = oracle.parameter_shift_gradient(1, [bs.Instruction(bs.Ry(t), [0])], [(1.0, {0: "Z"})])
    assert abs(e - math.cos(t)) < 1e-15 and abs(g[0] + math.sin(t)) < 1e-15
    # PhaseShift(t) on |+>: <X> = cos t, d/dt = -sin t; pow_exponent 2 doubles the angle
    ops = [bs.Instruction(bs.H(), [0]), bs.Instruction(bs.PhaseShift(t, pow_exponent=2.0), [0])]
    e, g = oracle.parameter_shift_gradient(1, ops, [(1.0, {0: "X"})])
    assert abs(e - math.cos(2 * t)) < 1e-15 and abs(g[1] + 2 * math.sin(2 * t)) < 1e-14
    # ZZ(t) on |+>|0> acts as Rz(t) on the first qubit: <X0> = cos t
    ops = [bs.Instruction(bs.H(), [0]), bs.Instruction(bs.ZZ(t), [0, 1])]
    e, g = oracle.parameter_shift_gradient(2, ops, [(1.0, {0: "X"})])
    assert abs(e - math.cos(t)) < 1e-15 and abs(g[1] + math.sin(t)) < 1e-15


@pytest.mark.parametrize("n", [3, 5])
def test_parameter_shift_matches_central_differences(n):
    rng = np.random.default_rng(n)
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    for _ in range(2):
        for q in range(n):
            g = [bs.Rx, bs.Ry, bs.Rz, bs.PhaseShift][rng.integers(4)]
            ops.append(bs.Instruction(g(float(rng.uniform(-np.pi, np.pi))), [q]))
        for q in range(n - 1):
            g = [bs.XX, bs.YY, bs.ZZ][rng.integers(3)]
            ops.append(bs.Instruction(g(float(rng.uniform(-np.pi, np.pi))), [q, (q + 2) % n]))
    h = [(float(rng.normal()), {int(q): "XYZ"[rng.integers(3)] for q in rng.choice(n, 2, replace=False)})
         for _ in range(5)]
    e, g = oracle.parameter_shift_gradient(n, ops, h)
    step = 1e-6
    for i, gi in g.items():
        ix = ops[i]
        op = ix.operator
        vals = []
        for s in (step, -step):
            shifted = ops[:i] + [bs.Instruction(type(op)(op.angle[0] + s), ix.target)] + ops[i + 1:]
            psi = oracle.OracleSV(n).evolve(shifted).psi
            vals.append(oracle.hamiltonian_energy(psi, n, h))
        assert abs(gi - (vals[0] - vals[1]) / (2 * step)) < 1e-8
