"""Host logic of the program layer: observable bookkeeping and basis rotations before sampling
(src/circuit.jl:86-309, src/BraketSimulator.jl:208-219).  No GPU."""
import math

import numpy as np
import pytest

from conftest import bs

O = bs.observables


def _names(ixs):
    return [(type(ix.operator).__name__, ix.target) for ix in ixs]


def _circuit(results, n=3):
    ixs = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    return bs.Circuit(ixs, results)


def test_fix_endianness_swaps_middle_rows_and_columns():
    m = np.arange(16.0).reshape(4, 4)
    f = bs.fix_endianness(m)
    perm = [0, 2, 1, 3]
    assert np.array_equal(f, m[np.ix_(perm, perm)])
    assert np.array_equal(bs.fix_endianness(np.eye(2)), np.eye(2))
    assert np.array_equal(bs.fix_endianness(np.eye(8)), np.eye(8))


def test_standard_basis_rotations():
    assert [type(g).__name__ for g in bs.basis_rotation_gates(O.X())] == ["H"]
    assert [type(g).__name__ for g in bs.basis_rotation_gates(O.Y())] == ["Z", "S", "H"]
    assert bs.basis_rotation_gates(O.Z()) == [] and bs.basis_rotation_gates(O.I()) == []
    (ry,) = bs.basis_rotation_gates(O.H())
    assert type(ry).__name__ == "Ry" and math.isclose(ry.angle[0], -math.pi / 4)


def test_hermitian_rotation_diagonalises():
    rng = np.random.default_rng(3)
    a = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    h = a + a.conj().T
    (u,) = bs.basis_rotation_gates(O.HermitianObservable(h))
    d = u.matrix @ h @ u.matrix.conj().T
    assert np.allclose(d, np.diag(np.diag(d)), atol=1e-12)
    assert np.all(np.diff(np.diag(d).real) >= -1e-12)   # ascending eigenvalues, as eigvecs orders them


def test_per_target_rotations():
    c = _circuit([bs.Expectation(O.X(), (0,)), bs.Sample(O.Y(), (1,)), bs.Probability((2,))])
    assert _names(c.compute_basis_rotation_instructions()) == [
        ("H", (0,)), ("Z", (1,)), ("S", (1,)), ("H", (1,))]


def test_tensor_product_rotations_per_factor():
    tp = O.TensorProduct([O.X(), O.Y(), O.Z()])
    d = bs.tensor_product_index_dict(tp, [4, 2, 7])
    assert [(type(f).__name__, t) for f, t in d.values()] == [("X", (4,)), ("Y", (2,)), ("Z", (7,))]
    c = _circuit([bs.Sample(tp, (0, 1, 2))])
    assert _names(c.compute_basis_rotation_instructions()) == [
        ("H", (0,)), ("Z", (1,)), ("S", (1,)), ("H", (1,))]


def test_tensor_product_with_two_qubit_hermitian_factor():
    rng = np.random.default_rng(5)
    a = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    herm = O.HermitianObservable(a + a.conj().T)
    tp = O.TensorProduct([O.X(), herm])
    d = bs.tensor_product_index_dict(tp, [0, 1, 2])
    assert [(type(f).__name__, t) for f, t in d.values()] == [
        ("X", (0,)), ("HermitianObservable", (1, 2)), ("HermitianObservable", (1, 2))]
    c = _circuit([bs.Expectation(tp, (0, 1, 2))])
    ixs = c.compute_basis_rotation_instructions()
    assert _names(ixs) == [("H", (0,)), ("Unitary", (1, 2))]
    (u,) = bs.basis_rotation_gates(herm)
    assert np.allclose(ixs[1].operator.matrix, bs.fix_endianness(u.matrix))


def test_all_qubit_observable():
    c = _circuit([bs.Sample(O.X(), ())], n=3)
    assert _names(c.compute_basis_rotation_instructions()) == [("H", (0,)), ("H", (1,)), ("H", (2,))]


def test_identity_and_repeats_commute():
    c = _circuit([bs.Expectation(O.I(), (0,)), bs.Expectation(O.X(), (0,)), bs.Variance(O.X(), (0,))])
    assert c.observables_simultaneously_measurable
    assert _names(c.compute_basis_rotation_instructions()) == [("H", (0,))]


def test_noncommuting_observables_drop_rotations():
    c = _circuit([bs.Expectation(O.X(), (0,)), bs.Expectation(O.Z(), (0,))])
    assert not c.observables_simultaneously_measurable
    assert c.compute_basis_rotation_instructions() == []
    # a later observable is not recorded once the set is known not to commute
    c.add_result(bs.Expectation(O.Y(), (1,)))
    assert c.compute_basis_rotation_instructions() == []


def test_all_qubit_observable_conflicts():
    c = _circuit([bs.Sample(O.X(), ()), bs.Sample(O.Y(), ())])
    assert not c.observables_simultaneously_measurable


def test_measured_qubit_checks():
    c = bs.Circuit([bs.Instruction(bs.H(), [0]), bs.Instruction(bs.Measure(), [0])])
    with pytest.raises(ValueError, match="measured qubits"):
        c.add_instruction(bs.Instruction(bs.X(), [0]))
    c.add_instruction(bs.Instruction(bs.X(), [1]))          # other qubits are free
    c.add_instruction(bs.Instruction(bs.Reset(), [0]))
    c.add_instruction(bs.Instruction(bs.X(), [0]))          # after a reset that follows the measure


def test_to_program_rotations_only_with_shots():
    c = _circuit([bs.Sample(O.X(), (0,))])
    assert c.to_program(0).basis_rotation_instructions == []
    p = c.to_program(100)
    assert _names(p.basis_rotation_instructions) == [("H", (0,))]
    assert len(p.instructions) == 3 and len(p.results) == 1
