"""Observables (src/observables.jl:1-241): X, Y, Z, H, I, HermitianObservable,
TensorProduct, Sum, with their diagonalizing gates."""
from __future__ import annotations

import math

import numpy as np

from .gates import H as HGate, Ry, Unitary


class Observable:
    coefficient = 1.0

    def qubit_count(self) -> int:
        return 1


class StandardObservable(Observable):
    label = "?"

    def __init__(self, coefficient: float = 1.0):
        self.coefficient = float(coefficient)

    def __eq__(self, o):
        return type(self) is type(o) and math.isclose(self.coefficient, o.coefficient)

    def __mul__(self, n):
        if isinstance(n, Observable):
            return TensorProduct([self, n])
        return type(self)(float(n) * self.coefficient)

    __rmul__ = __mul__

    def __repr__(self):
        return self.label.upper()

    def eigvals(self):
        return np.array([self.coefficient, -self.coefficient])


class X(StandardObservable):
    label = "x"
    matrix = np.array([[0, 1], [1, 0]], dtype=np.complex128)


class Y(StandardObservable):
    label = "y"
    matrix = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)


class Z(StandardObservable):
    label = "z"
    matrix = np.array([[1, 0], [0, -1]], dtype=np.complex128)


class H(StandardObservable):
    label = "h"
    matrix = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2.0)


class I(StandardObservable):
    label = "i"
    matrix = np.eye(2, dtype=np.complex128)

    def eigvals(self):
        return np.array([self.coefficient, self.coefficient])


class HermitianObservable(Observable):
    def __init__(self, matrix):
        m = np.array(matrix, dtype=np.complex128)
        if m.ndim != 2 or m.shape[0] != m.shape[1] or not np.array_equal(m, m.conj().T):
            raise ValueError("input matrix to HermitianObservable must be Hermitian.")
        self.matrix = m
        self.coefficient = 1.0

    def qubit_count(self):
        return int(round(math.log2(self.matrix.shape[0])))

    def __eq__(self, o):
        return isinstance(o, HermitianObservable) and o.matrix.shape == self.matrix.shape and np.allclose(o.matrix, self.matrix)

    def eigvals(self):
        return np.linalg.eigvalsh(self.matrix)


class TensorProduct(Observable):
    def __init__(self, factors, coefficient: float = 1.0):
        flat = []
        coeff = float(coefficient)
        for f in factors:
            if isinstance(f, str):
                f = {"x": X, "y": Y, "z": Z, "h": H, "i": I}[f.lower()]()
            if isinstance(f, Sum):
                raise ValueError("Sum observable not allowed in TensorProduct.")
            coeff *= f.coefficient
            if isinstance(f, TensorProduct):
                flat.extend(f.factors)
            elif isinstance(f, StandardObservable):
                flat.append(type(f)())
            else:
                flat.append(f)
        self.factors = flat
        self.coefficient = coeff

    def qubit_count(self):
        return sum(f.qubit_count() for f in self.factors)

    def __eq__(self, o):
        return isinstance(o, TensorProduct) and self.factors == o.factors and math.isclose(self.coefficient, o.coefficient)

    def eigvals(self):
        ev = np.array([self.coefficient])
        for f in self.factors:
            ev = np.kron(ev, f.eigvals() if not isinstance(f, StandardObservable) else np.array([1.0, -1.0]) if not isinstance(f, I) else np.array([1.0, 1.0]))
        return ev

    def __repr__(self):
        return " @ ".join(repr(f) for f in self.factors)


class Sum(Observable):
    """Declared by the reference, not evaluated by its simulators."""

    def __init__(self, summands):
        self.summands = list(summands)


def diagonalizing_gates(obs: Observable, targets):
    """src/observables.jl:220-241 -> list of (gate, targets)."""
    from .simulators import Instruction
    targets = [targets] if isinstance(targets, int) else list(targets)
    if isinstance(obs, (I, Z)):
        return []
    if isinstance(obs, H):
        return [Instruction(Ry(-math.pi / 4.0), [t]) for t in targets]
    if isinstance(obs, X):
        return [Instruction(HGate(), [t]) for t in targets]
    if isinstance(obs, Y):
        u = (1 / math.sqrt(2)) * np.array([[1.0, -1j], [1.0, 1j]])
        return [Instruction(Unitary(u), [t]) for t in targets]
    if isinstance(obs, HermitianObservable):
        vecs = np.linalg.eigh(obs.matrix)[1]
        if obs.matrix.shape[0] == 2 ** len(targets):
            return [Instruction(Unitary(vecs), targets)]
        if obs.matrix.shape[0] == 2 and len(targets) > 1:
            return [Instruction(Unitary(vecs), [t]) for t in targets]
        return []
    if isinstance(obs, TensorProduct):
        out = []
        for f, t in zip(obs.factors, targets):
            out.extend(diagonalizing_gates(f, t))
        return out
    raise TypeError(f"no diagonalizing gates for {obs!r}")
