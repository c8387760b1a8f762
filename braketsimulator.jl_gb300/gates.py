"""Gate types and their matrices, mirroring BraketSimulator.jl's operator model.

Matrices follow ``matrix_rep`` / ``matrix_rep_raw`` (src/gate_kernels.jl:225-478,
src/custom_gates.jl:41-360) including the reference's handling of the
``pow_exponent`` of each gate family.  Two-qubit matrices are written in the
reference's 2-target kernel convention (matrix index bit0 <-> first target,
src/gate_kernels.jl:555-571), which is why e.g. ``CPhaseShift01`` is
``diag(1, 1, e^{i phi}, 1)``.

``lower_gate`` restates the dispatch of ``apply_gate!`` (src/gate_kernels.jl:675-732,
src/custom_gates.jl:381-416): it decides which reference kernel a gate would reach
and returns the matrix, controls and target-convention flag that make the GB300
engine apply exactly that operation.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi

SQ2 = 1.0 / math.sqrt(2.0)


# --------------------------------------------------------------------------- matrix powers
def _is_integer(x: float) -> bool:
    return float(x).is_integer()


def _mat_pow(m: np.ndarray, p: float) -> np.ndarray:
    """A^p as LinearAlgebra computes it: integer powers by repeated product,
    Hermitian matrices by eigendecomposition with principal complex powers,
    others through the complex Schur form."""
    m = np.asarray(m, dtype=np.complex128)
    if _is_integer(p):
        e = int(p)
        if e >= 0:
            return np.linalg.matrix_power(m, e)
        return np.linalg.matrix_power(np.linalg.inv(m), -e)
    if np.allclose(m, np.diag(np.diag(m)), atol=0.0, rtol=0.0):
        return np.diag(np.power(np.diag(m).astype(np.complex128), p))
    if np.array_equal(m, m.conj().T):
        w, v = np.linalg.eigh(m)
        return (v * np.power(w.astype(np.complex128), p)) @ v.conj().T
    import scipy.linalg as sla
    t, z = sla.schur(m, output="complex")
    if np.allclose(t, np.diag(np.diag(t)), atol=1e-14, rtol=0.0):
        return (z * np.power(np.diag(t), p)) @ z.conj().T
    return sla.fractional_matrix_power(m, p)


def _sqrtm(m: np.ndarray) -> np.ndarray:
    return _mat_pow(m, 0.5)


def _eye(q: int) -> np.ndarray:
    return np.eye(2 ** q, dtype=np.complex128)


# --------------------------------------------------------------------------- base classes
class Operator:
    """Anything an Instruction can carry (reference src/operators.jl:131-149)."""


class QuantumOperator(Operator):
    pass


class Gate(QuantumOperator):
    """Gate with a ``pow_exponent`` (src/gates.jl:6-130)."""
    n_angles = 0
    qc = 1
    name = "gate"

    def __init__(self, *angles: float, pow_exponent: float = 1.0):
        if len(angles) != self.n_angles:
            raise ValueError(f"{type(self).__name__} takes {self.n_angles} angle(s)")
        self.angle = tuple(float(a) for a in angles)
        self.pow_exponent = float(pow_exponent)

    def qubit_count(self) -> int:
        return self.qc

    def __pow__(self, n: float):
        return type(self)(*self.angle, pow_exponent=self.pow_exponent * float(n))

    def inv(self):
        return type(self)(*self.angle, pow_exponent=-self.pow_exponent)

    def __eq__(self, other):
        return type(self) is type(other) and self.angle == other.angle and self.pow_exponent == other.pow_exponent

    def __repr__(self):
        a = ", ".join(repr(x) for x in self.angle)
        return f"{type(self).__name__}({a}{', ' if a else ''}pow={self.pow_exponent})"

    # raw matrix at the gate's own angles
    def raw(self) -> np.ndarray:
        raise NotImplementedError

    def matrix_rep(self) -> np.ndarray:
        """Generic rule of src/gate_kernels.jl:471-478."""
        n = self.pow_exponent
        if n == 1:
            return self.raw()
        if n == 0.5:
            return _sqrtm(self.raw())
        if n == -0.5:
            return np.linalg.inv(_sqrtm(self.raw()))
        return _mat_pow(self.raw(), n)


def _c(rows) -> np.ndarray:
    return np.array(rows, dtype=np.complex128)


# --------------------------------------------------------------------------- fixed gates
class I(Gate):
    name = "i"

    def raw(self):
        return _eye(1)

    def matrix_rep(self):
        return _eye(1)


class _EvenOddGate(Gate):
    """Y, H, Swap, CNot, CY, CZ, CCNot, CSwap, GPi, ECR (src/gate_kernels.jl:243-252)."""

    def matrix_rep(self):
        n = self.pow_exponent
        if _is_integer(n) and int(n) % 2 == 0:
            return _eye(self.qc)
        if _is_integer(n):
            return self.raw()
        return _mat_pow(self.raw(), n)


class H(_EvenOddGate):
    name = "h"

    def raw(self):
        return _c([[SQ2, SQ2], [SQ2, -SQ2]])


class Y(_EvenOddGate):
    name = "y"

    def raw(self):
        return _c([[0, -1j], [1j, 0]])


class X(Gate):
    """X and Z add the square-root special case (src/gate_kernels.jl:254-264)."""
    name = "x"

    def raw(self):
        return _c([[0, 1], [1, 0]])

    def half(self):
        return V().raw()

    def matrix_rep(self):
        n = self.pow_exponent
        if _is_integer(n) and int(n) % 2 == 0:
            return _eye(1)
        if _is_integer(n):
            return self.raw()
        if n == 0.5:
            return self.half()
        return _mat_pow(self.raw(), n)


class Z(X):
    name = "z"

    def raw(self):
        return _c([[1, 0], [0, -1]])

    def half(self):
        return S().raw()


class _Mod4Gate(Gate):
    """V, Vi, S, Si: exponent taken mod 4 (src/gate_kernels.jl:350-371)."""
    fwd = None
    back = None
    sq = None

    def matrix_rep(self):
        n = self.pow_exponent
        if _is_integer(n):
            r = int(n) % 4
            if r == 0:
                return _eye(1)
            if r == 1:
                return self.raw()
            if r == 2:
                return self.sq().raw()
            return self.back().raw()
        return _mat_pow(self.raw(), n)


class V(_Mod4Gate):
    name = "v"

    def raw(self):
        return _c([[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]])


class Vi(_Mod4Gate):
    name = "vi"

    def raw(self):
        return _c([[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]])


class S(_Mod4Gate):
    name = "s"

    def raw(self):
        return _c([[1, 0], [0, 1j]])


class Si(_Mod4Gate):
    name = "si"

    def raw(self):
        return _c([[1, 0], [0, -1j]])


V.sq, V.back = X, Vi
Vi.sq, Vi.back = X, V
S.sq, S.back = Z, Si
Si.sq, Si.back = Z, S


class T(Gate):
    name = "t"

    def raw(self):
        return _c([[1, 0], [0, np.exp(1j * math.pi / 4.0)]])

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(1)
        if n == 1:
            return self.raw()
        if n == -1:
            return Ti().raw()
        return PhaseShift(n * math.pi / 4).matrix_rep()


class Ti(Gate):
    name = "ti"

    def raw(self):
        return _c([[1, 0], [0, np.exp(-1j * math.pi / 4.0)]])

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(1)
        if n == 1:
            return self.raw()
        if n == -1:
            return T().raw()
        return PhaseShift(-n * math.pi / 4).matrix_rep()


class CNot(_EvenOddGate):
    name = "cnot"
    qc = 2

    def raw(self):
        return _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])


class CY(_EvenOddGate):
    name = "cy"
    qc = 2

    def raw(self):
        return _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]])


class CZ(_EvenOddGate):
    name = "cz"
    qc = 2

    def raw(self):
        return _c(np.diag([1, 1, 1, -1]))


class CCNot(_EvenOddGate):
    name = "ccnot"
    qc = 3

    def raw(self):
        m = np.eye(8, dtype=np.complex128)
        m[6, 6] = m[7, 7] = 0
        m[6, 7] = m[7, 6] = 1
        return m


class CSwap(_EvenOddGate):
    name = "cswap"
    qc = 3

    def raw(self):
        m = np.eye(8, dtype=np.complex128)
        m[5, 5] = m[6, 6] = 0
        m[5, 6] = m[6, 5] = 1
        return m


def _swaplike(factor) -> np.ndarray:
    return _c([[1, 0, 0, 0], [0, 0, factor, 0], [0, factor, 0, 0], [0, 0, 0, 1]])


class Swap(_EvenOddGate):
    name = "swap"
    qc = 2

    def raw(self):
        return _swaplike(1.0)


class ISwap(Gate):
    name = "iswap"
    qc = 2

    def raw(self):
        return _swaplike(1j)

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw()
        if n == -1:
            return _swaplike(-1j)
        return _mat_pow(self.raw(), n)


class CV(Gate):
    name = "cv"
    qc = 2

    def raw(self):
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = V().raw()
        return m

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw()
        if n == -1:
            m = np.eye(4, dtype=np.complex128)
            m[2:, 2:] = Vi().raw()
            return m
        return _mat_pow(self.raw(), n)


class ECR(_EvenOddGate):
    name = "ecr"
    qc = 2

    def raw(self):
        return SQ2 * _c([[0, 1, 0, 1j], [1, 0, -1j, 0], [0, 1j, 0, 1], [-1j, 0, 1, 0]])


# --------------------------------------------------------------------------- angled gates
class AngledGate(Gate):
    n_angles = 1

    def raw_at(self, theta: float) -> np.ndarray:
        raise NotImplementedError

    def raw(self):
        return self.raw_at(self.angle[0])


class _RotationGate(AngledGate):
    """Rx, Ry, Rz, PhaseShift (src/gate_kernels.jl:291-301)."""

    def matrix_rep(self):
        n, th = self.pow_exponent, self.angle[0]
        if n == 0:
            return _eye(1)
        if n == 1:
            return self.raw_at(th)
        if _is_integer(n):
            return self.raw_at(th * n)
        return _mat_pow(self.raw_at(th), n)


class Rx(_RotationGate):
    name = "rx"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[c, -1j * s], [-1j * s, c]])


class Ry(_RotationGate):
    name = "ry"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[c, -s], [s, c]])


class Rz(_RotationGate):
    name = "rz"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[c - 1j * s, 0], [0, c + 1j * s]])


class PhaseShift(_RotationGate):
    name = "phaseshift"

    def raw_at(self, t):
        return _c([[1, 0], [0, np.exp(1j * t)]])


class _CPhaseGate(AngledGate):
    """CPhaseShift*, ZZ: angle scaled by any exponent (src/gate_kernels.jl:303-311)."""
    qc = 2
    slot = 3

    def raw_at(self, t):
        d = np.ones(4, dtype=np.complex128)
        d[self.slot] = np.exp(1j * t)
        return np.diag(d)

    def matrix_rep(self):
        n, th = self.pow_exponent, self.angle[0]
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw_at(th)
        return self.raw_at(th * n)


class CPhaseShift(_CPhaseGate):
    name = "cphaseshift"
    slot = 3


class CPhaseShift00(_CPhaseGate):
    name = "cphaseshift00"
    slot = 0


class CPhaseShift01(_CPhaseGate):
    name = "cphaseshift01"
    slot = 2


class CPhaseShift10(_CPhaseGate):
    name = "cphaseshift10"
    slot = 1


class ZZ(_CPhaseGate):
    name = "zz"

    def raw_at(self, t):
        a = np.exp(-1j * t / 2.0)
        b = np.exp(1j * t / 2.0)
        return np.diag(np.array([a, b, b, a], dtype=np.complex128))


class _TwoQubitRotation(AngledGate):
    """XX, YY, XY, SingleExcitation(+/-), FermionicSWAP (src/gate_kernels.jl:313-322)."""
    qc = 2

    def matrix_rep(self):
        n, th = self.pow_exponent, self.angle[0]
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw_at(th)
        if _is_integer(n):
            return self.raw_at(th * n)
        return _mat_pow(self.raw_at(th), n)


class XX(_TwoQubitRotation):
    name = "xx"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[c, 0, 0, -1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [-1j * s, 0, 0, c]])


class YY(_TwoQubitRotation):
    name = "yy"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[c, 0, 0, 1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [1j * s, 0, 0, c]])


class XY(_TwoQubitRotation):
    name = "xy"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, 1]])


class SingleExcitation(_TwoQubitRotation):
    name = "single_excitation"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        return _c([[1, 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, 1]])


class SingleExcitationPlus(_TwoQubitRotation):
    name = "single_excitation_plus"
    sign = 1.0

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        e = np.exp(self.sign * 1j * t / 2.0)
        return _c([[e, 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, e]])


class SingleExcitationMinus(SingleExcitationPlus):
    name = "single_excitation_minus"
    sign = -1.0


class FermionicSWAP(_TwoQubitRotation):
    name = "fermionic_swap"

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        e2, e = np.exp(1j * t / 2.0), np.exp(1j * t)
        ie2 = 1j * e2
        return _c([[1, 0, 0, 0], [0, e2 * c, -ie2 * s, 0], [0, -ie2 * s, e2 * c, 0], [0, 0, 0, e]])


class _ExcitationGate(AngledGate):
    """DoubleExcitation(+/-), MultiRZ: angle scaled by any exponent (src/gate_kernels.jl:324-332)."""
    qc = 4

    def matrix_rep(self):
        n, th = self.pow_exponent, self.angle[0]
        if n == 0:
            return _eye(self.qc)
        if n == 1:
            return self.raw_at(th)
        return self.raw_at(th * n)


class DoubleExcitation(_ExcitationGate):
    name = "double_excitation"
    phase = 0

    def raw_at(self, t):
        s, c = math.sin(t / 2.0), math.cos(t / 2.0)
        diag = {0: 1.0, 1: np.exp(1j * t / 2.0), -1: np.exp(-1j * t / 2.0)}[self.phase]
        m = np.diag(np.full(16, diag, dtype=np.complex128))
        m[3, 3] = c
        m[12, 12] = c
        m[3, 12] = -s
        m[12, 3] = s
        return m


class DoubleExcitationPlus(DoubleExcitation):
    name = "double_excitation_plus"
    phase = 1


class DoubleExcitationMinus(DoubleExcitation):
    name = "double_excitation_minus"
    phase = -1


class MultiRZ(AngledGate):
    """Multi-qubit Z rotation; its target count comes from the instruction
    (src/custom_gates.jl:339-344,381-385)."""
    name = "multi_rz"
    qc = 1

    def raw_at(self, t):
        raise NotImplementedError("MultiRZ has no fixed matrix; it is applied per target count")


class GPi(_EvenOddGate, AngledGate):
    name = "gpi"

    def raw(self):
        t = self.angle[0]
        return _c([[0, np.exp(-1j * t)], [np.exp(1j * t), 0]])


class GPi2(AngledGate):
    name = "gpi2"

    def raw(self):
        t = self.angle[0]
        return SQ2 * _c([[1, -1j * np.exp(-1j * t)], [-1j * np.exp(1j * t), 1]])


class PRx(AngledGate):
    name = "prx"
    n_angles = 2

    def raw_at2(self, t, p):
        c, s = math.cos(t / 2.0), math.sin(t / 2.0)
        return _c([[c, -1j * np.exp(-1j * p) * s], [-1j * np.exp(1j * p) * s, c]])

    def raw(self):
        return self.raw_at2(*self.angle)

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(1)
        if n == 1:
            return self.raw()
        if n == -1:
            return self.raw_at2(-self.angle[0], self.angle[1])
        return _mat_pow(self.raw(), n)


class PSwap(AngledGate):
    name = "pswap"
    qc = 2

    def raw_at(self, t):
        return _swaplike(np.exp(1j * t))

    def matrix_rep(self):
        n, t = self.pow_exponent, self.angle[0]
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw_at(t)
        if _is_integer(n) and int(n) % 2 == 1:
            return self.raw_at(t * n)
        if _is_integer(n):
            e = np.exp(1j * t * n)
            return np.diag(np.array([1, e, e, 1], dtype=np.complex128))
        return _mat_pow(self.raw_at(t), n)


class MS(AngledGate):
    name = "ms"
    n_angles = 3
    qc = 2

    def raw_at3(self, a0, a1, a2):
        c, s = math.cos(a2 / 2.0), math.sin(a2 / 2.0)
        return _c([
            [c, 0, 0, -1j * np.exp(-1j * (a0 + a1)) * s],
            [0, c, -1j * np.exp(-1j * (a0 - a1)) * s, 0],
            [0, -1j * np.exp(1j * (a0 - a1)) * s, c, 0],
            [-1j * np.exp(1j * (a0 + a1)) * s, 0, 0, c],
        ])

    def raw(self):
        return self.raw_at3(*self.angle)

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(2)
        if n == 1:
            return self.raw()
        if n == -1:
            return self.raw_at3(self.angle[0] + math.pi, self.angle[1], self.angle[2])
        return _mat_pow(self.raw(), n)


class U(AngledGate):
    name = "u"
    n_angles = 3

    def raw_at3(self, t, p, l):
        c, s = math.cos(t / 2.0), math.sin(t / 2.0)
        return _c([[c, -np.exp(1j * l) * s], [np.exp(1j * p) * s, np.exp(1j * (l + p)) * c]])

    def raw(self):
        return self.raw_at3(*self.angle)

    def matrix_rep(self):
        n = self.pow_exponent
        if n == 0:
            return _eye(1)
        if n == 1:
            return self.raw()
        if n == -1:
            t, p, l = self.angle
            return self.raw_at3(-t, -l, -p)
        return _mat_pow(self.raw(), n)


class GPhase(AngledGate):
    """Global phase on N qubits (src/custom_gates.jl:355-362)."""
    name = "gphase"

    def __init__(self, n_qubits: int, angle: float, pow_exponent: float = 1.0):
        super().__init__(angle, pow_exponent=pow_exponent)
        self.n = int(n_qubits)
        self.qc = self.n

    def __pow__(self, n):
        return GPhase(self.n, self.angle[0], self.pow_exponent * float(n))

    def inv(self):
        return GPhase(self.n, self.angle[0], -self.pow_exponent)

    def __eq__(self, o):
        return isinstance(o, GPhase) and self.n == o.n and self.angle == o.angle and self.pow_exponent == o.pow_exponent

    def raw(self):
        return np.diag(np.full(2 ** self.n, np.exp(1j * self.angle[0]), dtype=np.complex128))


class Unitary(Gate):
    name = "unitary"

    def __init__(self, matrix, pow_exponent: float = 1.0):
        self.matrix = np.array(matrix, dtype=np.complex128)
        d = self.matrix.shape[0]
        if self.matrix.shape != (d, d) or d & (d - 1) or d < 2:
            raise ValueError("Unitary needs a square 2^k matrix")
        self.qc = int(round(math.log2(d)))
        self.angle = ()
        self.pow_exponent = float(pow_exponent)

    def __pow__(self, n):
        return Unitary(self.matrix, self.pow_exponent * float(n))

    def inv(self):
        return Unitary(self.matrix, -self.pow_exponent)

    def __eq__(self, o):
        return isinstance(o, Unitary) and np.array_equal(self.matrix, o.matrix) and self.pow_exponent == o.pow_exponent

    def raw(self):
        return self.matrix


class Control(Gate):
    """ctrl / negctrl modifier (src/custom_gates.jl:418-457)."""
    name = "control"

    def __init__(self, g: Gate, bitvals: Sequence[int], pow_exponent: float = 1.0):
        if isinstance(g, Control):
            bitvals = tuple(g.bitvals) + tuple(bitvals)
            pow_exponent = g.pow_exponent * pow_exponent
            g = g.g
        self.g = g
        self.bitvals = tuple(int(b) for b in bitvals)
        self.pow_exponent = float(pow_exponent)
        self.angle = ()
        self.qc = g.n if isinstance(g, GPhase) else g.qubit_count() + len(self.bitvals)

    def qubit_count(self):
        return self.qc

    def __pow__(self, n):
        return Control(self.g ** n, self.bitvals)

    def inv(self):
        return Control(self.g.inv(), self.bitvals)

    def __eq__(self, o):
        return isinstance(o, Control) and self.g == o.g and self.bitvals == o.bitvals and self.pow_exponent == o.pow_exponent

    def raw(self):
        if isinstance(self.g, GPhase):
            gm = self.g.matrix_rep()
            d = np.ones(2 ** self.g.n, dtype=np.complex128)
            ci = sum(b << i for i, b in enumerate(self.bitvals))
            d[ci] = gm[ci, ci]
            return np.diag(d)
        inner = self.g.matrix_rep()
        iq = self.g.qubit_count()
        full = np.eye(2 ** self.qc, dtype=np.complex128)
        ci = sum(b << (i + iq) for i, b in enumerate(self.bitvals))
        di = inner.shape[0]
        full[ci:ci + di, ci:ci + di] = inner
        return full


class Measure(QuantumOperator):
    def __init__(self, index: int = -1):
        self.index = index


class Reset(QuantumOperator):
    pass


class Barrier(QuantumOperator):
    pass


class Delay(QuantumOperator):
    def __init__(self, duration=None):
        self.duration = duration


def qubit_count(g) -> int:
    return g.qubit_count() if isinstance(g, Gate) else 1


# --------------------------------------------------------------------------- Pauli eigenvalues
def pauli_eigenvalues(n: int) -> np.ndarray:
    """Z^{(x)n} diagonal, src/operators.jl:156-185 (the coefficient is 1)."""
    i = np.arange(2 ** n, dtype=np.uint64)
    par = np.zeros(2 ** n, dtype=np.uint64)
    for b in range(n):
        par ^= (i >> np.uint64(b)) & np.uint64(1)
    return np.where(par == 1, -1.0, 1.0)


# --------------------------------------------------------------------------- dispatch
@dataclass
class LoweredGate:
    """One engine call: matrix (dense or diagonal), targets, controls and flags."""
    matrix: np.ndarray
    targets: tuple
    controls: tuple = ()
    control_values: tuple = ()
    flags: int = 0
    diagonal: bool = False
    extra: dict = field(default_factory=dict)


def _by_size_flags(k: int) -> int:
    """Target convention of the reference kernel a k-target matrix reaches:
    1 and 2 targets: bit j <-> targets[j]; >= 3: sorted (src/gate_kernels.jl:753-775)."""
    return _abi.BS_GATE_SORTED_TARGETS if k >= 3 else 0


_CONTROLLED = {CNot: (X, 1), CY: (Y, 1), CZ: (Z, 1), CV: (V, 1), CSwap: (Swap, 1), CCNot: (X, 2)}


def lower_gate(g: Gate, targets: Sequence[int], conj: bool = False) -> list:
    """Restate apply_gate!(Val(conj), g, state, targets...) as engine calls."""
    t = tuple(int(x) for x in targets)
    f = np.conj if conj else (lambda m: m)
    if isinstance(g, I):
        return []
    if isinstance(g, Control) and isinstance(g.g, GPhase):
        n = g.g.n
        factor = -1j if conj else 1j
        d = np.ones(2 ** n, dtype=np.complex128)
        pi = sum(b << i for i, b in enumerate(g.bitvals))
        d[pi] = np.exp(factor * g.g.angle[0] * g.g.pow_exponent * g.pow_exponent)
        return [LoweredGate(d, t, flags=_by_size_flags(len(t)), diagonal=True)]
    if isinstance(g, Control):
        tg = g.g ** g.pow_exponent
        nc = len(g.bitvals)
        mat = f(tg.matrix_rep())
        return [LoweredGate(mat, t[nc:], t[:nc], tuple(g.bitvals), flags=_by_size_flags(len(t) - nc))]
    for cls, (tcls, nc) in _CONTROLLED.items():
        if type(g) is cls:
            mat = f(tcls(pow_exponent=g.pow_exponent).matrix_rep())
            return [LoweredGate(mat, t[nc:], t[:nc], (1,) * nc, flags=0)]
    if isinstance(g, GPhase):
        e = np.exp(1j * g.angle[0] * g.pow_exponent)
        e = np.conj(e) if conj else e
        return [LoweredGate(np.full(2 ** len(t), e, dtype=np.complex128), t, flags=_by_size_flags(len(t)), diagonal=True)]
    if isinstance(g, MultiRZ):
        if len(t) == 1:
            return lower_gate(Rz(g.angle[0], pow_exponent=g.pow_exponent), t, conj)
        if len(t) == 2:
            return lower_gate(ZZ(g.angle[0], pow_exponent=g.pow_exponent), t, conj)
        factor = -1j * g.angle[0] / 2.0
        factor = np.conj(factor) if conj else factor
        d = np.exp(factor * pauli_eigenvalues(len(t)))
        return [LoweredGate(d, t, flags=_abi.BS_GATE_SORTED_TARGETS, diagonal=True)]
    if type(g) is DoubleExcitation:
        # two-amplitude kernel (src/custom_gates.jl:390-414), identical for both conj values
        m = DoubleExcitation(g.angle[0] * g.pow_exponent).raw()
        return [LoweredGate(m, t, flags=_abi.BS_GATE_MSB_FIRST)]
    mat = f(g.matrix_rep())
    k = int(round(math.log2(mat.shape[0])))
    if k != len(t):
        raise ValueError(f"{g!r} acts on {k} qubit(s), got targets {t}")
    return [LoweredGate(mat, t, flags=_by_size_flags(k))]
