"""Noise channels and their Kraus representations (src/noises.jl:6-104,
src/noise_kernels.jl:25-103).

``lower_noise`` restates ``apply_noise!``: PhaseFlip has its own full elementwise
kernel in the reference (src/noise_kernels.jl:7-23); every other channel goes
through ``kraus_rep`` to the 1-, 2- or k-target Kraus kernel whose index
conventions are kept by the flags returned here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from .gates import QuantumOperator

_I = np.eye(2, dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
_P = {"I": _I, "X": _X, "Y": _Y, "Z": _Z}


class Noise(QuantumOperator):
    qc = 1

    def qubit_count(self) -> int:
        return self.qc

    def kraus_rep(self) -> "Kraus":
        raise NotImplementedError


class Kraus(Noise):
    def __init__(self, matrices):
        self.matrices = [np.array(m, dtype=np.complex128) for m in matrices]
        d = self.matrices[0].shape[0]
        self.qc = int(round(math.log2(d)))

    def kraus_rep(self):
        return self


class BitFlip(Noise):
    def __init__(self, probability):
        self.probability = float(probability)

    def kraus_rep(self):
        p = self.probability
        return Kraus([math.sqrt(1 - p) * _I, math.sqrt(p) * _X])


class PhaseFlip(Noise):
    def __init__(self, probability):
        self.probability = float(probability)

    def kraus_rep(self):
        p = self.probability
        return Kraus([math.sqrt(1 - p) * _I, math.sqrt(p) * _Z])


class Depolarizing(Noise):
    def __init__(self, probability):
        self.probability = float(probability)

    def kraus_rep(self):
        p = self.probability
        return Kraus([math.sqrt(1.0 - p) * _I, math.sqrt(p / 3.0) * _X, math.sqrt(p / 3.0) * _Y, math.sqrt(p / 3.0) * _Z])


class PauliChannel(Noise):
    def __init__(self, probX, probY, probZ):
        self.probX, self.probY, self.probZ = float(probX), float(probY), float(probZ)

    def kraus_rep(self):
        return Kraus([math.sqrt(1 - self.probX - self.probY - self.probZ) * _I, math.sqrt(self.probX) * _X,
                      math.sqrt(self.probY) * _Y, math.sqrt(self.probZ) * _Z])


class AmplitudeDamping(Noise):
    def __init__(self, gamma):
        self.gamma = float(gamma)

    def kraus_rep(self):
        g = self.gamma
        return Kraus([np.array([[1.0, 0.0], [0.0, math.sqrt(1.0 - g)]], dtype=np.complex128),
                      np.array([[0.0, math.sqrt(g)], [0.0, 0.0]], dtype=np.complex128)])


class GeneralizedAmplitudeDamping(Noise):
    def __init__(self, probability, gamma):
        self.probability, self.gamma = float(probability), float(gamma)

    def kraus_rep(self):
        p, g = self.probability, self.gamma
        sp, sq = math.sqrt(p), math.sqrt(1.0 - p)
        return Kraus([sp * np.array([[1.0, 0.0], [0.0, math.sqrt(1.0 - g)]]),
                      sp * np.array([[0.0, math.sqrt(g)], [0.0, 0.0]]),
                      sq * np.array([[math.sqrt(1.0 - g), 0.0], [0.0, 1.0]]),
                      sq * np.array([[0.0, 0.0], [math.sqrt(g), 0.0]])])


class PhaseDamping(Noise):
    def __init__(self, gamma):
        self.gamma = float(gamma)

    def kraus_rep(self):
        g = self.gamma
        return Kraus([np.array([[1.0, 0.0], [0.0, math.sqrt(1.0 - g)]], dtype=np.complex128),
                      np.array([[0.0, 0.0], [0.0, math.sqrt(g)]], dtype=np.complex128)])


class TwoQubitDepolarizing(Noise):
    qc = 2

    def __init__(self, probability):
        self.probability = float(probability)

    def kraus_rep(self):
        p = self.probability
        ks = [_I, _X, _Y, _Z]
        mats = []
        for kj in ks:            # column-major order of [kron(ki, kj) for ki, kj]
            for ki in ks:
                mats.append(np.kron(ki, kj))
        out = [math.sqrt(1.0 - p) * mats[0]] + [math.sqrt(p / 15.0) * m for m in mats[1:]]
        return Kraus(out)


class TwoQubitDephasing(Noise):
    qc = 2

    def __init__(self, probability):
        self.probability = float(probability)

    def kraus_rep(self):
        p = self.probability
        return Kraus([math.sqrt(1 - p) * np.kron(_I, _I), math.sqrt(p / 3.0) * np.kron(_I, _Z),
                      math.sqrt(p / 3.0) * np.kron(_Z, _I), math.sqrt(p / 3.0) * np.kron(_Z, _Z)])


class MultiQubitPauliChannel(Noise):
    def __init__(self, probabilities: dict):
        self.probabilities = {k: float(v) for k, v in probabilities.items()}
        self.qc = len(next(iter(self.probabilities)))

    def kraus_rep(self):
        if self.qc != 2:
            raise NotImplementedError("the reference defines Kraus operators for the two-qubit Pauli channel only")
        total = sum(self.probabilities.values())
        ks = [math.sqrt(1.0 - total) * np.eye(4, dtype=np.complex128)]
        for k, v in self.probabilities.items():
            if k != "II":
                ks.append(math.sqrt(v) * np.kron(_P[k[0]], _P[k[1]]))
        return Kraus(ks)


def TwoQubitPauliChannel(probabilities: dict) -> MultiQubitPauliChannel:
    return MultiQubitPauliChannel(probabilities)


@dataclass
class LoweredNoise:
    matrices: list
    targets: tuple
    flags: int


def kraus_flags(k: int) -> int:
    """Target convention of the reference's Kraus kernel for k targets."""
    if k == 1:
        return 0
    if k == 2:
        return _abi.BS_GATE_MSB_FIRST          # (00, t2 flipped, t1 flipped, 11)
    return _abi.BS_GATE_SORTED_TARGETS


def lower_noise(n: Noise, targets, mode: int) -> LoweredNoise:
    t = tuple(int(x) for x in targets)
    kr = n.kraus_rep()
    if kr.qc != len(t):
        raise ValueError(f"{type(n).__name__} acts on {kr.qc} qubit(s), got targets {t}")
    flags = kraus_flags(len(t))
    if isinstance(n, PhaseFlip):
        flags |= _abi.BS_NOISE_PHYSICAL     # the reference's PhaseFlip kernel updates every element
    else:
        flags |= mode
    return LoweredNoise(kr.matrices, t, flags)
