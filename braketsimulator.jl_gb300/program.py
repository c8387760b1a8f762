"""``simulate`` orchestration over a parsed program (src/BraketSimulator.jl:97-408).

The OpenQASM front end (Quasar.jl) is not part of this backend: a ``Program``
here is the already-parsed form the reference builds (instructions, result
types, basis-rotation instructions).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .gates import Measure
from .results import calculate
from .simulators import DensityMatrixSimulator, StateVectorSimulator


@dataclass
class Program:
    instructions: list
    results: list = field(default_factory=list)
    basis_rotation_instructions: list = field(default_factory=list)

    def qubit_count(self) -> int:
        qs = {q for ix in self.instructions + self.basis_rotation_instructions for q in ix.target}
        for r in self.results:
            qs.update(getattr(r, "targets", ()) or ())
        return (max(qs) + 1) if qs else 0


def create_sim(simulator_id: str, shots: int):
    """src/BraketSimulator.jl:402-408."""
    if simulator_id == "braket_sv_v2":
        return StateVectorSimulator(0, shots)
    if simulator_id == "braket_dm_v2":
        return DensityMatrixSimulator(0, shots)
    raise ValueError(f"unknown simulator {simulator_id!r}")


def _measured_qubits(program: Program, n: int) -> list:
    """src/BraketSimulator.jl:193-200."""
    ms = [ix for ix in program.instructions if isinstance(ix.operator, Measure)]
    if not ms:
        return list(range(n))
    out = []
    for ix in ms:
        for q in ix.target:
            if q not in out:
                out.append(q)
    return out


def simulate(sim, program: Program, shots: int = 0, seed: int | None = None) -> dict:
    """simulate(sim, program, shots) (src/BraketSimulator.jl:307-322) for one program,
    or a list of programs (batch, :347-395) run one after another on the GPU."""
    if isinstance(program, (list, tuple)):
        return [simulate(sim.similar(shots=shots), p, shots, seed) for p in program]
    n = program.qubit_count()
    ops = list(program.instructions)
    if shots > 0 and program.basis_rotation_instructions:
        ops += list(program.basis_rotation_instructions)
    sim.reinit(n, shots)
    sim.evolve(ops)
    measured = sorted(_measured_qubits(program, n))
    results = []
    if shots == 0 and program.results:
        results = [(r, calculate(r, sim)) for r in program.results]
    measurements = None
    if shots > 0:
        s = sim.samples(seed)
        bits = ((s[:, None] >> np.arange(n - 1, -1, -1)[None, :]) & 1).astype(np.int64)
        measurements = bits[:, measured]
    return {"measurements": measurements, "resultTypes": results, "measuredQubits": measured,
            "deviceId": sim.device_id, "shots": shots}
