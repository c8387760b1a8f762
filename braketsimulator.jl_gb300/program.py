"""``simulate`` orchestration over a parsed program (src/BraketSimulator.jl:97-408).

The OpenQASM front end (Quasar.jl) is not part of this backend: a ``Program``
here is the already-parsed form the reference builds (instructions, result
types, basis-rotation instructions).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .gates import Barrier, Delay, H as HGate, Measure, Reset, Ry, S as SGate, Unitary, Z as ZGate
from .results import calculate
from .simulators import DensityMatrixSimulator, Instruction, StateVectorSimulator


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


ALL_QUBITS = -1


def basis_rotation_gates(obs) -> list:
    """Gates that rotate an observable's eigenbasis onto the computational basis
    (src/circuit.jl:120-126)."""
    from . import observables as O
    if isinstance(obs, O.H):
        return [Ry(-math.pi / 4.0)]
    if isinstance(obs, O.X):
        return [HGate()]
    if isinstance(obs, (O.I, O.Z)):
        return []
    if isinstance(obs, O.Y):
        return [ZGate(), SGate(), HGate()]
    if isinstance(obs, O.TensorProduct):
        return [g for f in obs.factors for g in basis_rotation_gates(f)]
    if isinstance(obs, O.HermitianObservable):
        return [Unitary(np.linalg.eigh(obs.matrix)[1].conj().T)]
    raise TypeError(f"no basis rotation for {obs!r}")


def fix_endianness(mat: np.ndarray) -> np.ndarray:
    """Swap the middle rows and columns of a 4x4 matrix (src/circuit.jl:128-142); other sizes pass."""
    if mat.shape != (4, 4):
        return mat
    out = np.array(mat, copy=True)
    out[:, [1, 2]] = out[:, [2, 1]]
    out[[1, 2], :] = out[[2, 1], :]
    return out


def _observable_to_instructions(obs, target_list) -> list:
    """src/circuit.jl:144-153."""
    out = []
    for g in basis_rotation_gates(obs):
        if isinstance(g, Unitary) and len(target_list) == 2:
            out.append(Instruction(Unitary(fix_endianness(g.matrix)), target_list))
        else:
            out.append(Instruction(g, target_list))
    return out


def tensor_product_index_dict(obs, obs_targets) -> dict:
    """Factor and factor targets for each position of a tensor product's targets
    (src/circuit.jl:99-118)."""
    factors = list(obs.factors)
    total = factors[0].qubit_count()
    out = {}
    i = 0
    while factors:
        if i >= total:
            factors.pop(0)
            if factors:
                total += factors[0].qubit_count()
        if factors:
            front = total - factors[0].qubit_count()
            out[i] = (factors[0], tuple(obs_targets[front:total]))
        i += 1
    return out


def _extract_observable(rt):
    """src/circuit.jl:86-88: the observable of Expectation / Variance / Sample, Z for Probability."""
    from . import observables as O
    from .results import Expectation, Probability, Sample, Variance
    if isinstance(rt, (Expectation, Variance, Sample)):
        return rt.observable
    if isinstance(rt, Probability):
        return O.Z()
    return None


class Circuit:
    """Instructions and result types with the observable bookkeeping that decides the basis
    rotations applied before sampling (src/circuit.jl:1-309: ``Circuit``, ``add_instruction!``,
    ``add_to_qubit_observable_mapping!``, ``basis_rotation_instructions!``).  ``to_program()``
    gives the ``Program`` that ``simulate`` runs."""

    def __init__(self, instructions=(), results=()):
        self.instructions = []
        self.result_types = []
        self.basis_rotation_instructions = []
        self.qubit_observable_mapping = {}
        self.qubit_observable_target_mapping = {}
        self.qubit_observable_set = set()
        self.observables_simultaneously_measurable = True
        self.measure_targets = []
        self.reset_targets = []
        for ix in instructions:
            self.add_instruction(ix)
        for rt in results:
            self.add_result(rt)

    def qubits(self) -> list:
        """src/circuit.jl:55."""
        qs = set(self.qubit_observable_set)
        for ix in self.instructions:
            qs.update(ix.target)
        return sorted(qs)

    def qubit_count(self) -> int:
        return len(self.qubits())

    def _check_measured(self, qubits):
        """src/circuit.jl:251-265."""
        if not self.measure_targets:
            return
        for q in qubits:
            if q not in self.measure_targets:
                continue
            if q not in self.reset_targets:
                raise ValueError("cannot apply instruction to measured qubits.")
            last_m = max(i for i, ix in enumerate(self.instructions) if isinstance(ix.operator, Measure) and q in ix.target)
            last_r = max(i for i, ix in enumerate(self.instructions) if isinstance(ix.operator, Reset) and q in ix.target)
            if last_m > last_r:
                raise ValueError("cannot apply instruction to measured qubits.")

    def add_instruction(self, ix) -> "Circuit":
        """src/circuit.jl:268-284."""
        if not isinstance(ix.operator, (Reset, Barrier, Delay)):
            self._check_measured(ix.target)
        if isinstance(ix.operator, Measure):
            self.measure_targets.extend(ix.target)
        if isinstance(ix.operator, Reset):
            self.reset_targets.extend(ix.target)
        self.instructions.append(ix)
        return self

    def _noncommuting(self):
        """src/circuit.jl:90-95."""
        self.observables_simultaneously_measurable = False
        self.qubit_observable_mapping.clear()
        self.qubit_observable_target_mapping.clear()

    def _add_observable(self, obs, obs_targets):
        """add_to_qubit_observable_mapping! (src/circuit.jl:182-246)."""
        from . import observables as O
        tp = isinstance(obs, O.TensorProduct)
        targets = list(obs_targets) if obs_targets else sorted(self.qubit_observable_set)
        all_obs = self.qubit_observable_mapping.get(ALL_QUBITS)
        tpd = tensor_product_index_dict(obs, targets) if tp and targets else {}
        ident = O.I()
        for ii, target in enumerate(targets):
            new = tpd[ii][0] if tp else obs
            cur = all_obs if all_obs is not None else self.qubit_observable_mapping.get(target)
            add = cur is None or (cur == ident and new != ident)
            if not add and cur != ident and new != ident and new != cur:
                return self._noncommuting()
            if obs_targets:
                new_targets = tpd[ii][1] if tp else tuple(obs_targets)
                if add:
                    self.qubit_observable_target_mapping[target] = new_targets
                    self.qubit_observable_mapping[target] = new
                elif new.qubit_count() > 1:
                    cur_t = self.qubit_observable_target_mapping.get(target)
                    if cur_t is not None and cur_t != new_targets:
                        if tp:
                            return self._noncommuting()
                        self._noncommuting()
        if not tp and not obs_targets:
            if all_obs is not None and all_obs != obs:
                return self._noncommuting()
            self.qubit_observable_mapping[ALL_QUBITS] = obs

    def add_result(self, rt) -> "Circuit":
        """The result-type half of to_circuit (src/circuit.jl:287-297)."""
        obs = _extract_observable(rt)
        if obs is not None and self.observables_simultaneously_measurable:
            self._add_observable(obs, tuple(getattr(rt, "targets", ()) or ()))
        from .results import Expectation, Sample, Variance
        if isinstance(rt, (Expectation, Variance, Sample)):
            self.qubit_observable_set.update(rt.targets or ())
        self.result_types.append(rt)
        return self

    def compute_basis_rotation_instructions(self) -> list:
        """basis_rotation_instructions! (src/circuit.jl:164-180)."""
        all_obs = self.qubit_observable_mapping.get(ALL_QUBITS)
        if all_obs is not None:
            out = [ix for q in self.qubits() for ix in _observable_to_instructions(all_obs, (q,))]
        else:
            out, seen = [], []
            for tl in self.qubit_observable_target_mapping.values():
                if tl in seen:
                    continue
                seen.append(tl)
                out.extend(_observable_to_instructions(self.qubit_observable_mapping[tl[0]], tl))
        self.basis_rotation_instructions = out
        return out

    def to_program(self, shots: int = 0) -> Program:
        """_prepare_program for a circuit (src/BraketSimulator.jl:208-219): basis rotations are
        computed when sampling."""
        if shots > 0:
            self.compute_basis_rotation_instructions()
        return Program(list(self.instructions), list(self.result_types), list(self.basis_rotation_instructions))


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


MMAP_THRESHOLD = 1 << 20   # bytes: result values above this go to files (src/BraketSimulator.jl:411)


def _device_file_kind(rt, sim):
    """The results the engine writes to a file itself: the full state vector and the full
    probability vector."""
    from .results import Probability, StateVector
    if isinstance(rt, StateVector) and isinstance(sim, StateVectorSimulator):
        return "state", 16
    if isinstance(rt, Probability) and not rt.targets:
        return "probabilities", 8
    return None, 0


def _mmap_results(sim, program: Program, n: int, threshold: int, directory=None):
    """Exact results with every value above ``threshold`` bytes in a temporary file
    (_mmap_large_result_values, src/BraketSimulator.jl:410-428): the value is left empty and the
    file path and element count are returned beside it.  The full state and probability vectors
    go from the device to the file in chunks, without a host copy of the whole vector."""
    import os
    import tempfile
    results, paths, lens = [], [], []
    for rt in program.results:
        what, eb = _device_file_kind(rt, sim)
        size = (1 << n) * eb
        if what is not None and size > threshold:
            fd, path = tempfile.mkstemp(dir=directory)
            os.close(fd)
            sim.write_result_file(what, path)
            results.append((rt, np.empty(0, dtype=np.complex128 if what == "state" else np.float64)))
            paths.append(path)
            lens.append(1 << n)
            continue
        val = calculate(rt, sim)
        arr = np.asarray(val)
        if arr.dtype != object and arr.nbytes > threshold:
            fd, path = tempfile.mkstemp(dir=directory)
            with os.fdopen(fd, "wb") as f:
                f.write(np.ascontiguousarray(arr).tobytes())
            paths.append(path)
            lens.append(int(arr.size))
            val = np.empty(0, dtype=arr.dtype)
        results.append((rt, val))
    return results, tuple(paths), tuple(lens)


def simulate(sim, program: Program, shots: int = 0, seed: int | None = None, mmap_threshold: int | None = None,
             mmap_dir=None) -> dict:
    """simulate(sim, program, shots) (src/BraketSimulator.jl:307-322) for one program,
    or a list of programs (batch, :347-395) run one after another on the GPU.

    With ``mmap_threshold`` (bytes; ``MMAP_THRESHOLD`` is the reference's 1 MiB), exact result
    values above it are written to temporary files instead, as the reference's entry for external
    callers does (src/BraketSimulator.jl:430-443); the returned dict then carries ``mmapPaths`` and
    ``mmapLengths`` (element counts)."""
    if isinstance(program, (list, tuple)):
        return [simulate(sim.similar(shots=shots), p, shots, seed, mmap_threshold, mmap_dir) for p in program]
    n = program.qubit_count()
    ops = list(program.instructions)
    if shots > 0 and program.basis_rotation_instructions:
        ops += list(program.basis_rotation_instructions)
    measured = sorted(_measured_qubits(program, n))
    small = isinstance(sim, StateVectorSimulator) and n <= 12 and shots > 0 and mmap_threshold is None
    if small:
        # reinit!, evolve! and the shots in one round trip (bs_run_small)
        sim.reinit(n, shots)
        _, s = sim.run(ops, shots, seed, probabilities=False)
    else:
        sim.reinit(n, shots)
        sim.evolve(ops)
    results, paths, lens = [], (), ()
    if shots == 0 and program.results:
        if mmap_threshold is None:
            results = [(r, calculate(r, sim)) for r in program.results]
        else:
            results, paths, lens = _mmap_results(sim, program, n, int(mmap_threshold), mmap_dir)
    measurements = None
    if shots > 0:
        if not small:
            s = sim.samples(seed)
        bits = ((s[:, None] >> np.arange(n - 1, -1, -1)[None, :]) & 1).astype(np.int64)
        measurements = bits[:, measured]
    out = {"measurements": measurements, "resultTypes": results, "measuredQubits": measured,
           "deviceId": sim.device_id, "shots": shots}
    if mmap_threshold is not None:
        out["mmapPaths"], out["mmapLengths"] = paths, lens
    return out
