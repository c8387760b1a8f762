"""StateVectorSimulator / DensityMatrixSimulator backed by the GB300 engine.

Mirrors the reference's simulator API (src/sv_simulator.jl, src/dm_simulator.jl,
src/result_types.jl): ``evolve`` (evolve!), ``reinit`` (reinit!), ``apply_gate``,
``apply_noise``, ``probabilities``, ``expectation``, ``samples``,
``state_vector``, ``density_matrix``, ``apply_observables`` (apply_observables!),
``state_with_observables``.  The state lives in GPU memory inside an engine
handle; every numerical step runs in the engine's CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import struct
from typing import Sequence

import numpy as np

from . import _abi
from .gates import Barrier, Control, Delay, Gate, Measure, Reset, Rx, Ry, Rz, Unitary, lower_gate
from .noises import Noise, lower_noise
from .observables import (H, HermitianObservable, I, Observable, StandardObservable, TensorProduct, X, Y, Z,
                          diagonalizing_gates)

NOISE_MODES = {"reference": _abi.BS_NOISE_REFERENCE, "physical": _abi.BS_NOISE_PHYSICAL}


class Instruction:
    """Operator plus target qubits (src/qubit_set.jl:111-117)."""

    def __init__(self, operator, target):
        self.operator = operator
        if isinstance(target, (int, np.integer)):
            target = [int(target)]
        self.target = tuple(int(t) for t in target)

    def __repr__(self):
        return f"Instruction({self.operator!r}, {list(self.target)})"


def _addr(a: np.ndarray) -> int:
    """Address of a writable contiguous array's data (cheaper than ``a.ctypes.data``)."""
    return C.addressof(C.c_char.from_buffer(a)) if a.size else a.ctypes.data


def _ops_for(instructions, dm: bool, noise_mode: int):
    """Lower instructions into a bs_op array; returns (array, keepalive buffers)."""
    ops = []    # the bs_op structs as bytes, joined into one array below
    keep = []
    skip = (Measure, Reset, Barrier, Delay)
    cache = _LOWER_CACHE
    rot_at, rot_vals = [], []   # 1-qubit rotations: their ops, and their matrices for one shared buffer
    for ix in instructions:
        op = ix.operator
        t = ix.target
        tp = type(op)
        if tp in _ROT_TYPES and len(t) == 1 and op.pow_exponent == 1:
            rot_at.append(len(ops))
            o = _ONE_TARGET_OPS.get(t[0])
            if o is None:
                o = _ONE_TARGET_OPS[t[0]] = _one_target_op(t[0])
            ops.append(o)
            rot_vals.extend(_rotation_values(op))
            continue
        if tp in _BY_VALUE:
            # a fixed gate lowered before (the common case of repeated circuits): no dispatch
            hit = cache.get((tp, op.angle, op.pow_exponent, t))
            if hit is not None:
                for o, buf in hit:
                    ops.append(o)
                    keep.append(buf)
                continue
        if isinstance(op, skip):
            continue
        if isinstance(op, Noise):
            if not dm:
                raise TypeError("noise channels need a DensityMatrixSimulator")
            ln = lower_noise(op, t, noise_mode)
            buf = np.concatenate([_abi.cplx_buffer(m) for m in ln.matrices])
            keep.append(buf)
            o = _abi.BsOp()
            o.kind = 1
            o.flags = ln.flags
            o.n_targets = len(ln.targets)
            o.n_controls = 0
            for j, q in enumerate(ln.targets):
                o.targets[j] = q
            o.n_matrices = len(ln.matrices)
            o.matrix = _abi.dptr(buf)
            ops.append(bytes(o))
            continue
        if not isinstance(op, Gate):
            raise TypeError(f"cannot apply {op!r}")
        for o, buf in _gate_ops(op, t):
            keep.append(buf)
            ops.append(o)
    n = len(ops)
    if n == 0:
        return (_abi.BsOp * 1)(), 0, keep
    arr = (_abi.BsOp * n).from_buffer_copy(b"".join(ops))
    if rot_at:
        # every rotation's matrix in one buffer, 8 doubles each; their ops point into it
        vals = np.array(rot_vals, dtype=np.float64)
        keep.append(vals)
        words = np.frombuffer(arr, dtype=np.uint64).reshape(n, _BSOP_SIZE // 8)
        words[rot_at, _OFF_MAT // 8] = np.uint64(_addr(vals)) + np.uint64(64) * np.arange(len(rot_at), dtype=np.uint64)
    return arr, n, keep


# Lowered engine ops of fixed gates, keyed by (gate type, angles, pow_exponent, targets).  Gates
# that carry a matrix or a sub-gate (Unitary, Control) are lowered every time.  The cached matrix
# buffers are only read by the engine.
_LOWER_CACHE: dict = {}
_LOWER_CACHE_MAX = 1 << 16


_BSOP_SIZE = C.sizeof(_abi.BsOp)
_OFF_NT, _OFF_T0, _OFF_MAT = _abi.BsOp.n_targets.offset, _abi.BsOp.targets.offset, _abi.BsOp.matrix.offset
_ONE_TARGET_OP = bytearray(_BSOP_SIZE)   # a gate op with one target, the rest zero
struct.pack_into("<i", _ONE_TARGET_OP, _OFF_NT, 1)
_ONE_TARGET_OP = bytes(_ONE_TARGET_OP)
_ROTATIONS = (Rx, Ry, Rz)
_ROT_TYPES = frozenset(_ROTATIONS)
_ONE_TARGET_OPS: dict = {}   # target -> _one_target_op(target)
# gate types whose lowering is cached by value (type, angles, pow_exponent, targets): every Gate
# type but the matrix-carrying ones (Unitary, Control), added as they are first lowered
_BY_VALUE = set()


def _rotation_values(op) -> tuple:
    """The 8 doubles (row-major, interleaved) of Rx/Ry/Rz at pow_exponent 1, written directly: the
    same doubles, signed zeros included, as the complex arithmetic of raw_at."""
    t = op.angle[0]
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    tp = type(op)
    if tp is Rx:      # [[c, -i s], [-i s, c]]
        return (c, 0.0, 0.0, -s, 0.0, -s, c, 0.0)
    if tp is Ry:      # [[c, -s], [s, c]]
        return (c, 0.0, -s, 0.0, s, 0.0, c, 0.0)
    return (c, 0.0 - s, 0.0, 0.0, 0.0, 0.0, c, 0.0 + s)   # Rz: [[c - i s, 0], [0, c + i s]]


def _rotation_buffer(op) -> np.ndarray:
    """matrix_rep of Rx/Ry/Rz as the engine's interleaved buffer."""
    if op.pow_exponent != 1:
        return _abi.cplx_buffer(op.matrix_rep())
    return np.array(_rotation_values(op), dtype=np.float64)


def _one_target_op(q: int) -> bytes:
    """A gate op on one target q with no matrix yet (the rest zero)."""
    b = bytearray(_ONE_TARGET_OP)
    struct.pack_into("<i", b, _OFF_T0, q)
    return bytes(b)


def _rotation_op(op, q: int):
    """The lowering of a 1-qubit rotation (what lower_gate gives: its dense matrix_rep, no flags),
    without the generic dispatch: rotations in variational and random circuits rarely repeat an
    angle, so they miss the cache and their lowering cost is the batch's host time."""
    buf = _rotation_buffer(op)
    b = bytearray(_ONE_TARGET_OP)
    struct.pack_into("<i", b, _OFF_T0, q)
    struct.pack_into("<Q", b, _OFF_MAT, _addr(buf))
    return [(bytes(b), buf)]


def _gate_ops(op, t):
    """[(bs_op struct bytes, matrix buffer)] for one gate on targets t (a tuple of ints)."""
    if type(op) in _ROTATIONS and len(t) == 1:
        return _rotation_op(op, t[0])
    key = None
    if not isinstance(op, (Unitary, Control)):
        _BY_VALUE.add(type(op))
        key = (type(op), op.angle, op.pow_exponent, t)
        hit = _LOWER_CACHE.get(key)
        if hit is not None:
            return hit
    res = []
    for lg in lower_gate(op, t):
        buf = _abi.cplx_buffer(lg.matrix)
        o = _abi.BsOp()
        o.kind = 0
        o.flags = lg.flags | (_abi.BS_GATE_DIAGONAL if lg.diagonal else 0)
        if len(lg.targets) > _abi.BS_MAX_TARGETS or len(lg.controls) > _abi.BS_MAX_CONTROLS:
            raise ValueError("too many qubits in one instruction")
        o.n_targets = len(lg.targets)
        for j, q in enumerate(lg.targets):
            o.targets[j] = q
        o.n_controls = len(lg.controls)
        for j, (q, v) in enumerate(zip(lg.controls, lg.control_values)):
            o.controls[j] = q
            o.control_values[j] = v
        o.matrix = _abi.dptr(buf)
        res.append((bytes(o), buf))
    if key is not None:
        if len(_LOWER_CACHE) >= _LOWER_CACHE_MAX:
            _LOWER_CACHE.clear()
        _LOWER_CACHE[key] = res
    return res


PRECISIONS = {"c128": _abi.BS_PREC_C128, "c64": _abi.BS_PREC_C64}


class _Handle:
    """Owns one engine handle (bs_sim*)."""

    def __init__(self, kind: int, n: int, precision: str = "c128"):
        self._lib = _abi.lib()
        h = C.c_void_p()
        rc = self._lib.bs_create(kind, n, PRECISIONS[precision], C.byref(h))
        if rc != 0:
            raise _abi.BraketGB300Error(rc, "bs_create failed")
        self.h = h

    def call(self, name, *args):
        _abi.check(self.h, getattr(self._lib, name)(self.h, *args))

    def close(self):
        if self.h:
            self._lib.bs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AbstractSimulator:
    kind = _abi.BS_KIND_SV

    def __init__(self, qubit_count: int, shots: int = 0, noise_mode: str = "reference", precision: str = "c128"):
        """precision "c128" (complex128 state) or "c64" (complex64 state, FP32 gate arithmetic,
        probabilities / expectations / sampling still accumulated at FP64 accuracy)."""
        self.qubit_count = int(qubit_count)
        self.shots = int(shots)
        self.noise_mode = noise_mode
        self.precision = precision
        self._h = _Handle(self.kind, self.qubit_count, precision)
        self._obs = None
        self.seed = 0

    # ---- lifecycle
    def reinit(self, qubit_count: int, shots: int):
        """reinit! (src/sv_simulator.jl:96-127, src/dm_simulator.jl:96-128)."""
        self._h.call("bs_reinit", int(qubit_count))
        self.qubit_count = int(qubit_count)
        self.shots = int(shots)
        self._obs = None
        return self

    def similar(self, shots: int | None = None):
        return type(self)(self.qubit_count, self.shots if shots is None else shots, self.noise_mode, self.precision)

    def copy(self):
        s = self.similar()
        s._h.call("bs_copy_state", self._h.h)
        return s

    def copyto(self, src):
        self._h.call("bs_copy_state", src._h.h)
        return self

    # ---- evolution
    def evolve(self, instructions: Sequence[Instruction]):
        """evolve! (src/sv_simulator.jl:140-148, src/dm_simulator.jl:170-179)."""
        arr, n, keep = _ops_for(instructions, self.kind == _abi.BS_KIND_DM, NOISE_MODES[self.noise_mode])
        self._h.call("bs_evolve", arr, n, NOISE_MODES[self.noise_mode])
        del keep
        return self

    def apply_gate(self, gate: Gate, *targets: int):
        return self.evolve([Instruction(gate, list(targets))])

    def last_stats(self) -> dict:
        st = _abi.BsStats()
        self._h.call("bs_last_stats", C.byref(st))
        return {"sweeps": st.sweeps, "kernel_launches": st.kernel_launches, "gates": st.gates,
                "bytes_moved": st.bytes_moved, "gpu_ms": st.gpu_ms, "tc_gates": st.tc_gates,
                "tc_launches": st.tc_launches, "tc_ms": st.tc_ms}

    # ---- state
    def _get(self) -> np.ndarray:
        n = (1 << self.qubit_count) if self.kind == _abi.BS_KIND_SV else (1 << (2 * self.qubit_count))
        out = np.empty(n, dtype=np.complex128)
        self._h.call("bs_get_state", _abi.dptr(out.view(np.float64)), n)
        return out

    def _set(self, v: np.ndarray):
        v = np.ascontiguousarray(np.asarray(v, dtype=np.complex128).ravel(order="F"))
        self._h.call("bs_set_state", _abi.dptr(v.view(np.float64)), v.size)

    def probabilities(self) -> np.ndarray:
        n = 1 << self.qubit_count
        out = np.empty(n, dtype=np.float64)
        self._h.call("bs_probabilities", _abi.dptr(out), n)
        return out

    # ---- expectations
    def expectation(self, observable: Observable, *targets: int) -> float:
        return _expectation(self, observable, tuple(int(t) for t in targets))

    def apply_observables(self, observables):
        """apply_observables! (src/sv_simulator.jl:256-265, src/dm_simulator.jl:232-243)."""
        if self._obs is not None:
            raise RuntimeError("observables have already been applied.")
        ops = []
        for obs, targets in observables:
            ops.extend(diagonalizing_gates(obs, targets))
        cp = self.copy()
        cp.evolve(ops)
        self._obs = cp
        return self

    def state_with_observables(self):
        if self._obs is None:
            raise RuntimeError("observables have not been applied.")
        return self._obs._state_value()

    # ---- sampling
    def samples(self, seed: int | None = None) -> np.ndarray:
        """samples (src/result_types.jl:56-80): shots basis indices (0-based)."""
        out = np.empty(self.shots, dtype=np.int64)
        if seed is None:
            self.seed += 1
            seed = self.seed
        self._h.call("bs_sample", C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), self.shots, _abi.i64ptr(out))
        return out

    def samples_from_stream(self, j: np.ndarray, u: np.ndarray, wsum: float | None = None,
                            probabilities: np.ndarray | None = None, parallel: bool = False) -> np.ndarray:
        """Alias-table draws on a supplied stream: j plays rand(rng, 1:N) - 1, u plays rand(rng).
        With ``probabilities`` the table is built from that vector (bit-exact with the reference's
        make_alias_table! given the same wsum); otherwise from the simulator's state, serially in the
        reference's order or, with ``parallel``, by the parallel construction (same distribution,
        another table)."""
        j = np.ascontiguousarray(j, dtype=np.int64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        if probabilities is not None:
            p = np.ascontiguousarray(probabilities, dtype=np.float64)
            ws = float(np.sum(p)) if wsum is None else float(wsum)
            self._h.call("bs_alias_build_from", _abi.dptr(p), p.size, ws)
        else:
            self.alias_build(wsum, parallel)
        out = np.empty(j.size, dtype=np.int64)
        self._h.call("bs_sample_alias", _abi.i64ptr(j), _abi.dptr(u), j.size, _abi.i64ptr(out))
        return out

    def alias_build(self, wsum: float | None = None, parallel: bool = False):
        """Alias table of the current probabilities on the device (make_alias_table!,
        src/result_types.jl:8-54): serial in the reference's order, or the parallel construction."""
        flags = _abi.BS_ALIAS_PARALLEL if parallel else _abi.BS_ALIAS_EXACT
        self._h.call("bs_alias_build", -1.0 if wsum is None else float(wsum), flags)

    def alias_table(self):
        n = 1 << self.qubit_count
        ap = np.empty(n, dtype=np.float64)
        al = np.empty(n, dtype=np.int64)
        self._h.call("bs_alias_table", _abi.dptr(ap), _abi.i64ptr(al), n)
        return ap, al

    def samples_direct(self, u: np.ndarray, wsum: float = -1.0) -> np.ndarray:
        """Inverse-CDF draws (the reference's >= 30-qubit path) on a supplied uniform stream."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty(u.size, dtype=np.int64)
        self._h.call("bs_sample_direct", _abi.dptr(u), u.size, float(wsum), _abi.i64ptr(out))
        return out

    def reduced_density_matrix(self, qubits) -> np.ndarray:
        """Partial trace keeping ``qubits`` (1..16 of them), on the device; row/column index bit r
        belongs to the r-th highest-numbered kept qubit (the reference's loop order)."""
        q = np.ascontiguousarray(list(qubits), dtype=np.int32)
        d = 1 << q.size
        out = np.empty(2 * d * d, dtype=np.float64)
        self._h.call("bs_reduced_density_matrix", int(q.size), _abi.iptr(q), _abi.dptr(out))
        return out.view(np.complex128).reshape(d, d)

    def write_result_file(self, what: str, path) -> int:
        """Write ``"state"`` (state-vector simulators: 2^n complex128) or ``"probabilities"``
        (2^n float64) from the device straight to ``path``, in the byte layout of the reference's
        memory-mapped result values; returns the number of bytes written."""
        code = {"state": _abi.BS_FILE_STATE, "probabilities": _abi.BS_FILE_PROBABILITIES}[what]
        n = C.c_int64()
        self._h.call("bs_write_result_file", code, os.fsencode(os.fspath(path)), C.byref(n))
        return n.value

    def marginal_probabilities(self, targets) -> np.ndarray:
        t = np.ascontiguousarray(targets, dtype=np.int32)
        out = np.empty(1 << t.size, dtype=np.float64)
        self._h.call("bs_marginal_probabilities", int(t.size), _abi.iptr(t), _abi.dptr(out))
        return out

    def close(self):
        self._h.close()


class StateVectorSimulator(AbstractSimulator):
    """StateVectorSimulator(qubit_count, shots) (src/sv_simulator.jl:6-68)."""
    kind = _abi.BS_KIND_SV
    device_id = "braket_sv_v2"

    @property
    def state_vector(self) -> np.ndarray:
        return self._get()

    @state_vector.setter
    def state_vector(self, v):
        self._set(v)

    def run(self, instructions: Sequence[Instruction], shots: int | None = None, seed: int | None = None,
            probabilities: bool = True):
        """simulate of one circuit from |0...0> (src/BraketSimulator.jl:307-322: reinit!, evolve!, then
        probabilities and samples) in one round trip to the GPU for states of at most 12 qubits:
        returns (probabilities or None, samples).  The samples are those ``samples(seed)`` draws after
        ``reinit`` and ``evolve``; the simulator keeps the final state."""
        shots = self.shots if shots is None else int(shots)
        if seed is None:
            self.seed += 1
            seed = self.seed
        arr, n_ops, keep = _ops_for(instructions, False, 0)
        p = np.empty(1 << self.qubit_count, dtype=np.float64) if probabilities else None
        smp = np.empty(shots, dtype=np.int64)
        self._h.call("bs_run_small", arr, n_ops, shots, C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF),
                     _addr(p) if p is not None else None, _addr(smp))
        del keep
        self._obs = None
        return p, smp

    def density_matrix(self) -> np.ndarray:
        """psi psi^dagger (src/sv_simulator.jl:151-152), formed on the device (at most 16 qubits)."""
        return self.reduced_density_matrix(range(self.qubit_count))

    def _state_value(self):
        return self._get()

    def __repr__(self):
        return f"StateVectorSimulator(qubit_count={self.qubit_count}, shots={self.shots})"


class DensityMatrixSimulator(AbstractSimulator):
    """DensityMatrixSimulator(qubit_count, shots) (src/dm_simulator.jl:6-65).

    ``noise_mode="reference"`` reproduces the reference's block-diagonal Kraus update;
    ``"physical"`` applies the full channel to every element."""
    kind = _abi.BS_KIND_DM
    device_id = "braket_dm_v2"

    @property
    def density_matrix(self) -> np.ndarray:
        d = 1 << self.qubit_count
        return self._get().reshape((d, d), order="F")

    @density_matrix.setter
    def density_matrix(self, m):
        self._set(np.asarray(m, dtype=np.complex128))

    def _state_value(self):
        return self.density_matrix

    def apply_noise(self, noise: Noise, *targets: int):
        return self.evolve([Instruction(noise, list(targets))])

    def __repr__(self):
        return f"DensityMatrixSimulator(qubit_count={self.qubit_count}, shots={self.shots})"


# ----------------------------------------------------------------------------- expectation
def _permute_bits(m: np.ndarray, src: Sequence[int], dst: Sequence[int]) -> np.ndarray:
    """Re-index a matrix whose index bit j belongs to qubit src[j] so that bit j belongs to dst[j]."""
    k = len(src)
    pos = [list(src).index(q) for q in dst]
    d = 1 << k
    perm = np.zeros(d, dtype=np.int64)
    for new in range(d):
        old = 0
        for j in range(k):
            if (new >> j) & 1:
                old |= 1 << pos[j]
        perm[new] = old
    return m[np.ix_(perm, perm)]


def _factor_matrix_lsb(obs, targets, dm: bool) -> np.ndarray:
    """Factor matrix in the convention 'bit j <-> targets[j]' as the reference applies it."""
    if isinstance(obs, StandardObservable):
        return obs.matrix
    m = obs.matrix
    k = len(targets)
    if dm or k >= 3:
        # reference: matrix bit j <-> j-th largest qubit index (sorted kernels)
        sorted_q = sorted(targets, reverse=True)
        return _permute_bits(m, sorted_q, list(targets))
    if k == 2:
        # SV 2-target Hermitian kernel: (00, t2 flipped, t1 flipped, 11) -> bit0 <-> t2
        return _permute_bits(m, [targets[1], targets[0]], list(targets))
    return m


def _pauli_terms(factors_targets):
    """Expand a product of X/Y/Z/H/I factors into Pauli strings (x, z masks, coefficient)."""
    terms = [(0, 0, 1.0)]
    for f, t in factors_targets:
        b = 1 << t
        if isinstance(f, I):
            continue
        if isinstance(f, X):
            opts = [(b, 0, 1.0)]
        elif isinstance(f, Z):
            opts = [(0, b, 1.0)]
        elif isinstance(f, Y):
            opts = [(b, b, 1.0)]
        elif isinstance(f, H):
            opts = [(b, 0, 1 / math.sqrt(2)), (0, b, 1 / math.sqrt(2))]
        else:
            return None
        terms = [(x | ox, z | oz, c * oc) for (x, z, c) in terms for (ox, oz, oc) in opts]
    return terms


def _split_factors(observable, targets):
    if isinstance(observable, TensorProduct):
        out, i = [], 0
        for f in observable.factors:
            k = f.qubit_count()
            out.append((f, tuple(targets[i:i + k])))
            i += k
        return out
    return [(observable, tuple(targets))]


def _expectation(sim, observable, targets) -> float:
    """expectation (src/sv_simulator.jl:240-248, src/dm_simulator.jl:253-260).  Like the
    reference, coefficients of the observable are not applied."""
    dm = sim.kind == _abi.BS_KIND_DM
    parts = _split_factors(observable, targets)
    # the reference applies a standard observable given several targets on each of them
    flat = []
    for f, t in parts:
        if isinstance(f, StandardObservable):
            flat.extend((type(f)(), q) for q in t)
        else:
            flat.append((f, t))
    if all(isinstance(f, StandardObservable) for f, _ in flat):
        terms = _pauli_terms(flat)
        xm = np.array([x for x, _, _ in terms], dtype=np.uint64)
        zm = np.array([z for _, z, _ in terms], dtype=np.uint64)
        co = np.array([c for _, _, c in terms], dtype=np.float64)
        out = np.empty(len(terms), dtype=np.float64)
        sim._h.call("bs_expectation_pauli", len(terms), _abi.u64ptr(xm), _abi.u64ptr(zm), _abi.dptr(co), _abi.dptr(out))
        return float(np.sum(out))
    # general: kron of factor matrices, bit j <-> all_targets[j]
    all_t = []
    full = np.ones((1, 1), dtype=np.complex128)
    for f, t in flat:
        ft = (t,) if isinstance(t, int) else tuple(t)
        m = _factor_matrix_lsb(f, list(ft), dm)
        full = np.kron(m, full)        # later factors take the higher bits
        all_t.extend(ft)
    buf = _abi.cplx_buffer(full)
    tt = np.array(all_t, dtype=np.int32)
    out = np.empty(1, dtype=np.float64)
    sim._h.call("bs_expectation_matrix", _abi.dptr(buf), len(all_t), _abi.iptr(tt), 0, _abi.dptr(out))
    return float(out[0])


# ----------------------------------------------------------------------------- module-level API
def evolve(sim, instructions):
    return sim.evolve(instructions)


def reinit(sim, qubit_count, shots):
    return sim.reinit(qubit_count, shots)


def probabilities(sim):
    return sim.probabilities()


def expectation(sim, observable, *targets):
    return sim.expectation(observable, *targets)


def samples(sim, seed=None):
    return sim.samples(seed)


def state_vector(sim):
    return sim.state_vector.copy()


def density_matrix(sim):
    return sim.density_matrix() if isinstance(sim, StateVectorSimulator) else sim.density_matrix.copy()


def apply_observables(sim, observables):
    return sim.apply_observables(observables)


def state_with_observables(sim):
    return sim.state_with_observables()


def qubit_count(sim):
    return sim.qubit_count
