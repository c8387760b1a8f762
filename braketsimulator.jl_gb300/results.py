"""Result types and ``calculate`` (src/result_types.jl:82-246, src/results.jl)."""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

from .observables import HermitianObservable, I, Observable, StandardObservable, TensorProduct
from .simulators import DensityMatrixSimulator, StateVectorSimulator


@dataclass
class StateVector:
    pass


@dataclass
class Amplitude:
    states: list


@dataclass
class Probability:
    targets: tuple = ()


@dataclass
class DensityMatrix:
    targets: tuple = ()


@dataclass
class Expectation:
    observable: Observable
    targets: tuple = ()


@dataclass
class Variance:
    observable: Observable
    targets: tuple = ()


@dataclass
class Sample:
    observable: Observable
    targets: tuple = ()


def marginal_probability(probs: np.ndarray, qubit_count: int, targets) -> np.ndarray:
    """src/result_types.jl:96-113 on a host vector a caller holds: output bit j <-> j-th smallest
    endian target.  Simulators compute marginals on the device (``marginal_probabilities``)."""
    targets = list(targets)
    p = np.asarray(probs, dtype=np.float64).reshape([2] * qubit_count) if qubit_count else np.asarray(probs)
    unused = [q for q in range(qubit_count) if q not in targets]
    # axis a of the reshaped array is qubit a (C order: qubit 0 = most significant)
    m = p.sum(axis=tuple(unused)) if unused else p
    kept = sorted(targets)
    return np.ascontiguousarray(m).reshape(-1) if kept else np.array([float(np.sum(p))])


def _permuted_indices(qubit_count: int, targets) -> np.ndarray:
    """new index of every ix (vectorised): bit q of new = bit (qubit_count - targets[q] - 1) of ix."""
    t = list(targets)
    ix = np.arange(1 << len(t), dtype=np.int64)
    new = np.zeros_like(ix)
    for q, tt in enumerate(t[:qubit_count]):
        new |= ((ix >> (qubit_count - tt - 1)) & 1) << q
    return new


def permute_probability(probs: np.ndarray, qubit_count: int, targets) -> np.ndarray:
    """src/result_types.jl:115-127 (assignment in ascending ix: the last write to a slot wins)."""
    new = _permuted_indices(qubit_count, targets)
    out = np.zeros(new.size)
    rev = new[::-1]
    _, first = np.unique(rev, return_index=True)
    out[rev[first]] = np.asarray(probs)[: new.size][::-1][first]
    return out


def permute_density_matrix(rho: np.ndarray, qubit_count: int, targets) -> np.ndarray:
    """src/result_types.jl:129-149 (assignment in row-major order: the last write wins)."""
    new = _permuted_indices(qubit_count, targets)
    d = new.size
    out = np.zeros((d, d), dtype=rho.dtype)
    tgt = (new[:, None] * d + new[None, :]).ravel()[::-1]
    _, first = np.unique(tgt, return_index=True)
    out.ravel()[tgt[first]] = np.asarray(rho)[:d, :d].ravel()[::-1][first]
    return out


def _jshl(x, k):
    """Julia's x << k: a negative count shifts the other way."""
    return x << k if k >= 0 else x >> -k


def _swap_bits(ix, mapping):
    """swap_bits (src/dm_simulator.jl:264-278), with Julia's shift semantics: a mapping entry whose
    source bit is negative (unsorted targets numbered beyond the output size) reads as 0 and flips
    only the other bit."""
    for a, b in mapping.items():
        if a < b:
            av = _jshl(_jshl(1, a) & ix, -a)
            bv = _jshl(_jshl(1, b) & ix, -b)
            if av != bv:
                ix ^= _jshl(1, a) ^ _jshl(1, b)
    return ix


def partial_trace(state, output_qubits=None):
    """Reduced density matrix of a host array (src/sv_simulator.jl:273-318 for a vector,
    src/dm_simulator.jl:280-323 for a matrix), the reference's loops restated for arrays a caller
    holds; simulators compute the same on the device (``reduced_density_matrix``)."""
    state = np.asarray(state, dtype=np.complex128)
    vec = state.ndim == 1
    n = int(round(np.log2(state.shape[0])))
    if output_qubits is None:
        output_qubits = list(range(n))
    output_qubits = list(output_qubits)
    if not output_qubits:
        return np.sum(np.abs(state) ** 2) if vec else np.trace(state)
    if len(set(output_qubits)) == n:
        return np.outer(state, state.conj()) if vec else state
    traced = [q for q in range(n) if q not in output_qubits]
    endian = sorted(n - q - 1 for q in traced)
    combos = [()] + [c for r in range(1, len(endian) + 1) for c in itertools.combinations(endian, r)]
    dim = 1 << (n - len(traced))
    out = np.zeros((dim, dim), dtype=np.complex128)
    needs_perm = output_qubits != sorted(output_qubits)
    fn = len(output_qubits)
    mapping = dict(zip([fn - q - 1 for q in output_qubits], [fn - q - 1 for q in range(fn)])) if needs_perm else {}

    def pad(ix):
        for b in endian:
            low = ix & ((1 << b) - 1)
            ix = ((ix >> b) << (b + 1)) | low
        return ix

    for ix in range(dim):
        for jx in range(dim if not vec else dim):
            if vec and jx < ix:
                continue
            pi, pj = pad(ix), pad(jx)
            fi = [pi ^ sum(1 << b for b in c) for c in combos]
            fj = [pj ^ sum(1 << b for b in c) for c in combos]
            oi = _swap_bits(ix, mapping) if needs_perm else ix
            oj = _swap_bits(jx, mapping) if needs_perm else jx
            if vec:
                tr = np.vdot(state[fj], state[fi])
                out[oi, oj] += tr
                if oj != oi:
                    out[oj, oi] += np.conj(tr)
            else:
                out[oi, oj] = np.sum(state[fi, fj])
    return out


def reduced_density_matrix(sim, output_qubits):
    """partial_trace of the simulator's state keeping output_qubits (any order), computed on the
    device; the final reordering of unsorted targets follows ``partial_trace`` above."""
    output_qubits = list(output_qubits)
    out = sim.reduced_density_matrix(output_qubits)
    if output_qubits == sorted(output_qubits):
        return out
    fn = len(output_qubits)
    mapping = dict(zip([fn - q - 1 for q in output_qubits], [fn - q - 1 for q in range(fn)]))
    dim = out.shape[0]
    perm = np.array([_swap_bits(ix, mapping) for ix in range(dim)], dtype=np.int64)
    res = np.zeros_like(out)
    if isinstance(sim, DensityMatrixSimulator):
        # the reference assigns entry by entry in row-major order: the last write to a cell wins
        tgt = (perm[:, None] * dim + perm[None, :]).ravel()[::-1]
        _, first = np.unique(tgt, return_index=True)
        src = out.ravel()[::-1][first]
        res.ravel()[tgt[first]] = src
    else:
        # the reference accumulates over ix <= jx and mirrors the conjugate off the diagonal
        iu, ju = np.triu_indices(dim)
        oi, oj = perm[iu], perm[ju]
        np.add.at(res, (oi, oj), out[iu, ju])
        off = oi != oj
        np.add.at(res, (oj[off], oi[off]), np.conj(out[iu, ju][off]))
    return res


def _targets(rt, sim):
    t = tuple(rt.targets) if rt.targets is not None else ()
    return t if t else tuple(range(sim.qubit_count))


def _op_squared(sim, obs, targets):
    """expectation_op_squared (src/result_types.jl:168-194)."""
    if isinstance(obs, (StandardObservable, I)):
        return 1.0
    if isinstance(obs, TensorProduct):
        if all(isinstance(f, (StandardObservable, I)) for f in obs.factors):
            return 1.0
        sq = [I() if isinstance(f, (StandardObservable, I)) else HermitianObservable(f.matrix @ f.matrix) for f in obs.factors]
        return sim.expectation(TensorProduct(sq), *targets)
    return sim.expectation(HermitianObservable(obs.matrix @ obs.matrix), *targets)


def calculate(rt, sim):
    """calculate (src/result_types.jl:82-246)."""
    n = sim.qubit_count
    if isinstance(rt, StateVector):
        return sim.state_vector.copy()
    if isinstance(rt, Amplitude):
        sv = sim.state_vector
        return {s: sv[int(s, 2)] for s in rt.states}
    if isinstance(rt, Probability):
        t = tuple(rt.targets or ())
        if not t or list(t) == list(range(n)):
            return sim.probabilities()
        if len(t) == n:
            return permute_probability(sim.probabilities(), n, list(t))
        return sim.marginal_probabilities(sorted(t))
    if isinstance(rt, Expectation):
        t = _targets(rt, sim)
        if len(t) == rt.observable.qubit_count():
            return sim.expectation(rt.observable, *t)
        return [sim.expectation(rt.observable, q) for q in t]
    if isinstance(rt, Variance):
        t = _targets(rt, sim)
        if len(t) == rt.observable.qubit_count():
            return _op_squared(sim, rt.observable, t) - sim.expectation(rt.observable, *t) ** 2
        return [_op_squared(sim, rt.observable, (q,)) - sim.expectation(rt.observable, q) ** 2 for q in t]
    if isinstance(rt, DensityMatrix):
        t = tuple(rt.targets or ())
        full = isinstance(sim, DensityMatrixSimulator)
        rho = sim.density_matrix if full else None
        if not t or list(t) == list(range(n)):
            return rho if full else sim.density_matrix()
        if len(t) == n:
            return permute_density_matrix(rho if full else sim.density_matrix(), n, list(t))
        return reduced_density_matrix(sim, list(t))
    raise TypeError(f"unsupported result type {rt!r}")
