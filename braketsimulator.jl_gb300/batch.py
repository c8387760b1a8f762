"""Batched simulation of many uneven circuits (the reference's
``simulate(sim, ::Vector, shots; max_parallel)``, src/BraketSimulator.jl:347-395).

``batch_simulate`` lowers every circuit with the same dispatch as ``evolve`` and
hands the whole batch to ``bs_run_batch``: small circuits run whole in one CTA each
inside one persistent launch, larger ones as tile sweeps on a pool of streams.
``CapturedBatch`` captures the same work once into a CUDA graph and replays it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .adjoint import pauli_masks
from .simulators import PRECISIONS, _ops_for


def _lower_all(circuits):
    arrays, keeps, counts = [], [], []
    for ins in circuits:
        arr, n, keep = _ops_for(ins, False, 0)
        arrays.append(arr)
        keeps.append(keep)
        counts.append(n)
    ptrs = (C.POINTER(_abi.BsOp) * max(1, len(circuits)))(*[C.cast(a, C.POINTER(_abi.BsOp)) for a in arrays])
    return ptrs, np.array(counts, dtype=np.int64), (arrays, keeps)


def _masks(observables, nc):
    n_terms = len(observables[0]) if (len(observables) and nc) else 0
    xm = np.zeros(max(1, nc * n_terms), dtype=np.uint64)
    zm = np.zeros(max(1, nc * n_terms), dtype=np.uint64)
    for c in range(nc):
        if len(observables) and len(observables[c]) != n_terms:
            raise ValueError("every circuit needs the same number of observables")
        for t in range(n_terms):
            xm[c * n_terms + t], zm[c * n_terms + t] = pauli_masks(observables[c][t])
    return n_terms, xm, zm


def _stats(st) -> dict:
    return {"sweeps": st.sweeps, "kernel_launches": st.kernel_launches, "gates": st.gates,
            "bytes_moved": st.bytes_moved, "gpu_ms": st.gpu_ms, "tc_gates": st.tc_gates,
            "tc_launches": st.tc_launches, "tc_ms": st.tc_ms}


def batch_simulate(circuits, qubit_counts, observables=(), shots: int = 0, seed: int = 0, precision: str = "c64"):
    """circuits: list of instruction lists; qubit_counts: list of ints;
    observables: per circuit a list of {qubit: 'X'|'Y'|'Z'} Pauli strings (same count for all).
    Returns (expectations [n_circuits, n_terms], samples [n_circuits, shots], stats dict)."""
    nc = len(circuits)
    if nc != len(qubit_counts):
        raise ValueError("one qubit count per circuit")
    ptrs, nops, keeps = _lower_all(circuits)
    nq = np.array(qubit_counts, dtype=np.int32)
    n_terms, xm, zm = _masks(observables, nc)
    exp = np.zeros(max(1, nc * n_terms), dtype=np.float64)
    smp = np.zeros(max(1, nc * shots), dtype=np.int64)
    st = _abi.BsStats()
    rc = _abi.lib().bs_run_batch(nc, _abi.iptr(nq), ptrs, _abi.i64ptr(nops), n_terms, _abi.u64ptr(xm), _abi.u64ptr(zm),
                                 int(shots), C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), PRECISIONS[precision],
                                 _abi.dptr(exp), _abi.i64ptr(smp), C.byref(st))
    if rc != 0:
        raise _abi.BraketGB300Error(rc, "bs_run_batch failed")
    del keeps
    return exp[: nc * n_terms].reshape(nc, n_terms), smp[: nc * shots].reshape(nc, shots), _stats(st)


class CapturedBatch:
    """The batch of ``batch_simulate`` captured once into a CUDA graph (``bs_batch_create``) and
    replayed by ``launch()``; ``set_circuits`` swaps in new circuits of the same qubit counts (e.g.
    new parameters of a variational ansatz) and updates the graph.  A replay repeats the same shot
    seeds.  The first results come from the eager run inside the constructor's capture step."""

    def __init__(self, circuits, qubit_counts, observables=(), shots: int = 0, seed: int = 0,
                 precision: str = "c64"):
        self.nc = len(circuits)
        if self.nc != len(qubit_counts) or self.nc == 0:
            raise ValueError("one qubit count per circuit, at least one circuit")
        self.shots = int(shots)
        ptrs, nops, keeps = _lower_all(circuits)
        self._nq = np.array(qubit_counts, dtype=np.int32)
        self.n_terms, xm, zm = _masks(observables, self.nc)
        h = C.c_void_p()
        rc = _abi.lib().bs_batch_create(self.nc, _abi.iptr(self._nq), ptrs, _abi.i64ptr(nops), self.n_terms,
                                        _abi.u64ptr(xm), _abi.u64ptr(zm), self.shots,
                                        C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), PRECISIONS[precision], C.byref(h))
        del keeps
        if rc != 0:
            raise _abi.BraketGB300Error(rc, "bs_batch_create failed")
        self._h = h

    def set_circuits(self, circuits):
        if len(circuits) != self.nc:
            raise ValueError("same number of circuits")
        ptrs, nops, keeps = _lower_all(circuits)
        rc = _abi.lib().bs_batch_set_ops(self._h, ptrs, _abi.i64ptr(nops))
        del keeps
        if rc != 0:
            raise _abi.BraketGB300Error(rc, "bs_batch_set_ops failed")

    def set_tuning(self, **values):
        """Tunables (see ``autotune.PARAMS``) on every handle of the batch, then a graph rebuild;
        None restores the environment / default value."""
        from .autotune import PARAMS
        for name in values:
            if name not in PARAMS:
                raise KeyError(f"unknown tunable {name!r}")
        ids = np.array([PARAMS[k] for k in values], dtype=np.int32)
        vals = np.array([-1.0 if v is None else float(v) for v in values.values()], dtype=np.float64)
        rc = _abi.lib().bs_batch_set_tuning(self._h, len(ids), _abi.iptr(ids), _abi.dptr(vals))
        if rc != 0:
            raise _abi.BraketGB300Error(rc, "bs_batch_set_tuning failed")

    def autotune(self, candidates=None, repeats: int = 2) -> dict:
        """Time replays under each candidate setting (default: tile bits x sweep threads, and for
        complex128 the tensor-core fusion widths) and keep the fastest."""
        import time
        from .autotune import PARAMS
        if candidates is None:
            candidates = [{"tile_bits": tb, "tile_threads": thr, "tc": 0} for tb in (10, 11, 12) for thr in (256, 512)]
            candidates += [{"tile_bits": 12, "tc": 1, "tc_min_bits": 0, "tc_cost": c} for c in (1.0, 2.0, 4.0)]
        timings = []
        for cand in candidates:
            self.set_tuning(**{**{k: None for k in PARAMS}, **cand})
            self.launch()
            best = float("inf")
            for _ in range(max(1, repeats)):
                t0 = time.perf_counter()
                self.launch()
                best = min(best, time.perf_counter() - t0)
            timings.append({"setting": cand, "seconds": best})
        win = min(timings, key=lambda r: r["seconds"])
        self.set_tuning(**{**{k: None for k in PARAMS}, **win["setting"]})
        return {"setting": win["setting"], "seconds": win["seconds"], "timings": timings}

    def launch(self):
        """Replay; returns (expectations [n_circuits, n_terms], samples [n_circuits, shots], stats)."""
        exp = np.zeros(max(1, self.nc * self.n_terms), dtype=np.float64)
        smp = np.zeros(max(1, self.nc * self.shots), dtype=np.int64)
        st = _abi.BsStats()
        rc = _abi.lib().bs_batch_launch(self._h, _abi.dptr(exp), _abi.i64ptr(smp), C.byref(st))
        if rc != 0:
            raise _abi.BraketGB300Error(rc, "bs_batch_launch failed")
        nc, nt, ns = self.nc, self.n_terms, self.shots
        return exp[: nc * nt].reshape(nc, nt), smp[: nc * ns].reshape(nc, ns), _stats(st)

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().bs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
