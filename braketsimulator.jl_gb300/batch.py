"""Batched simulation of many uneven circuits (the reference's
``simulate(sim, ::Vector, shots; max_parallel)``, src/BraketSimulator.jl:347-395).

``batch_simulate`` lowers every circuit with the same dispatch as ``evolve`` and
hands the whole batch to ``bs_run_batch``: small circuits run whole in one CTA each
inside one persistent launch, larger ones as tile sweeps on a pool of streams.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .adjoint import pauli_masks
from .simulators import PRECISIONS, _ops_for


def batch_simulate(circuits, qubit_counts, observables=(), shots: int = 0, seed: int = 0, precision: str = "c64"):
    """circuits: list of instruction lists; qubit_counts: list of ints;
    observables: per circuit a list of {qubit: 'X'|'Y'|'Z'} Pauli strings (same count for all).
    Returns (expectations [n_circuits, n_terms], samples [n_circuits, shots], stats dict)."""
    nc = len(circuits)
    if nc != len(qubit_counts):
        raise ValueError("one qubit count per circuit")
    n_terms = len(observables[0]) if (len(observables) and nc) else 0
    arrays, keeps, counts = [], [], []
    for ins in circuits:
        arr, n, keep = _ops_for(ins, False, 0)
        arrays.append(arr)
        keeps.append(keep)
        counts.append(n)
    ptrs = (C.POINTER(_abi.BsOp) * max(1, nc))(*[C.cast(a, C.POINTER(_abi.BsOp)) for a in arrays])
    nq = np.array(qubit_counts, dtype=np.int32)
    nops = np.array(counts, dtype=np.int64)
    xm = np.zeros(max(1, nc * n_terms), dtype=np.uint64)
    zm = np.zeros(max(1, nc * n_terms), dtype=np.uint64)
    for c in range(nc):
        if len(observables) and len(observables[c]) != n_terms:
            raise ValueError("every circuit needs the same number of observables")
        for t in range(n_terms):
            xm[c * n_terms + t], zm[c * n_terms + t] = pauli_masks(observables[c][t])
    exp = np.zeros(max(1, nc * n_terms), dtype=np.float64)
    smp = np.zeros(max(1, nc * shots), dtype=np.int64)
    st = _abi.BsStats()
    rc = _abi.lib().bs_run_batch(nc, _abi.iptr(nq), ptrs, _abi.i64ptr(nops), n_terms, _abi.u64ptr(xm), _abi.u64ptr(zm),
                                 int(shots), C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), PRECISIONS[precision],
                                 _abi.dptr(exp), _abi.i64ptr(smp), C.byref(st))
    if rc != 0:
        raise _abi.BraketGB300Error(rc, "bs_run_batch failed")
    del keeps
    stats = {"sweeps": st.sweeps, "kernel_launches": st.kernel_launches, "gates": st.gates,
             "bytes_moved": st.bytes_moved, "gpu_ms": st.gpu_ms, "tc_gates": st.tc_gates,
                "tc_launches": st.tc_launches, "tc_ms": st.tc_ms}
    return exp[: nc * n_terms].reshape(nc, n_terms), smp[: nc * shots].reshape(nc, shots), stats
