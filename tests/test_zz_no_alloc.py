"""The allocation-free expectation entry point.

It exists for callers that cannot allocate GPU memory at the moment they ask for an
expectation value (their runtime owns all of HBM, or a cudaMalloc would stall a
real-time loop).  Its results must equal those of the allocating entry point, on the
same state, call after call: the static scratch array it reuses must not leak one
call's partial sums into the next.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import bs, random_circuit

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _terms(n, rng, count):
    xs = [0] + [int(rng.integers(0, 2 ** n)) for _ in range(count - 1)]
    zs = [int(rng.integers(0, 2 ** n)) for _ in range(count)]
    xs[1] = xs[2] = xs[3]          # several terms sharing one flip mask
    return np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64), rng.normal(size=count)


@pytest.mark.parametrize("kind", ["sv", "dm"])
def test_noalloc_expectation_equals_allocating_one(kind):
    lib = bs._abi.lib()
    rng = np.random.default_rng(2024)
    n = 13 if kind == "sv" else 6
    cls = bs.StateVectorSimulator if kind == "sv" else bs.DensityMatrixSimulator
    sim = cls(n, 0).evolve(random_circuit(n, 40, rng))
    xm, zm, co = _terms(n, rng, 20)
    ref = np.empty(xm.size)
    sim._h.call("bs_expectation_pauli", xm.size, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm), bs._abi.dptr(co),
                bs._abi.dptr(ref))
    ptr = C.c_void_p()
    sim._h.call("bs_state_device_ptr", C.byref(ptr))
    k = bs._abi.BS_KIND_SV if kind == "sv" else bs._abi.BS_KIND_DM
    for _ in range(2):          # two calls in a row on the shared scratch array
        out = np.full(xm.size, np.nan)
        rc = lib.bs_expectation_pauli_noalloc(ptr, k, n, xm.size, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm),
                                              bs._abi.dptr(co), bs._abi.dptr(out), None)
        assert rc == 0
        assert np.max(np.abs(out - ref)) < TOL


def _oracle_terms(psi_or_rho, n, kind, xm, zm, co):
    f = oracle.expectation_pauli_sv if kind == "sv" else oracle.expectation_pauli_dm
    return np.array([c * f(psi_or_rho, n, int(x), int(z)) for x, z, c in zip(xm, zm, co)])


@pytest.mark.parametrize("kind,n", [("sv", 18), ("sv", 21), ("dm", 10)])
def test_noalloc_full_scratch_on_a_caller_stream_vs_oracle(kind, n):
    """The largest request the scratch array takes: 32 terms, one flip mask shared by 13 terms
    (two passes over the state for that mask, the first flushed at 8 terms) and, for the state
    vectors, a grid at the 512-block cap, so the partial sums fill all 512 x 32 slots; on a
    stream the caller created; two calls in a row, each against the FP64 oracle's expectation
    of the same state and against the allocating entry point."""
    import torch
    lib = bs._abi.lib()
    rng = np.random.default_rng(77 + n)
    cls = bs.StateVectorSimulator if kind == "sv" else bs.DensityMatrixSimulator
    sim = cls(n, 0).evolve(random_circuit(n, 30, rng))
    xm = np.array([int(rng.integers(0, 2 ** n)) for _ in range(32)], dtype=np.uint64)
    zm = np.array([int(rng.integers(0, 2 ** n)) for _ in range(32)], dtype=np.uint64)
    xm[3:15] = xm[2]              # 13 terms share one flip mask
    xm[20] = 0                    # and one diagonal term
    co = rng.normal(size=32)
    ref = np.empty(32)
    sim._h.call("bs_expectation_pauli", 32, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm), bs._abi.dptr(co),
                bs._abi.dptr(ref))
    state = sim.state_vector if kind == "sv" else sim.density_matrix.ravel(order="F")
    exact = _oracle_terms(state, n, kind, xm, zm, co)
    assert np.max(np.abs(ref - exact)) < TOL
    ptr = C.c_void_p()
    sim._h.call("bs_state_device_ptr", C.byref(ptr))
    k = bs._abi.BS_KIND_SV if kind == "sv" else bs._abi.BS_KIND_DM
    stream = torch.cuda.Stream()
    for _ in range(2):
        out = np.full(32, np.nan)
        rc = lib.bs_expectation_pauli_noalloc(ptr, k, n, 32, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm),
                                              bs._abi.dptr(co), bs._abi.dptr(out), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        assert np.max(np.abs(out - exact)) < TOL
        assert np.max(np.abs(out - ref)) < TOL


def test_noalloc_rejects_requests_beyond_its_scratch():
    lib = bs._abi.lib()
    sim = bs.StateVectorSimulator(4, 0)
    ptr = C.c_void_p()
    sim._h.call("bs_state_device_ptr", C.byref(ptr))
    xm = np.zeros(33, dtype=np.uint64)
    zm = np.ones(33, dtype=np.uint64)
    out = np.empty(33)
    rc = lib.bs_expectation_pauli_noalloc(ptr, 0, 4, 33, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm), None,
                                          bs._abi.dptr(out), None)
    assert rc == 5          # BS_ERR_UNSUPPORTED: more terms than the static array holds
