"""Parity at the benchmarked configurations' own sizes.

* dense random circuit: the full 2 x 20-layer circuit at 28 qubits against the FP64
  oracle, a shortened circuit at 30 qubits (both passes, strides 1, 8 and 16) against
  the oracle, and the full 30-qubit circuit followed by its inverse, which must give
  back |0...0> (a size-independent property of the benchmarked circuit itself);
  the same at 28 qubits with a dense CNOT in place of CZ;
* noisy density matrix, 14 qubits, depth 12, against the oracle (the reference's noise rule; the
  physical channel at 14 qubits for 2 layers and at 12 qubits for all 12);
* the 512-circuit complex64 batch against the complex128 oracle for every circuit
  of at most 22 qubits.
Amplitude and density-matrix bar: 1e-12 relative (norm-wise); the mirror check
runs twice the depth and is held to the same 1e-12 on the returned |0...0>."""
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT, bs, rel_err

pytestmark = pytest.mark.gpu
sys.path.insert(0, ROOT)
import bench  # noqa: E402  (workload generators of the benchmark)

TOL = 1e-12


def _rel_err_big(a, b, chunk=1 << 24):
    """rel_err for multi-GiB vectors, chunk by chunk (no full-size temporaries)."""
    num = na = nb = 0.0
    for i in range(0, a.size, chunk):
        x, y = a[i:i + chunk], b[i:i + chunk]
        d = x - y
        num += float(np.vdot(d, d).real)
        na += float(np.vdot(x, x).real)
        nb += float(np.vdot(y, y).real)
    return float(np.sqrt(num) / max(np.sqrt(na), np.sqrt(nb), 1e-300))


def _zz(psi, n, a, b):
    """<Z_a Z_b> on the oracle's state."""
    return oracle.expectation_pauli_fast(psi, n, 0, (1 << a) | (1 << b))


@pytest.mark.parametrize("two_qubit", ["cz", "cnot"])
def test_dense_circuit_28q_full_depth_vs_oracle(two_qubit):
    n = 28
    ops = bench.dense_circuit(bs, n=n, two_qubit=two_qubit)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    got = sim.state_vector
    zz = sim.expectation(bs.observables.TensorProduct([bs.observables.Z(), bs.observables.Z()]), 0, n - 1)
    del sim
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert _rel_err_big(got, ref) < TOL
    assert abs(zz - _zz(ref, n, 0, n - 1)) < TOL


def test_dense_circuit_30q_both_passes_vs_oracle():
    """2 brick layers, then 3 layers at strides 1, 8 and 16, on the 16 GiB 30-qubit state."""
    n = 30
    ops = bench.dense_circuit(bs, n=n, layers=2, layers2=3)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    got = sim.state_vector
    zz = sim.expectation(bs.observables.TensorProduct([bs.observables.Z(), bs.observables.Z()]), 0, n - 1)
    del sim
    ref = oracle.OracleSV(n).evolve(ops).psi
    assert _rel_err_big(got, ref) < TOL
    assert abs(zz - _zz(ref, n, 0, n - 1)) < TOL
    del got, ref


def _mirror_error(n, two_qubit="cz"):
    ops = bench.dense_circuit(bs, n=n, two_qubit=two_qubit)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    st = sim.last_stats()
    sim.evolve(bench.inverse_circuit(bs, ops))
    psi = sim.state_vector
    rest = 0.0
    for i in range(1, psi.size, 1 << 24):
        x = psi[i:i + (1 << 24)]
        rest += float(np.vdot(x, x).real)
    err = np.sqrt(abs(psi[0] - 1.0) ** 2 + rest)
    del psi
    return err, st


def test_dense_circuit_30q_mirror_returns_to_zero_state():
    """The benchmarked 30-qubit circuit (all 1777 gates, the same fused tensor-core sweeps the
    benchmark times), then its inverse: |0...0> back to 1e-12."""
    err, st = _mirror_error(30)
    assert st["tc_gates"] > 0
    assert err < TOL


def test_dense_circuit_cnot_28q_mirror():
    err, _ = _mirror_error(28, "cnot")
    assert err < TOL


@pytest.mark.parametrize("mode,n,layers", [("reference", 14, 12), ("physical", 14, 2), ("physical", 12, 12)])
def test_noisy_dm_circuit_vs_oracle(mode, n, layers):
    """The noisy density-matrix workload: 14 qubits at full depth in the reference's noise rule; the
    physical channel (whose oracle applies every channel to all 4^n elements on the host) at 14 qubits
    for the first 2 of its 12 layers and at 12 qubits for all 12."""
    ops = bench.dm_circuit(bs, n=n)
    ops = ops[: len(ops) * layers // 12]
    sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode).evolve(ops)
    got = sim.density_matrix.ravel(order="F")          # vec(S), a view
    diag = sim.probabilities()
    x4 = sim.expectation(bs.observables.TensorProduct([bs.observables.X()] * 4), 0, 1, 2, 3)
    del sim
    ref = oracle.OracleDM(n, physical=(mode == "physical")).evolve(ops)
    assert _rel_err_big(got, ref.rho) < TOL
    assert rel_err(diag, ref.probabilities()) < TOL
    ex = oracle.expectation_pauli_dm(ref.rho, n, 0b1111, 0)
    assert abs(x4 - ex) < TOL


def test_batch512_complex64_vs_complex128_oracle():
    """The benchmark's 512 uneven circuits in complex64 (FP64 reductions): every expectation of
    every circuit of <= 22 qubits against the complex128 oracle, error stated per result."""
    circuits, counts, obs = bench.batch_circuits(bs)
    exp, smp, st = bs.batch_simulate(circuits, counts, obs, shots=1000, seed=2, precision="c64")
    errs = []
    for c, (ins, n, terms) in enumerate(zip(circuits, counts, obs)):
        if n > 22:
            continue
        psi = oracle.OracleSV(n).evolve(ins).psi
        for t, term in enumerate(terms):
            x = sum(1 << q for q, p in term.items() if p in "XY")
            z = sum(1 << q for q, p in term.items() if p in "YZ")
            errs.append(abs(exp[c, t] - oracle.expectation_pauli_fast(psi, n, x, z)))
        assert np.all(np.abs(psi[smp[c]]) ** 2 > 1e-14)     # shots land on populated states
    assert len(errs) > 8 * 300
    assert max(errs) < 2e-5
