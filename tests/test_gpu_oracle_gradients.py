"""Adjoint gradients against the FP64 oracle's parameter-shift rule.

The engine's adjoint sweep and the oracle share no code: the oracle evaluates
2 shifted circuits per parameter on its own CPU restatement of the reference's
kernels (oracle.parameter_shift_gradient), exact for Rx/Ry/Rz/XX/YY/ZZ/PhaseShift.
Bar: max |grad - oracle| <= 1e-10 for complex128 states."""
import os
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT, bs

pytestmark = pytest.mark.gpu
from importlib import import_module  # noqa: E402

adj = import_module("braketsimulator_gb300.adjoint")
sys.path.insert(0, ROOT)
import bench  # noqa: E402  (workload generators of the benchmark)

TOL = 1e-10


def all_generators_ansatz(n, layers, rng):
    """Every differentiable generator, on near and far qubit pairs."""
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    for _ in range(layers):
        for q in range(n):
            g = [bs.Rx, bs.Ry, bs.Rz, bs.PhaseShift][rng.integers(4)]
            ops.append(bs.Instruction(g(float(rng.uniform(-np.pi, np.pi))), [q]))
        for q in range(0, n - 1, 2):
            r = int(rng.integers(1, n))
            pair = [q, (q + r) % n] if (q + r) % n != q else [q, (q + 1) % n]
            g = [bs.XX, bs.YY, bs.ZZ][rng.integers(3)]
            ops.append(bs.Instruction(g(float(rng.uniform(-np.pi, np.pi))), pair))
        ops.append(bs.Instruction(bs.CNot(), [n - 1, 0]))
    return ops


def hamiltonian(n, terms, rng):
    h = []
    for _ in range(terms):
        w = int(rng.integers(1, min(4, n) + 1))
        qs = rng.choice(n, w, replace=False)
        h.append((float(rng.normal()), {int(q): "XYZ"[rng.integers(3)] for q in qs}))
    return h


@pytest.mark.parametrize("n,layers", [(3, 2), (8, 3), (12, 2)])
def test_adjoint_vs_oracle_parameter_shift_every_generator(n, layers):
    rng = np.random.default_rng(500 + n)
    ops = all_generators_ansatz(n, layers, rng)
    h = hamiltonian(n, 12, rng)
    e, g = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0), ops, h)
    e_ref, gref = oracle.parameter_shift_gradient(n, ops, h)
    pidx = adj.parameterised(ops)
    assert sorted(gref) == pidx
    assert abs(e - e_ref) < 1e-12
    ref = np.array([gref[i] for i in pidx])
    assert np.max(np.abs(g - ref)) < TOL


def test_adjoint_vs_oracle_with_pow_exponents():
    """Integer pow_exponent scales the generator angle: d/dtheta carries the factor p."""
    n = 5
    rng = np.random.default_rng(9)
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    ops += [bs.Instruction(bs.Rx(0.4, pow_exponent=2.0), [0]), bs.Instruction(bs.ZZ(-0.3, pow_exponent=3.0), [1, 4]),
            bs.Instruction(bs.PhaseShift(0.9, pow_exponent=-1.0), [2]), bs.Instruction(bs.CNot(), [2, 3]),
            bs.Instruction(bs.YY(1.3), [3, 0]), bs.Instruction(bs.Ry(-2.0, pow_exponent=2.0), [4])]
    h = hamiltonian(n, 8, rng)
    e, g = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0), ops, h)
    e_ref, gref = oracle.parameter_shift_gradient(n, ops, h)
    ref = np.array([gref[i] for i in adj.parameterised(ops)])
    assert abs(e - e_ref) < 1e-12
    assert np.max(np.abs(g - ref)) < TOL


def test_adjoint_24q_720_params_vs_oracle_subset():
    """The 24-qubit, 720-parameter, 48-term configuration: the full adjoint gradient on the GPU,
    24 of its entries (spread over the whole circuit, first and last included) against the
    oracle's FP64 parameter shift; the complex64 variant's error against the same entries."""
    n = 24
    ops, h = bench.adjoint_workload(bs, n=n, layers=10, terms=48, seed=3)
    pidx = adj.parameterised(ops)
    assert len(pidx) == 720 and len(h) == 48
    e, g = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0), ops, h)
    pick = np.unique(np.linspace(0, len(pidx) - 1, 24).round().astype(int))
    e_ref, gref = oracle.parameter_shift_gradient(n, ops, h, which=[pidx[k] for k in pick])
    ref = np.array([gref[pidx[k]] for k in pick])
    assert abs(e - e_ref) < 1e-10
    assert np.max(np.abs(g[pick] - ref)) < TOL
    e64, g64 = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0, precision="c64"), ops, h)
    scale = sum(abs(c) for c, _ in h)
    assert abs(e64 - e_ref) < 2e-5 * scale
    assert np.max(np.abs(g64[pick] - ref)) < 2e-5 * scale
