"""Adjoint gradients vs the parameter-shift rule (exact for these generators) and
central finite differences."""
import numpy as np
import pytest

from conftest import bs

pytestmark = pytest.mark.gpu
from importlib import import_module  # noqa: E402

adj = import_module("braketsimulator_gb300.adjoint")


def ansatz(n, layers, rng):
    ops = []
    for _ in range(layers):
        for q in range(n):
            ops.append(bs.Instruction(bs.Ry(float(rng.uniform(-np.pi, np.pi))), [q]))
            ops.append(bs.Instruction(bs.Rz(float(rng.uniform(-np.pi, np.pi))), [q]))
        for q in range(n):
            ops.append(bs.Instruction(bs.ZZ(float(rng.uniform(-np.pi, np.pi))), [q, (q + 1) % n]))
    return ops


def hamiltonian(n, terms, rng):
    h = []
    for _ in range(terms):
        w = int(rng.integers(1, min(4, n) + 1))
        qs = rng.choice(n, w, replace=False)
        h.append((float(rng.normal()), {int(q): "XYZ"[rng.integers(3)] for q in qs}))
    return h


@pytest.mark.parametrize("n,layers", [(2, 1), (4, 2), (7, 2), (12, 2)])
def test_adjoint_matches_parameter_shift(n, layers):
    rng = np.random.default_rng(n)
    ops = ansatz(n, layers, rng)
    h = hamiltonian(n, 8, rng)
    sim = bs.StateVectorSimulator(n, 0)
    e, g = adj.adjoint_gradient(sim, ops, h)
    e_ref = adj.energy(sim, ops, h)
    ps = adj.parameter_shift_gradient(sim, ops, h)
    assert abs(e - e_ref) < 1e-12
    assert np.max(np.abs(g - ps)) < 1e-10


def test_adjoint_other_generators_and_shared_parameters():
    rng = np.random.default_rng(4)
    n = 5
    ops = [bs.Instruction(bs.H(), [q]) for q in range(n)]
    ops += [bs.Instruction(bs.Rx(0.3), [0]), bs.Instruction(bs.XX(0.7), [1, 3]), bs.Instruction(bs.YY(-0.4), [2, 4]),
            bs.Instruction(bs.PhaseShift(1.1), [2]), bs.Instruction(bs.CNot(), [0, 4]), bs.Instruction(bs.Rx(0.3), [3])]
    h = hamiltonian(n, 6, rng)
    sim = bs.StateVectorSimulator(n, 0)
    e, g = adj.adjoint_gradient(sim, ops, h)
    ps = adj.parameter_shift_gradient(sim, ops, h)
    fd = adj.finite_difference_gradient(sim, ops, h)
    assert np.max(np.abs(g - ps)) < 1e-10
    assert np.max(np.abs(g - fd)) < 1e-6
    # shared parameter: both Rx gates use slot 0
    pidx = [-1] * n + [0, 1, 2, 3, -1, 0]
    e2, g2 = adj.adjoint_gradient(sim, ops, h, pidx)
    assert abs(g2[0] - (g[0] + g[4])) < 1e-12


@pytest.mark.parametrize("n", [6, 13])
def test_adjoint_complex64_state(n):
    """complex64 state, float-float arithmetic and FP64-grade inner products: the gradient differs
    from the complex128 one by the complex64 rounding of the stored states only."""
    rng = np.random.default_rng(60 + n)
    ops = ansatz(n, 3, rng)
    h = hamiltonian(n, 10, rng)
    e128, g128 = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0), ops, h)
    e64, g64 = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0, precision="c64"), ops, h)
    scale = max(1.0, sum(abs(c) for c, _ in h))
    assert abs(e64 - e128) < 2e-5 * scale
    assert np.max(np.abs(g64 - g128)) < 2e-5 * scale


@pytest.mark.parametrize("segments", [1, 2, 5, 40])
def test_adjoint_checkpoint_segments(segments):
    """Forward checkpoints (psi kept after each segment, restored on the way back) give the same
    gradients as pure uncomputation, for any segment count (including more segments than gates
    per segment allow)."""
    n = 9
    rng = np.random.default_rng(77)
    ops = ansatz(n, 3, rng)
    h = hamiltonian(n, 8, rng)
    ref = bs.StateVectorSimulator(n, 0)
    bs.set_tuning(ref, adj_segments=1)
    e1, g1 = adj.adjoint_gradient(ref, ops, h)
    sim = bs.StateVectorSimulator(n, 0)
    bs.set_tuning(sim, adj_segments=segments)
    e, g = adj.adjoint_gradient(sim, ops, h)
    assert abs(e - e1) < 1e-12
    assert np.max(np.abs(g - g1)) < 1e-12
    ps = adj.parameter_shift_gradient(sim, ops, h)
    assert np.max(np.abs(g - ps)) < 1e-10


def test_adjoint_checkpoints_bound_complex64_drift():
    """complex64: uncomputing psi through a deep circuit drifts; checkpoints reset it per segment."""
    n = 10
    rng = np.random.default_rng(90)
    ops = ansatz(n, 12, rng)
    h = hamiltonian(n, 10, rng)
    _, g128 = adj.adjoint_gradient(bs.StateVectorSimulator(n, 0), ops, h)
    errs = {}
    for seg in (1, 16):
        sim = bs.StateVectorSimulator(n, 0, precision="c64")
        bs.set_tuning(sim, adj_segments=seg)
        _, g64 = adj.adjoint_gradient(sim, ops, h)
        errs[seg] = float(np.max(np.abs(g64 - g128)))
    scale = max(1.0, sum(abs(c) for c, _ in h))
    assert errs[16] < 2e-5 * scale
    assert errs[16] <= errs[1] * 1.5


def test_rrule_and_torch_autograd():
    import torch
    n = 6
    rng = np.random.default_rng(12)
    h = hamiltonian(n, 6, rng)
    theta0 = rng.uniform(-np.pi, np.pi, size=3 * n)

    def build(th):
        ops = []
        for q in range(n):
            ops.append(bs.Instruction(bs.Ry(float(th[q])), [q]))
            ops.append(bs.Instruction(bs.Rz(float(th[n + q])), [q]))
        for q in range(n):
            ops.append(bs.Instruction(bs.ZZ(float(th[2 * n + q])), [q, (q + 1) % n]))
        return ops

    sim = bs.StateVectorSimulator(n, 0)
    e, pb = bs.energy_rrule(sim, build(theta0), h)
    ps = adj.parameter_shift_gradient(sim, build(theta0), h)
    assert np.max(np.abs(pb(2.0) - 2.0 * ps)) < 1e-10
    f = bs.torch_energy(build, h, sim)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    out = 3.0 * f(theta)
    out.backward()
    assert abs(out.item() - 3.0 * e) < 1e-12
    assert np.max(np.abs(theta.grad.numpy() - 3.0 * ps)) < 1e-10
