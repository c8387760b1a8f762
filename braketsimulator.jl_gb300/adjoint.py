"""Expectation gradients of parameterised circuits.

``adjoint_gradient`` runs the engine's adjoint method (one forward pass, one
fused reverse sweep over psi and lambda = H psi).  ``parameter_shift_gradient``
is the reference workaround for the same quantity: the reference has no
gradient result (``AdjointGradient`` is declared in src/results.jl:90-159 and
rejected in src/pragmas.jl:67-68), so users evaluate 2P shifted circuits.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Sequence

import numpy as np

from . import _abi
from .gates import PhaseShift, Rx, Ry, Rz, XX, YY, ZZ
from .simulators import Instruction, StateVectorSimulator, _ops_for

_GENERATORS = {Rx: ("X",), Ry: ("Y",), Rz: ("Z",), XX: ("X", "X"), YY: ("Y", "Y"), ZZ: ("Z", "Z")}


def pauli_masks(term: dict) -> tuple:
    """{qubit: 'X'|'Y'|'Z'} -> (xmask, zmask) with bit q <-> qubit q."""
    x = z = 0
    for q, p in term.items():
        p = p.upper()
        if p in ("X", "Y"):
            x |= 1 << int(q)
        if p in ("Z", "Y"):
            z |= 1 << int(q)
    return x, z


def _generator(ix: Instruction):
    g = ix.operator
    if isinstance(g, PhaseShift):
        return 1, 0, 0
    for cls, paulis in _GENERATORS.items():
        if type(g) is cls:
            return 0, *pauli_masks(dict(zip(ix.target, paulis)))
    return None


def parameterised(instructions) -> list:
    """Indices of instructions whose angle is differentiable here."""
    return [i for i, ix in enumerate(instructions) if _generator(ix) is not None]


def adjoint_gradient(sim: StateVectorSimulator, instructions: Sequence[Instruction], hamiltonian,
                     param_index: Sequence[int] | None = None):
    """<H> and d<H>/dtheta for a circuit applied to |0...0>.

    hamiltonian: list of (coefficient, {qubit: 'X'|'Y'|'Z'}) terms.
    param_index[i] = parameter slot of instruction i (-1: not a parameter); by default every
    differentiable gate gets its own slot in order.  Returns (energy, gradient array)."""
    instructions = list(instructions)
    if param_index is None:
        param_index, p = [], 0
        for ix in instructions:
            if _generator(ix) is not None:
                param_index.append(p)
                p += 1
            else:
                param_index.append(-1)
    n_params = max([-1] + list(param_index)) + 1
    arr, n_ops, keep = _ops_for(instructions, False, 0)
    if n_ops != len(instructions):
        raise ValueError("adjoint_gradient expects one engine op per instruction (no no-ops, no split gates)")
    pi = np.array(param_index, dtype=np.int32)
    gk = np.zeros(n_ops, dtype=np.int32)
    gx = np.zeros(n_ops, dtype=np.uint64)
    gz = np.zeros(n_ops, dtype=np.uint64)
    scale = np.ones(n_params)
    for i, ix in enumerate(instructions):
        if pi[i] < 0:
            continue
        gen = _generator(ix)
        if gen is None:
            raise ValueError(f"{ix.operator!r} has no supported generator")
        gk[i], gx[i], gz[i] = gen
        scale[pi[i]] = ix.operator.pow_exponent
    xm = np.array([pauli_masks(t)[0] for _, t in hamiltonian], dtype=np.uint64)
    zm = np.array([pauli_masks(t)[1] for _, t in hamiltonian], dtype=np.uint64)
    co = np.array([c for c, _ in hamiltonian], dtype=np.float64)
    energy = C.c_double()
    grad = np.zeros(max(1, n_params), dtype=np.float64)
    sim.reinit(sim.qubit_count, sim.shots)
    sim._h.call("bs_adjoint_gradient", arr, n_ops, _abi.iptr(pi), _abi.iptr(gk), _abi.u64ptr(gx), _abi.u64ptr(gz),
                n_params, len(co), _abi.u64ptr(xm), _abi.u64ptr(zm), _abi.dptr(co), C.byref(energy), _abi.dptr(grad))
    del keep
    return energy.value, grad[:n_params] * scale


def energy(sim: StateVectorSimulator, instructions, hamiltonian) -> float:
    """<H> after the circuit, from |0...0>."""
    sim.reinit(sim.qubit_count, sim.shots)
    sim.evolve(instructions)
    xm = np.array([pauli_masks(t)[0] for _, t in hamiltonian], dtype=np.uint64)
    zm = np.array([pauli_masks(t)[1] for _, t in hamiltonian], dtype=np.uint64)
    co = np.array([c for c, _ in hamiltonian], dtype=np.float64)
    out = np.empty(len(co), dtype=np.float64)
    sim._h.call("bs_expectation_pauli", len(co), _abi.u64ptr(xm), _abi.u64ptr(zm), _abi.dptr(co), _abi.dptr(out))
    return float(np.sum(out))


def _with_angle(ix: Instruction, delta: float) -> Instruction:
    g = ix.operator
    return Instruction(type(g)(g.angle[0] + delta / g.pow_exponent, pow_exponent=g.pow_exponent), list(ix.target))


def parameter_shift_gradient(sim: StateVectorSimulator, instructions, hamiltonian, param_index=None,
                             shift: float = math.pi / 2):
    """Two-term parameter-shift rule, exact for generators with eigenvalues +-1 (and the
    PhaseShift projector): dE/dtheta = [E(theta + s) - E(theta - s)] / (2 sin s)."""
    instructions = list(instructions)
    pidx = parameterised(instructions) if param_index is None else [i for i, p in enumerate(param_index) if p >= 0]
    slots = list(range(len(pidx))) if param_index is None else [param_index[i] for i in pidx]
    grad = np.zeros(max(slots) + 1 if slots else 0)
    for slot, i in zip(slots, pidx):
        ix = instructions[i]
        plus = instructions[:i] + [_with_angle(ix, shift)] + instructions[i + 1:]
        minus = instructions[:i] + [_with_angle(ix, -shift)] + instructions[i + 1:]
        d = (energy(sim, plus, hamiltonian) - energy(sim, minus, hamiltonian)) / (2.0 * math.sin(shift))
        grad[slot] += d * ix.operator.pow_exponent
    return grad


def finite_difference_gradient(sim, instructions, hamiltonian, h: float = 1e-6):
    instructions = list(instructions)
    pidx = parameterised(instructions)
    grad = np.zeros(len(pidx))
    for slot, i in enumerate(pidx):
        ix = instructions[i]
        g = ix.operator
        up = Instruction(type(g)(g.angle[0] + h, pow_exponent=g.pow_exponent), list(ix.target))
        dn = Instruction(type(g)(g.angle[0] - h, pow_exponent=g.pow_exponent), list(ix.target))
        e1 = energy(sim, instructions[:i] + [up] + instructions[i + 1:], hamiltonian)
        e0 = energy(sim, instructions[:i] + [dn] + instructions[i + 1:], hamiltonian)
        grad[slot] = (e1 - e0) / (2 * h)
    return grad


def energy_rrule(sim: StateVectorSimulator, instructions: Sequence[Instruction], hamiltonian,
                 param_index: Sequence[int] | None = None):
    """Reverse-mode rule for <H>(theta) in the form of a ChainRulesCore ``rrule``: returns
    ``(energy, pullback)`` where ``pullback(de)`` gives the cotangent of every parameter slot,
    ``de * d<H>/dtheta``.  One adjoint evaluation serves both."""
    e, g = adjoint_gradient(sim, instructions, hamiltonian, param_index)

    def pullback(de):
        return float(de) * g

    return e, pullback


def torch_energy(build, hamiltonian, sim: StateVectorSimulator):
    """A torch.autograd function theta -> <H>(theta): ``build(theta: np.ndarray)`` returns the
    instruction list whose differentiable gates take theta in order of appearance.  Forward runs
    the adjoint method once; backward returns grad_output * gradient (device-independent: theta may
    live anywhere, the engine is called with host values)."""
    import torch

    class _Energy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            e, g = adjoint_gradient(sim, build(theta.detach().double().cpu().numpy()), hamiltonian)
            ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
            return theta.new_tensor(e)

        @staticmethod
        def backward(ctx, grad_output):
            (g,) = ctx.saved_tensors
            return grad_output * g

    return _Energy.apply
