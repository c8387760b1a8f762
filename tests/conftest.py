"""Shared fixtures: package loading, gate factories, GPU marker."""
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    name = "braketsimulator_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "braketsimulator.jl_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


bs = load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


def pytest_collection_modifyitems(config, items):
    # run GPU tests only where a GPU is visible
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


GATES_1 = {"h": bs.H, "x": bs.X, "y": bs.Y, "z": bs.Z, "s": bs.S, "si": bs.Si, "t": bs.T, "ti": bs.Ti, "v": bs.V,
           "vi": bs.Vi, "i": bs.I, "cnot": bs.CNot, "cy": bs.CY, "cz": bs.CZ, "cv": bs.CV, "swap": bs.Swap,
           "iswap": bs.ISwap, "ecr": bs.ECR, "ccnot": bs.CCNot, "cswap": bs.CSwap}
GATES_A = {"rx": bs.Rx, "ry": bs.Ry, "rz": bs.Rz, "phaseshift": bs.PhaseShift, "cphaseshift": bs.CPhaseShift,
           "cphaseshift00": bs.CPhaseShift00, "cphaseshift01": bs.CPhaseShift01, "cphaseshift10": bs.CPhaseShift10,
           "xx": bs.XX, "yy": bs.YY, "xy": bs.XY, "zz": bs.ZZ, "gpi": bs.GPi, "gpi2": bs.GPi2, "ms": bs.MS, "u": bs.U,
           "prx": bs.PRx, "pswap": bs.PSwap, "single_excitation": bs.SingleExcitation,
           "single_excitation_plus": bs.SingleExcitationPlus, "single_excitation_minus": bs.SingleExcitationMinus,
           "fermionic_swap": bs.FermionicSWAP, "double_excitation": bs.DoubleExcitation,
           "double_excitation_plus": bs.DoubleExcitationPlus, "double_excitation_minus": bs.DoubleExcitationMinus,
           "multi_rz": bs.MultiRZ}
NOISES = {"bit_flip": bs.BitFlip, "phase_flip": bs.PhaseFlip, "depolarizing": bs.Depolarizing,
          "amplitude_damping": bs.AmplitudeDamping, "generalized_amplitude_damping": bs.GeneralizedAmplitudeDamping,
          "pauli_channel": bs.PauliChannel, "phase_damping": bs.PhaseDamping,
          "two_qubit_depolarizing": bs.TwoQubitDepolarizing, "two_qubit_dephasing": bs.TwoQubitDephasing}


def make_op(spec, pw=1.0):
    """(name, angles, targets[, extra]) -> product Instruction."""
    name, ang, targets = spec[0], spec[1], spec[2]
    if name in GATES_1:
        op = GATES_1[name](pow_exponent=pw)
    elif name in GATES_A:
        op = GATES_A[name](*ang, pow_exponent=pw)
    elif name == "unitary":
        op = bs.Unitary(spec[3], pw)
    elif name == "gphase":
        op = bs.GPhase(len(targets), ang[0], pw)
    elif name == "kraus":
        op = bs.Kraus(ang)
    elif name in NOISES:
        op = NOISES[name](*ang)
    else:
        raise KeyError(name)
    return bs.Instruction(op, list(targets))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(a), np.linalg.norm(b), 1e-300))


def random_circuit(n, depth, rng, kinds=None, pows=False):
    """Random instructions over every gate family (product types)."""
    names1 = ["h", "x", "y", "z", "s", "si", "t", "ti", "v", "vi"]
    namesa1 = ["rx", "ry", "rz", "phaseshift", "gpi", "gpi2", "u", "prx"]
    names2 = ["cnot", "cy", "cz", "cv", "swap", "iswap", "ecr"]
    namesa2 = ["cphaseshift", "cphaseshift00", "cphaseshift01", "cphaseshift10", "xx", "yy", "xy", "zz", "ms",
               "pswap", "single_excitation", "single_excitation_plus", "single_excitation_minus", "fermionic_swap"]
    names3 = ["ccnot", "cswap"]
    out = []
    for _ in range(depth):
        r = rng.random()
        pw = float(rng.choice([1.0, 1.0, 1.0, 2.0, 0.5, -1.0, 2.5, -0.5, 3.0])) if pows else 1.0
        if r < 0.25 or n < 2:
            nm = names1[rng.integers(len(names1))]
            op = GATES_1[nm](pow_exponent=pw)
            t = [int(rng.integers(n))]
        elif r < 0.5:
            nm = namesa1[rng.integers(len(namesa1))]
            na = GATES_A[nm].n_angles
            op = GATES_A[nm](*rng.uniform(-np.pi, np.pi, na), pow_exponent=pw)
            t = [int(rng.integers(n))]
        elif r < 0.65:
            nm = names2[rng.integers(len(names2))]
            op = GATES_1[nm](pow_exponent=pw)
            t = [int(x) for x in rng.choice(n, 2, replace=False)]
        elif r < 0.85:
            nm = namesa2[rng.integers(len(namesa2))]
            na = GATES_A[nm].n_angles
            op = GATES_A[nm](*rng.uniform(-np.pi, np.pi, na), pow_exponent=pw)
            t = [int(x) for x in rng.choice(n, 2, replace=False)]
        elif r < 0.9 and n >= 3:
            nm = names3[rng.integers(len(names3))]
            op = GATES_1[nm](pow_exponent=pw)
            t = [int(x) for x in rng.choice(n, 3, replace=False)]
        elif r < 0.95 and n >= 4:
            nm = ["double_excitation", "double_excitation_plus", "double_excitation_minus"][rng.integers(3)]
            op = GATES_A[nm](float(rng.uniform(-np.pi, np.pi)), pow_exponent=pw)
            t = [int(x) for x in rng.choice(n, 4, replace=False)]
        else:
            k = int(rng.integers(1, min(n, 3) + 1))
            a = rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k))
            q, _ = np.linalg.qr(a)
            op = bs.Unitary(q)
            t = [int(x) for x in rng.choice(n, k, replace=False)]
        out.append(bs.Instruction(op, t))
    return out
