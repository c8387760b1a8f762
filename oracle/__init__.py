"""ORACLE — test infrastructure only, never part of the product path.

CPU FP64 restatement of the reference BraketSimulator.jl hot path, used by
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as the
checker.  ``ref_kernels.c`` restates the data-parallel kernels with their exact
index conventions; this module restates the host-side dispatch that picks a
kernel and the gate matrix tables (``matrix_rep``), written independently of the
product package.

Parity pinning: the reference is Julia and cannot run here (no julia binary, no
Quasar/StaticArrays/StatsBase).  The oracle is pinned against the golden vectors
of the reference's own tests (test/test_sv_simulator.jl, test/test_dm_simulator.jl,
test/test_custom_gates.jl, test/test_result_types.jl, test/test_gate_operations.jl),
transcribed in tests/golden/reference_kats.py.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_kernels.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp", src, "-lm"], check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I, I64, D = C.c_void_p, C.c_int, C.c_int64, C.c_double
        sig = {
            "orc_apply_1q": [P, I64, P, I],
            "orc_apply_2q": [P, I64, P, I, I],
            "orc_apply_c1t1": [P, I64, P, I, I, I],
            "orc_apply_c1t2": [P, I64, P, I, I, I, I],
            "orc_apply_c2t1": [P, I64, P, I, I, I, I, I],
            "orc_apply_nq": [P, I64, P, I, P],
            "orc_apply_double_excitation": [P, I64, D, P],
            "orc_dm_phase_flip": [P, I64, D, I],
            "orc_dm_kraus_1q": [P, I64, P, I, I],
            "orc_dm_kraus_2q": [P, I64, P, I, I, I],
            "orc_dm_kraus_nq": [P, I64, P, I, I, P],
            "orc_dm_kraus_full": [P, I64, P, I, I, P],
            "orc_make_alias_table": [P, I64, D, P, P, P, P],
            "orc_sample_alias": [P, P, P, P, I64, P],
            "orc_sample_direct": [P, I64, D, P, I64, P],
        }
        for name, args in sig.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None
        L.orc_pairwise_sum.argtypes = [P, I64]
        L.orc_pairwise_sum.restype = D
        L.orc_expect_pauli.argtypes = [P, I64, C.c_uint64, C.c_uint64, I]
        L.orc_expect_pauli.restype = D
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _cm(m):
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128))


# ============================================================================ matrices
# Restatement of matrix_rep / matrix_rep_raw (src/gate_kernels.jl:225-478,
# src/custom_gates.jl:41-360), keyed by the gate's reference name.
SQ2 = 1.0 / math.sqrt(2.0)


def _rot(kind, t):
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    return {
        "rx": [[c, -1j * s], [-1j * s, c]],
        "ry": [[c, -s], [s, c]],
        "rz": [[c - 1j * s, 0], [0, c + 1j * s]],
        "phaseshift": [[1, 0], [0, np.exp(1j * t)]],
        "xx": [[c, 0, 0, -1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [-1j * s, 0, 0, c]],
        "yy": [[c, 0, 0, 1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [1j * s, 0, 0, c]],
        "xy": [[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, 1]],
        "single_excitation": [[1, 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, 1]],
        "single_excitation_plus": [[np.exp(1j * t / 2), 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, np.exp(1j * t / 2)]],
        "single_excitation_minus": [[np.exp(-1j * t / 2), 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, np.exp(-1j * t / 2)]],
        "fermionic_swap": [[1, 0, 0, 0], [0, np.exp(1j * t / 2) * c, -1j * np.exp(1j * t / 2) * s, 0],
                           [0, -1j * np.exp(1j * t / 2) * s, np.exp(1j * t / 2) * c, 0], [0, 0, 0, np.exp(1j * t)]],
        "zz": np.diag([np.exp(-1j * t / 2), np.exp(1j * t / 2), np.exp(1j * t / 2), np.exp(-1j * t / 2)]),
        "cphaseshift": np.diag([1, 1, 1, np.exp(1j * t)]),
        "cphaseshift00": np.diag([np.exp(1j * t), 1, 1, 1]),
        "cphaseshift01": np.diag([1, 1, np.exp(1j * t), 1]),
        "cphaseshift10": np.diag([1, np.exp(1j * t), 1, 1]),
    }[kind]


def _dexc(t, phase):
    s, c = math.sin(t / 2.0), math.cos(t / 2.0)
    d = {0: 1.0, 1: np.exp(1j * t / 2), -1: np.exp(-1j * t / 2)}[phase]
    m = np.eye(16, dtype=np.complex128) * d
    m[3, 3], m[12, 12], m[3, 12], m[12, 3] = c, c, -s, s
    return m


FIXED = {
    "i": [[1, 0], [0, 1]], "h": [[SQ2, SQ2], [SQ2, -SQ2]], "x": [[0, 1], [1, 0]], "y": [[0, -1j], [1j, 0]],
    "z": [[1, 0], [0, -1]], "v": [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]],
    "vi": [[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]], "s": [[1, 0], [0, 1j]], "si": [[1, 0], [0, -1j]],
    "t": [[1, 0], [0, np.exp(1j * math.pi / 4)]], "ti": [[1, 0], [0, np.exp(-1j * math.pi / 4)]],
    "cnot": [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]],
    "cy": [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]],
    "cz": np.diag([1, 1, 1, -1]), "swap": [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],
    "iswap": [[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]],
    "cv": [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0.5 + 0.5j, 0.5 - 0.5j], [0, 0, 0.5 - 0.5j, 0.5 + 0.5j]],
    "ecr": (SQ2 * np.array([[0, 1, 0, 1j], [1, 0, -1j, 0], [0, 1j, 0, 1], [-1j, 0, 1, 0]])),
}
FIXED["ccnot"] = np.eye(8)[[0, 1, 2, 3, 4, 5, 7, 6]]
FIXED["cswap"] = np.eye(8)[[0, 1, 2, 3, 4, 6, 5, 7]]


def _angled_raw(name, a):
    if name in ("gpi",):
        return [[0, np.exp(-1j * a[0])], [np.exp(1j * a[0]), 0]]
    if name == "gpi2":
        return SQ2 * np.array([[1, -1j * np.exp(-1j * a[0])], [-1j * np.exp(1j * a[0]), 1]])
    if name == "prx":
        c, s = math.cos(a[0] / 2), math.sin(a[0] / 2)
        return [[c, -1j * np.exp(-1j * a[1]) * s], [-1j * np.exp(1j * a[1]) * s, c]]
    if name == "ms":
        c, s = math.cos(a[2] / 2), math.sin(a[2] / 2)
        return [[c, 0, 0, -1j * np.exp(-1j * (a[0] + a[1])) * s], [0, c, -1j * np.exp(-1j * (a[0] - a[1])) * s, 0],
                [0, -1j * np.exp(1j * (a[0] - a[1])) * s, c, 0], [-1j * np.exp(1j * (a[0] + a[1])) * s, 0, 0, c]]
    if name == "u":
        c, s = math.cos(a[0] / 2), math.sin(a[0] / 2)
        return [[c, -np.exp(1j * a[2]) * s], [np.exp(1j * a[1]) * s, np.exp(1j * (a[2] + a[1])) * c]]
    if name == "pswap":
        e = np.exp(1j * a[0])
        return [[1, 0, 0, 0], [0, 0, e, 0], [0, e, 0, 0], [0, 0, 0, 1]]
    if name in ("double_excitation", "double_excitation_plus", "double_excitation_minus"):
        return _dexc(a[0], {"double_excitation": 0, "double_excitation_plus": 1, "double_excitation_minus": -1}[name])
    return _rot(name, a[0])


def _power(m, p):
    m = np.asarray(m, dtype=np.complex128)
    if float(p).is_integer():
        return np.linalg.matrix_power(m if p >= 0 else np.linalg.inv(m), int(abs(p)))
    if np.array_equal(m, m.conj().T):
        w, v = np.linalg.eigh(m)
        return (v * np.power(w.astype(np.complex128), p)) @ v.conj().T
    w, v = np.linalg.eig(m)
    return (v * np.power(w, p)) @ np.linalg.inv(v)


def matrix_rep(name: str, angles=(), pw: float = 1.0, unitary=None):
    """matrix_rep of a gate given by reference name, angles and pow_exponent."""
    n = float(pw)
    integer = n.is_integer()
    if name == "unitary":
        raw = np.asarray(unitary, dtype=np.complex128)
        if n == 1:
            return raw
        if n == 0.5:
            return _power(raw, 0.5)
        if n == -0.5:
            return np.linalg.inv(_power(raw, 0.5))
        return _power(raw, n)
    if name in ("y", "h", "swap", "cnot", "cy", "cz", "ccnot", "cswap", "gpi", "ecr"):
        raw = np.asarray(FIXED[name] if name != "gpi" else _angled_raw(name, angles), dtype=np.complex128)
        if integer:
            return np.eye(raw.shape[0], dtype=np.complex128) if int(n) % 2 == 0 else raw
        return _power(raw, n)
    if name in ("x", "z"):
        raw = np.asarray(FIXED[name], dtype=np.complex128)
        if integer:
            return np.eye(2, dtype=np.complex128) if int(n) % 2 == 0 else raw
        if n == 0.5:
            return np.asarray(FIXED["v" if name == "x" else "s"], dtype=np.complex128)
        return _power(raw, n)
    if name in ("v", "vi", "s", "si"):
        fwd, sq, back = {"v": ("v", "x", "vi"), "vi": ("vi", "x", "v"), "s": ("s", "z", "si"), "si": ("si", "z", "s")}[name]
        if integer:
            return np.asarray([FIXED["i"], FIXED[fwd], FIXED[sq], FIXED[back]][int(n) % 4], dtype=np.complex128)
        return _power(FIXED[name], n)
    if name in ("t", "ti"):
        if n == 0:
            return np.eye(2, dtype=np.complex128)
        if n == 1:
            return np.asarray(FIXED[name], dtype=np.complex128)
        if n == -1:
            return np.asarray(FIXED["ti" if name == "t" else "t"], dtype=np.complex128)
        return matrix_rep("phaseshift", ((1 if name == "t" else -1) * n * math.pi / 4,), 1.0)
    if name == "i":
        return np.eye(2, dtype=np.complex128)
    if name in ("iswap", "cv"):
        raw = np.asarray(FIXED[name], dtype=np.complex128)
        if n == 0:
            return np.eye(4, dtype=np.complex128)
        if n == 1:
            return raw
        if n == -1:
            return raw.conj().T
        return _power(raw, n)
    a = tuple(angles)
    if name in ("rx", "ry", "rz", "phaseshift", "xx", "yy", "xy", "single_excitation", "single_excitation_plus",
                "single_excitation_minus", "fermionic_swap"):
        k = 2 if name in ("rx", "ry", "rz", "phaseshift") else 4
        if n == 0:
            return np.eye(k, dtype=np.complex128)
        if integer:
            return np.asarray(_rot(name, a[0] * n), dtype=np.complex128)
        return _power(_rot(name, a[0]), n)
    if name in ("cphaseshift", "cphaseshift00", "cphaseshift01", "cphaseshift10", "zz"):
        return np.eye(4, dtype=np.complex128) if n == 0 else np.asarray(_rot(name, a[0] * n), dtype=np.complex128)
    if name in ("double_excitation", "double_excitation_plus", "double_excitation_minus"):
        return np.eye(16, dtype=np.complex128) if n == 0 else _angled_raw(name, (a[0] * n,))
    if name == "pswap":
        if n == 0:
            return np.eye(4, dtype=np.complex128)
        if n == 1:
            return np.asarray(_angled_raw(name, a), dtype=np.complex128)
        if integer and int(n) % 2 == 1:
            return np.asarray(_angled_raw(name, (a[0] * n,)), dtype=np.complex128)
        if integer:
            e = np.exp(1j * a[0] * n)
            return np.diag([1, e, e, 1]).astype(np.complex128)
        return _power(_angled_raw(name, a), n)
    if name in ("prx", "ms", "u"):
        raw = np.asarray(_angled_raw(name, a), dtype=np.complex128)
        if n == 0:
            return np.eye(raw.shape[0], dtype=np.complex128)
        if n == 1:
            return raw
        if n == -1:
            if name == "prx":
                inv = (-a[0], a[1])
            elif name == "ms":
                inv = (a[0] + math.pi, a[1], a[2])
            else:
                inv = (-a[0], -a[2], -a[1])
            return np.asarray(_angled_raw(name, inv), dtype=np.complex128)
        return _power(raw, n)
    if name in ("gpi2",):
        raw = np.asarray(_angled_raw(name, a), dtype=np.complex128)
        if n == 1:
            return raw
        if n == 0.5:
            return _power(raw, 0.5)
        if n == -0.5:
            return np.linalg.inv(_power(raw, 0.5))
        return _power(raw, n)
    raise KeyError(name)


# ============================================================================ dispatch
def _gate_desc(g):
    """(name, angles, pow, extra) read from a gate object by attribute only."""
    name = getattr(g, "name", type(g).__name__.lower())
    return name, tuple(getattr(g, "angle", ())), float(getattr(g, "pow_exponent", 1.0))


def _kernel(psi, mat, targets, conj):
    L = lib()
    m = _cm(np.conj(mat) if conj else mat)
    n = psi.size
    k = len(targets)
    if k == 1:
        L.orc_apply_1q(_p(psi), n, _p(m), targets[0])
    elif k == 2:
        L.orc_apply_2q(_p(psi), n, _p(m), targets[0], targets[1])
    else:
        t = np.array(targets, dtype=np.int32)
        L.orc_apply_nq(_p(psi), n, _p(m), k, _p(t))


def _diag_kernel(psi, d, targets, conj):
    _kernel(psi, np.diag(d), targets, conj)


_CTRL = {"cnot": ("x", 1), "cy": ("y", 1), "cz": ("z", 1), "cv": ("v", 1), "cswap": ("swap", 1), "ccnot": ("x", 2)}


def _controlled(psi, tmat, bits, qubits, conj):
    L = lib()
    m = _cm(np.conj(tmat) if conj else tmat)
    nb = len(bits)
    nt = len(qubits) - nb
    if nb == 1 and nt == 1:
        L.orc_apply_c1t1(_p(psi), psi.size, _p(m), int(bits[0] == 1), qubits[0], qubits[1])
    elif nb == 1 and nt == 2:
        L.orc_apply_c1t2(_p(psi), psi.size, _p(m), int(bits[0] == 1), qubits[0], qubits[1], qubits[2])
    elif nb == 2 and nt == 1:
        L.orc_apply_c2t1(_p(psi), psi.size, _p(m), int(bits[0] == 1), int(bits[1] == 1), qubits[0], qubits[1], qubits[2])
    else:
        raise NotImplementedError("the reference has no kernel for this control/target combination")


def pauli_eigenvalues(n):
    return np.array([(-1.0) ** bin(i).count("1") for i in range(2 ** n)])


def apply_gate(g, psi: np.ndarray, targets, conj: bool = False):
    """apply_gate!(Val(conj), g, psi, targets...) (src/gate_kernels.jl:675-775,
    src/custom_gates.jl:381-416) on a complex128 numpy vector, in place."""
    name, ang, pw = _gate_desc(g)
    t = [int(x) for x in targets]
    if name in ("i",):
        return
    if name == "control":
        inner = g.g
        iname, iang, ipw = _gate_desc(inner)
        if iname == "gphase":
            f = -1j if conj else 1j
            d = np.ones(2 ** inner.n, dtype=np.complex128)
            d[sum(b << i for i, b in enumerate(g.bitvals))] = np.exp(f * iang[0] * ipw * pw)
            _diag_kernel(psi, d, t, False)
            return
        tm = matrix_rep(iname, iang, ipw * pw, getattr(inner, "matrix", None))
        _controlled(psi, tm, g.bitvals, t, conj)
        return
    if name in _CTRL:
        tn, nb = _CTRL[name]
        _controlled(psi, matrix_rep(tn, (), pw), (1,) * nb, t, conj)
        return
    if name == "gphase":
        e = np.exp(1j * ang[0] * pw)
        _diag_kernel(psi, np.full(2 ** len(t), np.conj(e) if conj else e), t, False)
        return
    if name == "multi_rz":
        if len(t) == 1:
            apply_gate(_Fake("rz", ang, pw), psi, t, conj)
        elif len(t) == 2:
            apply_gate(_Fake("zz", ang, pw), psi, t, conj)
        else:
            f = -1j * ang[0] / 2.0
            _diag_kernel(psi, np.exp((np.conj(f) if conj else f) * pauli_eigenvalues(len(t))), t, False)
        return
    if name == "double_excitation":
        tt = np.array(t, dtype=np.int32)
        lib().orc_apply_double_excitation(_p(psi), psi.size, ang[0] * pw / 2.0, _p(tt))
        return
    m = matrix_rep(name, ang, pw, getattr(g, "matrix", None))
    _kernel(psi, m, t, conj)


class _Fake:
    def __init__(self, name, angle, pw):
        self.name, self.angle, self.pow_exponent = name, angle, pw


# ---------------------------------------------------------------------------- noise
_PI = np.eye(2, dtype=np.complex128)
_PX = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_PY = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_PZ = np.array([[1, 0], [0, -1]], dtype=np.complex128)


def kraus_rep(nz):
    """kraus_rep (src/noise_kernels.jl:30-103) from attributes of a noise object."""
    cls = type(nz).__name__
    if cls == "Kraus":
        return [np.asarray(m, dtype=np.complex128) for m in nz.matrices]
    if cls == "BitFlip":
        p = nz.probability
        return [math.sqrt(1 - p) * _PI, math.sqrt(p) * _PX]
    if cls == "PhaseFlip":
        p = nz.probability
        return [math.sqrt(1 - p) * _PI, math.sqrt(p) * _PZ]
    if cls == "Depolarizing":
        p = nz.probability
        return [math.sqrt(1 - p) * _PI] + [math.sqrt(p / 3) * m for m in (_PX, _PY, _PZ)]
    if cls == "PauliChannel":
        return [math.sqrt(1 - nz.probX - nz.probY - nz.probZ) * _PI, math.sqrt(nz.probX) * _PX,
                math.sqrt(nz.probY) * _PY, math.sqrt(nz.probZ) * _PZ]
    if cls == "AmplitudeDamping":
        g = nz.gamma
        return [np.array([[1, 0], [0, math.sqrt(1 - g)]], dtype=np.complex128), np.array([[0, math.sqrt(g)], [0, 0]], dtype=np.complex128)]
    if cls == "GeneralizedAmplitudeDamping":
        p, g = nz.probability, nz.gamma
        return [math.sqrt(p) * np.array([[1, 0], [0, math.sqrt(1 - g)]]), math.sqrt(p) * np.array([[0, math.sqrt(g)], [0, 0]]),
                math.sqrt(1 - p) * np.array([[math.sqrt(1 - g), 0], [0, 1]]), math.sqrt(1 - p) * np.array([[0, 0], [math.sqrt(g), 0]])]
    if cls == "PhaseDamping":
        g = nz.gamma
        return [np.array([[1, 0], [0, math.sqrt(1 - g)]], dtype=np.complex128), np.array([[0, 0], [0, math.sqrt(g)]], dtype=np.complex128)]
    if cls == "TwoQubitDepolarizing":
        p = nz.probability
        ks = [np.kron(ki, kj) for kj in (_PI, _PX, _PY, _PZ) for ki in (_PI, _PX, _PY, _PZ)]
        return [math.sqrt(1 - p) * ks[0]] + [math.sqrt(p / 15) * k for k in ks[1:]]
    if cls == "TwoQubitDephasing":
        p = nz.probability
        return [math.sqrt(1 - p) * np.kron(_PI, _PI), math.sqrt(p / 3) * np.kron(_PI, _PZ),
                math.sqrt(p / 3) * np.kron(_PZ, _PI), math.sqrt(p / 3) * np.kron(_PZ, _PZ)]
    if cls == "MultiQubitPauliChannel":
        P = {"I": _PI, "X": _PX, "Y": _PY, "Z": _PZ}
        tot = sum(nz.probabilities.values())
        return [math.sqrt(1 - tot) * np.eye(4, dtype=np.complex128)] + [
            math.sqrt(v) * np.kron(P[k[0]], P[k[1]]) for k, v in nz.probabilities.items() if k != "II"]
    raise KeyError(cls)


def apply_noise(nz, rho: np.ndarray, targets, physical: bool = False):
    """apply_noise!(noise, rho, targets...) (src/noise_kernels.jl:7-196) on a column-major
    density matrix held as a flat complex128 vector, in place.  physical=True applies the
    full channel (conj(K) S K^T on every element) instead of the reference's block update."""
    L = lib()
    dim = int(round(math.sqrt(rho.size)))
    t = [int(x) for x in targets]
    if type(nz).__name__ == "PhaseFlip" and not physical:
        L.orc_dm_phase_flip(_p(rho), dim, nz.probability, t[0])
        return
    ks = kraus_rep(nz)
    kb = _cm(np.stack(ks))
    if physical:
        # canonical convention of the full channel: bit j <-> ct[j]
        if len(t) == 1:
            ct = t
        elif len(t) == 2:
            ct = [t[1], t[0]]
        else:
            ct = sorted(t, reverse=True)
        tt = np.array(ct, dtype=np.int32)
        L.orc_dm_kraus_full(_p(rho), dim, _p(kb), len(ks), len(t), _p(tt))
        return
    if len(t) == 1:
        L.orc_dm_kraus_1q(_p(rho), dim, _p(kb), len(ks), t[0])
    elif len(t) == 2:
        L.orc_dm_kraus_2q(_p(rho), dim, _p(kb), len(ks), t[0], t[1])
    else:
        tt = np.array(t, dtype=np.int32)
        L.orc_dm_kraus_nq(_p(rho), dim, _p(kb), len(ks), len(t), _p(tt))


# ---------------------------------------------------------------------------- simulators
class OracleSV:
    """StateVectorSimulator restated on the CPU (src/sv_simulator.jl)."""

    def __init__(self, n):
        self.n = n
        self.psi = np.zeros(2 ** n, dtype=np.complex128)
        self.psi[0] = 1.0

    def evolve(self, instructions):
        for ix in instructions:
            op = ix.operator
            if type(op).__name__ in ("Measure", "Reset", "Barrier", "Delay"):
                continue
            apply_gate(op, self.psi, ix.target)
        return self

    def probabilities(self):
        return np.abs(self.psi) ** 2


class OracleDM:
    """DensityMatrixSimulator restated on the CPU (src/dm_simulator.jl); vec(S) column-major."""

    def __init__(self, n, physical=False):
        self.n = n
        self.rho = np.zeros(4 ** n, dtype=np.complex128)
        self.rho[0] = 1.0
        self.physical = physical

    def evolve(self, instructions):
        for ix in instructions:
            op = ix.operator
            cls = type(op).__name__
            if cls in ("Measure", "Reset", "Barrier", "Delay"):
                continue
            if hasattr(op, "kraus_rep") or cls == "Kraus":
                apply_noise(op, self.rho, ix.target, self.physical)
            else:
                # _evolve_op! (src/dm_simulator.jl:130-140)
                apply_gate(op, self.rho, ix.target, conj=False)
                apply_gate(op, self.rho, [self.n + q for q in ix.target], conj=True)
        return self

    @property
    def matrix(self):
        d = 2 ** self.n
        return self.rho.reshape((d, d), order="F")

    def probabilities(self):
        d = 2 ** self.n
        return np.real(self.rho[:: d + 1]).copy()


# ---------------------------------------------------------------------------- sampling
def pairwise_sum(p):
    p = np.ascontiguousarray(p, dtype=np.float64)
    return lib().orc_pairwise_sum(_p(p), p.size)


def alias_table(p, wsum=None):
    """make_alias_table! (src/result_types.jl:8-54); alias entries 0-based, -1 if unset."""
    p = np.ascontiguousarray(p, dtype=np.float64)
    n = p.size
    ws = pairwise_sum(p) if wsum is None else float(wsum)
    ap = np.empty(n)
    al = np.empty(n, dtype=np.int64)
    lg = np.empty(n, dtype=np.int64)
    sm = np.empty(n, dtype=np.int64)
    lib().orc_make_alias_table(_p(p), n, ws, _p(ap), _p(al), _p(lg), _p(sm))
    return ap, al


def sample_alias(ap, al, j, u):
    j = np.ascontiguousarray(j, dtype=np.int64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(j.size, dtype=np.int64)
    lib().orc_sample_alias(_p(np.ascontiguousarray(ap)), _p(np.ascontiguousarray(al)), _p(j), _p(u), j.size, _p(out))
    return out


def sample_direct(p, u, wsum=None):
    p = np.ascontiguousarray(p, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    ws = pairwise_sum(p) if wsum is None else float(wsum)
    out = np.empty(u.size, dtype=np.int64)
    lib().orc_sample_direct(_p(p), p.size, ws, _p(u), u.size, _p(out))
    return out


# ---------------------------------------------------------------------------- expectations
def expectation_pauli_sv(psi, n, xmask, zmask):
    """<psi|P|psi> with P = prod over qubits (bit q <-> qubit q) of X/Y/Z."""
    phi = psi.copy()
    for q in range(n):
        x, z = (xmask >> q) & 1, (zmask >> q) & 1
        if x and z:
            apply_gate(_Fake("y", (), 1.0), phi, [q])
        elif x:
            apply_gate(_Fake("x", (), 1.0), phi, [q])
        elif z:
            apply_gate(_Fake("z", (), 1.0), phi, [q])
    return float(np.real(np.vdot(psi, phi)))


def expectation_pauli_dm(rho, n, xmask, zmask):
    """real(tr(apply_observable(P, S))) as src/dm_simulator.jl:181-189,253-260 compute it."""
    s = rho.copy()
    for q in range(n):
        x, z = (xmask >> q) & 1, (zmask >> q) & 1
        g = "y" if (x and z) else ("x" if x else ("z" if z else None))
        if g:
            apply_gate(_Fake(g, (), 1.0), s, [q])
    d = 2 ** n
    return float(np.real(np.sum(s[:: d + 1])))


def expectation_pauli_fast(psi, n, xmask, zmask):
    """Same number as expectation_pauli_sv (bit q <-> qubit q), from the one-pass C kernel."""
    xi = zi = 0
    ny = 0
    for q in range(n):
        x, z = (xmask >> q) & 1, (zmask >> q) & 1
        if x:
            xi |= 1 << (n - 1 - q)
        if z:
            zi |= 1 << (n - 1 - q)
        ny += int(x and z)
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    return lib().orc_expect_pauli(_p(psi), psi.size, xi, zi, ny)


# ---------------------------------------------------------------------------- gradients
# The reference has no gradient (AdjointGradient is declared in src/results.jl:90-159 and
# rejected in src/pragmas.jl:67-68).  Its users differentiate by the parameter-shift rule:
# two forward simulations per parameter.  That is restated here on the oracle's FP64
# simulator as the checker for the engine's adjoint gradients.  For a gate exp(-i phi G / 2)
# with G^2 = 1 (Rx, Ry, Rz, XX, YY, ZZ; PhaseShift = e^{i phi/2} Rz(phi)), the rule is exact:
#   dE/dphi = [E(phi + pi/2) - E(phi - pi/2)] / 2,
# and a gate raised to pow_exponent p has phi = p * theta, so dE/dtheta = p * dE/dphi.
SHIFT_GATES = ("rx", "ry", "rz", "xx", "yy", "zz", "phaseshift")


class _Ix:
    def __init__(self, operator, target):
        self.operator, self.target = operator, list(target)


def _is_param(ix):
    return _gate_desc(ix.operator)[0] in SHIFT_GATES


def hamiltonian_energy(psi, n, hamiltonian):
    """sum_t c_t <psi|P_t|psi> for terms (c_t, {qubit: 'X'|'Y'|'Z'})."""
    e = 0.0
    for c, term in hamiltonian:
        x = sum(1 << int(q) for q, p in term.items() if p.upper() in "XY")
        z = sum(1 << int(q) for q, p in term.items() if p.upper() in "YZ")
        e += float(c) * expectation_pauli_fast(psi, n, x, z)
    return e


def parameter_shift_gradient(n, instructions, hamiltonian, which=None):
    """(energy, {instruction index: dE/dtheta}) on the FP64 oracle from |0...0>.

    which: instruction indices to differentiate (default: every Rx/Ry/Rz/XX/YY/ZZ/PhaseShift).
    The state before each chosen gate is carried forward once, so the cost is one full
    forward pass plus two suffix passes per parameter."""
    ins = list(instructions)
    idx = [i for i, ix in enumerate(ins) if _is_param(ix)] if which is None else sorted(int(i) for i in which)
    sv = OracleSV(n)
    pos = 0
    grads = {}
    for i in idx:
        sv.evolve(ins[pos:i])
        pos = i
        name, ang, pw = _gate_desc(ins[i].operator)
        if name not in SHIFT_GATES:
            raise ValueError(f"instruction {i} ({name}) has no two-term shift rule")
        vals = []
        for sgn in (1.0, -1.0):
            s = OracleSV(n)
            s.psi = sv.psi.copy()
            shifted = _Ix(_Fake(name, (ang[0] + sgn * (math.pi / 2) / pw,), pw), ins[i].target)
            s.evolve([shifted] + ins[i + 1:])
            vals.append(hamiltonian_energy(s.psi, n, hamiltonian))
        grads[i] = pw * (vals[0] - vals[1]) / 2.0
    sv.evolve(ins[pos:])
    return hamiltonian_energy(sv.psi, n, hamiltonian), grads
