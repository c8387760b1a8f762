"""CPU-only checks of the boundary: the engine library loads, exports every entry
point the header declares, and the host-side lowering keeps the reference's
kernel conventions.  No compute call is made (no GPU here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, bs

HEADER = os.path.join(ROOT, "include", "braket_gb300.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(bs_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def libpath():
    b = bs_build()
    return b


def bs_build():
    import importlib
    build = importlib.import_module("braketsimulator_gb300.build")
    try:
        return build.build_library()
    except RuntimeError as e:   # pragma: no cover - nvcc missing
        pytest.skip(str(e))


def test_library_exports_every_declared_entry_point(libpath):
    L = ctypes.CDLL(libpath)
    decl = _declared()
    assert len(decl) >= 29
    for name in decl:
        assert hasattr(L, name), name
    # and the ctypes table covers the header
    assert set(decl) == set(bs._abi.SIGNATURES), set(decl) ^ set(bs._abi.SIGNATURES)
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bs_\w+)", out))
    assert set(decl) <= exported


def test_version_string_without_gpu(libpath):
    L = ctypes.CDLL(libpath)
    L.bs_version.restype = ctypes.c_char_p
    assert b"sm_103a" in L.bs_version()


def test_null_handle_is_rejected_without_gpu(libpath):
    L = ctypes.CDLL(libpath)
    L.bs_destroy.argtypes = [ctypes.c_void_p]
    assert L.bs_destroy(None) == 0
    L.bs_reinit.argtypes = [ctypes.c_void_p, ctypes.c_int]
    assert L.bs_reinit(None, 3) == 1
    L.bs_last_error.restype = ctypes.c_char_p
    L.bs_last_error.argtypes = [ctypes.c_void_p]
    assert L.bs_last_error(None) == b"null handle"


def test_op_struct_layout_matches_header():
    # bs_op: 4 int32 header, targets[10], controls[16], control_values[16], 2 int32, pointer
    assert ctypes.sizeof(bs._abi.BsOp) == 4 * 4 + 4 * (10 + 16 + 16) + 8 + 8


# ---------------------------------------------------------------- host lowering conventions
def test_two_target_gates_use_first_target_as_bit0():
    lg = bs.gates.lower_gate(bs.ECR(), [3, 1])
    assert len(lg) == 1 and lg[0].targets == (3, 1) and lg[0].flags == 0
    assert np.allclose(lg[0].matrix, bs.ECR().matrix_rep())


def test_three_plus_targets_use_sorted_convention():
    u = np.eye(8)
    lg = bs.gates.lower_gate(bs.Unitary(u), [2, 0, 1])
    assert lg[0].flags & bs._abi.BS_GATE_SORTED_TARGETS


def test_controlled_builtins_lower_to_controls():
    lg = bs.gates.lower_gate(bs.CCNot(), [4, 2, 0])
    assert lg[0].controls == (4, 2) and lg[0].targets == (0,) and lg[0].control_values == (1, 1)
    assert np.allclose(lg[0].matrix, [[0, 1], [1, 0]])
    lg = bs.gates.lower_gate(bs.Control(bs.Ry(0.3), (0, 1)), [1, 2, 3])
    assert lg[0].control_values == (0, 1)


def test_double_excitation_uses_big_endian_two_amplitude_rule():
    lg = bs.gates.lower_gate(bs.DoubleExcitation(0.4, pow_exponent=2.0), [0, 1, 2, 3])
    assert lg[0].flags == bs._abi.BS_GATE_MSB_FIRST
    m = lg[0].matrix
    assert np.isclose(m[3, 12], -np.sin(0.4)) and np.isclose(m[12, 3], np.sin(0.4))


def test_kraus_flags_follow_reference_kernels():
    from braketsimulator_gb300.noises import kraus_flags, lower_noise
    assert kraus_flags(1) == 0
    assert kraus_flags(2) == bs._abi.BS_GATE_MSB_FIRST
    assert kraus_flags(3) == bs._abi.BS_GATE_SORTED_TARGETS
    ln = lower_noise(bs.PhaseFlip(0.1), [0], bs._abi.BS_NOISE_REFERENCE)
    assert ln.flags & bs._abi.BS_NOISE_PHYSICAL      # the reference's PhaseFlip kernel is a full update


def test_multirz_dispatch():
    assert isinstance(bs.gates.lower_gate(bs.MultiRZ(0.3), [2])[0].matrix, np.ndarray)
    lg = bs.gates.lower_gate(bs.MultiRZ(0.3, pow_exponent=5.0), [0, 1, 2])
    # pow_exponent is ignored for >= 3 targets, as in the reference
    assert lg[0].diagonal and np.allclose(lg[0].matrix, np.exp(-0.15j * bs.gates.pauli_eigenvalues(3)))


def test_new_entry_points_reject_bad_arguments_without_a_gpu_call():
    """Argument checks of the batch, tuning and partial-trace entry points run on the host and
    return a status before any device work (NULL handles, bad counts)."""
    import ctypes as C
    L = bs._abi.lib()
    out = C.c_void_p()
    assert L.bs_batch_create(0, None, None, None, 0, None, None, 0, 0, 0, C.byref(out)) != 0
    assert L.bs_batch_launch(None, None, None, None) != 0
    assert L.bs_batch_set_ops(None, None, None) != 0
    assert L.bs_batch_set_tuning(None, 0, None, None) != 0
    assert L.bs_batch_destroy(None) == 0
    v = C.c_double()
    assert L.bs_set_tuning(None, 0, 1.0) != 0
    assert L.bs_get_tuning(None, 0, C.byref(v)) != 0
    assert L.bs_reduced_density_matrix(None, 1, None, None) != 0
    n = C.c_int64()
    assert L.bs_write_result_file(None, 0, b"/dev/null", C.byref(n)) != 0
    assert L.bs_selftest_wait_timeout(None, 0.01) != 0


def test_rotation_fast_lowering_matches_generic_lowering():
    """1-qubit rotations skip the generic dispatch; the op struct and matrix they produce are the
    generic lowering's (no flags, one target, the gate's own matrix_rep, powers included)."""
    import numpy as np
    from braketsimulator_gb300 import gates as G, simulators as S
    rng = np.random.default_rng(1)
    for cls in (G.Rx, G.Ry, G.Rz):
        for pw in (1.0, 0.5, -2.0):
            g = cls(float(rng.uniform(-7, 7)), pow_exponent=pw)
            q = int(rng.integers(20))
            (raw, buf), = S._rotation_op(g, q)
            (lg,) = G.lower_gate(g, (q,))
            o = bs._abi.BsOp.from_buffer_copy(raw)
            assert (o.kind, o.flags, o.n_targets, o.targets[0], o.n_controls, o.n_matrices) == (0, lg.flags, 1, q, 0, 0)
            assert np.array_equal(buf, bs._abi.cplx_buffer(lg.matrix))
            assert S._gate_ops(g, (q,))[0][1].dtype == np.float64
    # at pow_exponent 1 the entries are written directly: the same bytes as the complex arithmetic,
    # signed zeros included
    for cls in (G.Rx, G.Ry, G.Rz):
        for a in [0.0, -0.0, np.pi, -np.pi, 2 * np.pi, 1e-300, -1e-300] + list(rng.uniform(-50, 50, 400)):
            g = cls(float(a))
            assert S._rotation_buffer(g).tobytes() == bs._abi.cplx_buffer(g.matrix_rep()).tobytes()


def test_lowered_op_arrays_match_gate_by_gate_lowering():
    """_ops_for puts every pow-1 rotation's matrix into one buffer shared by the list: each op must
    equal the gate-by-gate lowering's (struct fields, and the matrix bytes it points at)."""
    import ctypes as C
    import numpy as np
    from braketsimulator_gb300 import gates as G, simulators as S
    rng = np.random.default_rng(5)
    kinds = [lambda q: (G.Rx(float(rng.uniform(-9, 9))), (q,)), lambda q: (G.Ry(float(rng.uniform(-9, 9))), (q,)),
             lambda q: (G.Rz(float(rng.uniform(-9, 9))), (q,)), lambda q: (G.Rz(0.0), (q,)),
             lambda q: (G.Rx(0.4, pow_exponent=2.0), (q,)), lambda q: (G.H(), (q,)),
             lambda q: (G.CNot(), (q, (q + 1) % 6)), lambda q: (G.XX(0.3), (q, (q + 2) % 6)),
             lambda q: (G.Unitary(np.eye(2) * np.exp(0.1j)), (q,))]
    for trial in range(20):
        ops = []
        for _ in range(40):
            g, t = kinds[int(rng.integers(len(kinds)))](int(rng.integers(6)))
            ops.append(bs.Instruction(g, list(t)))
        arr, n, keep = S._ops_for(ops, False, 0)
        expect = [pair for ix in ops for pair in S._gate_ops(ix.operator, tuple(ix.target))]
        assert n == len(expect)
        size = C.sizeof(bs._abi.BsOp)
        off = bs._abi.BsOp.matrix.offset
        for i, (raw, buf) in enumerate(expect):
            got = bytes(C.string_at(C.addressof(arr) + i * size, size))
            assert got[:off] == raw[:off] and got[off + 8:] == raw[off + 8:]
            nbytes = buf.size * 8
            assert C.string_at(arr[i].matrix, nbytes) == buf.tobytes()
