"""Pins the oracle (CPU restatement of the reference) to the reference's own golden
vectors, and the product's host gate model to the oracle's independent matrix tables."""
import math

import numpy as np
import pytest

import oracle
from conftest import bs, make_op, rel_err
from golden import reference_kats as K


def _sv(case):
    ins, n, sv, probs = case
    o = oracle.OracleSV(n).evolve([make_op(s) for s in ins])
    return o, n, sv, probs


@pytest.mark.parametrize("case", K.SV_KATS + K.CUSTOM_KATS, ids=lambda c: "+".join(s[0] for s in c[0]))
def test_oracle_sv_kats(case):
    o, n, sv, probs = _sv(case)
    assert rel_err(o.psi, sv) < 1e-7
    if probs is not None:
        assert rel_err(o.probabilities(), probs) < 1e-7


@pytest.mark.parametrize("case", K.SV_KATS + K.CUSTOM_KATS[:-1], ids=lambda c: "+".join(s[0] for s in c[0]))
def test_oracle_dm_runs_sv_kats(case):
    # the reference runs every SV known-answer circuit on the DM simulator too (test_sv_simulator.jl:272-280)
    ins, n, sv, probs = case
    o = oracle.OracleDM(n).evolve([make_op(s) for s in ins])
    assert rel_err(o.probabilities(), probs) < 1e-7


@pytest.mark.parametrize("case", K.DM_KATS, ids=lambda c: "+".join(s[0] for s in c[0]))
def test_oracle_dm_kats(case):
    ins, n, dm, probs = case
    o = oracle.OracleDM(n).evolve([make_op(s) for s in ins])
    assert rel_err(o.matrix, dm) < 1e-7
    assert rel_err(o.probabilities(), probs) < 1e-7


def test_oracle_two_qubit_pauli_channel_equals_kraus():
    # test/test_dm_simulator.jl:23-30,92-104
    a = oracle.OracleDM(2).evolve([make_op(("x", (), [0])), make_op(("x", (), [1])),
                                   bs.Instruction(bs.TwoQubitPauliChannel({"XX": 0.1, "YZ": 0.2}), [0, 1])])
    b = oracle.OracleDM(2).evolve([make_op(("x", (), [0])), make_op(("x", (), [1])),
                                   bs.Instruction(bs.Kraus(K.TQPC_KRAUS), [0, 1])])
    assert rel_err(a.matrix, b.matrix) < 1e-14


@pytest.mark.parametrize("nq", [1, 2, 3, 4])
def test_oracle_gphase(nq):
    # test/test_custom_gates.jl:89-110
    ins = [make_op(("h", (), [q])) for q in range(nq)] + [bs.Instruction(bs.GPhase(nq, K.GPHASE_PHI), list(range(nq)))]
    o = oracle.OracleSV(nq).evolve(ins)
    assert rel_err(o.psi, np.exp(1j * K.GPHASE_PHI) / math.sqrt(2 ** nq) * np.ones(2 ** nq)) < 1e-12


@pytest.mark.parametrize("nq", [1, 2, 3, 4, 5, 6])
def test_oracle_multirz(nq):
    # test/test_custom_gates.jl:111-127
    phi = 2.12
    ins = [make_op(("h", (), [q])) for q in range(nq)] + [bs.Instruction(bs.MultiRZ(phi), list(range(nq)))]
    o = oracle.OracleSV(nq).evolve(ins)
    ev = oracle.pauli_eigenvalues(nq)
    assert rel_err(o.psi, math.sqrt(1 / 2 ** nq) * np.exp(-1j * phi / 2 * ev)) < 1e-12


def test_pauli_eigenvalue_formula_matches_parity():
    # src/operators.jl:156-185 restated literally for N < 5, recursion for N >= 5
    def ref(N, i):
        if N == 1:
            return (1.0, -1.0)[i - 1]
        i_block = (i - 1) // 2
        split = (2 ** (N - 1) - 1) // 2
        if N < 5:
            ev = 1.0 if (i - 1) % 2 == 0 else -1.0
            if i_block <= split:
                mi, di = i_block % 2, i_block // 2
                return -ev if (mi % 2 == 1) ^ (di % 2 == 1) else ev
            mi, di = (i_block - split - 1) % 2, (i_block - split - 1) // 2
            return ev if (mi % 2 == 1) ^ (di % 2 == 1) else -ev
        new_i = i - 2 ** (N - 1) if i > 2 ** (N - 1) else i
        od = ref(N - 1, new_i)
        return od if i_block <= split else -od
    for N in range(1, 9):
        assert np.array_equal([ref(N, i) for i in range(1, 2 ** N + 1)], oracle.pauli_eigenvalues(N))
        assert np.array_equal(bs.gates.pauli_eigenvalues(N), oracle.pauli_eigenvalues(N))


@pytest.mark.parametrize("nq,g", [(2, "cnot"), (3, "ccnot")])
def test_oracle_control(nq, g):
    # test/test_custom_gates.jl:128-158
    cx = bs.Control(bs.X(), (1,))
    gate = cx if nq == 2 else bs.Control(cx, (1,))
    ins = [make_op(("h", (), [0]))] + [make_op(("cnot", (), [q, q + 1])) for q in range(nq - 2)]
    a = oracle.OracleSV(nq).evolve(ins + [bs.Instruction(gate, list(range(nq)))])
    b = oracle.OracleSV(nq).evolve(ins + [make_op((g, (), list(range(nq))))])
    v = np.zeros(2 ** nq)
    v[0] = v[-1] = 1 / math.sqrt(2)
    assert rel_err(a.psi, v) < 1e-12 and rel_err(b.psi, v) < 1e-12


def test_oracle_qft_uniform():
    # test/test_sv_simulator.jl:360-384 (4..12 here; the GPU test covers up to 20)
    for n in range(4, 13):
        ops = []
        for t in range(n):
            ops.append(bs.Instruction(bs.H(), [t]))
            ang = math.pi / 2
            for c in range(t + 1, n):
                ops.append(bs.Instruction(bs.CPhaseShift(ang), [c, t]))
                ang /= 2
        o = oracle.OracleSV(n).evolve(ops)
        assert rel_err(o.probabilities(), np.full(2 ** n, 1 / 2 ** n)) < 1e-10


def test_oracle_partial_trace_kats():
    # test/test_result_types.jl:44-58,239-246 (rtol 1e-6)
    psi = K.RT_STATE
    rho3 = bs.partial_trace(psi, [3])
    assert np.allclose(rho3, K.RT_DM_3, rtol=1e-6, atol=1e-8)
    rho021 = bs.partial_trace(psi, [0, 2, 1])
    assert np.allclose(rho021, K.RT_DM_021, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("nq", [3, 4, 5])
def test_partial_trace_sv_equals_dm(nq):
    # test/test_sv_simulator.jl:654-662
    rng = np.random.default_rng(nq)
    psi = rng.normal(size=2 ** nq) + 1j * rng.normal(size=2 ** nq)
    psi /= np.linalg.norm(psi)
    full = np.outer(psi, psi.conj())
    import itertools
    for r in range(1, nq + 1):
        for q in itertools.combinations(range(nq), r):
            assert np.allclose(bs.partial_trace(psi, list(q)), bs.partial_trace(full, list(q)), atol=1e-13)


def test_marginal_probability_kat():
    # test/test_result_types.jl:31-40
    p = np.abs(K.RT_STATE) ** 2
    m12 = [p[[0, 1, 8, 9]].sum(), p[[2, 3, 10, 11]].sum(), p[[4, 5, 12, 13]].sum(), p[[6, 7, 14, 15]].sum()]
    assert np.allclose(bs.marginal_probability(p, 4, [1, 2]), m12, rtol=1e-14)
    # test/test_result_types.jl:209-214: reversed targets leave the vector unchanged
    assert np.allclose(bs.permute_probability(p, 4, [3, 2, 1, 0]), p)
    rho = np.outer(K.RT_STATE, K.RT_STATE.conj())
    assert np.allclose(bs.permute_density_matrix(rho, 4, [3, 2, 1, 0]), rho)


# ---------------------------------------------------------------- gate model vs oracle tables
_ANGLED = ["rx", "ry", "rz", "phaseshift", "cphaseshift", "cphaseshift00", "cphaseshift01", "cphaseshift10", "xx", "yy",
           "xy", "zz", "gpi", "gpi2", "single_excitation", "single_excitation_plus", "single_excitation_minus",
           "fermionic_swap", "double_excitation", "double_excitation_plus", "double_excitation_minus", "pswap"]
_FIXED = ["h", "x", "y", "z", "s", "si", "t", "ti", "v", "vi", "i", "cnot", "cy", "cz", "cv", "swap", "iswap", "ecr",
          "ccnot", "cswap"]


@pytest.mark.parametrize("pw", K.GO_POWS + (-1, 5, 1.5, -3))
def test_product_matrices_match_oracle_tables(pw):
    from conftest import GATES_1, GATES_A
    for nm in _FIXED:
        g = GATES_1[nm](pow_exponent=pw)
        assert np.allclose(g.matrix_rep(), oracle.matrix_rep(nm, (), pw), atol=1e-13), (nm, pw)
    for nm in _ANGLED:
        g = GATES_A[nm](K.GO_PHI, pow_exponent=pw)
        assert np.allclose(g.matrix_rep(), oracle.matrix_rep(nm, (K.GO_PHI,), pw), atol=1e-13), (nm, pw)
    for nm, a in (("prx", (K.GO_THETA, K.GO_PHI)), ("ms", (K.GO_THETA, K.GO_PHI, K.GO_LAMBDA)),
                  ("u", (K.GO_THETA, K.GO_PHI, K.GO_LAMBDA))):
        g = GATES_A[nm](*a, pow_exponent=pw)
        assert np.allclose(g.matrix_rep(), oracle.matrix_rep(nm, a, pw), atol=1e-13), (nm, pw)


@pytest.mark.parametrize("pw", K.GO_POWS)
def test_pow_identity(pw):
    # test/test_gate_operations.jl:84-110: matrix_rep(g)^pow == matrix_rep(g^pow)
    from conftest import GATES_1, GATES_A
    for nm in ["x", "y", "z", "h", "s", "si", "t", "ti", "v", "vi"]:
        g = GATES_1[nm]()
        assert np.allclose(bs.gates._mat_pow(g.matrix_rep(), pw), (g ** pw).matrix_rep(), atol=1e-8), nm
    for nm in ["rx", "ry", "rz", "phaseshift", "gpi", "gpi2"]:
        g = GATES_A[nm](K.GO_PHI)
        assert np.allclose(bs.gates._mat_pow(g.matrix_rep(), pw), (g ** pw).matrix_rep(), atol=1e-8), nm


def test_inverse_identity():
    # test/test_gate_operations.jl:10-36
    from conftest import GATES_1, GATES_A
    gs = [GATES_1[n]() for n in ["x", "y", "z", "h", "s", "si", "t", "ti", "v", "vi", "cnot", "cy", "cz", "cv", "swap", "iswap", "ecr"]]
    gs += [GATES_A[n](K.GO_PHI) for n in ["rx", "ry", "rz", "phaseshift", "gpi", "gpi2", "xx", "yy", "zz", "xy", "pswap"]]
    gs += [bs.U(K.GO_THETA, K.GO_PHI, K.GO_LAMBDA), bs.PRx(K.GO_THETA, K.GO_PHI), bs.MS(K.GO_THETA, K.GO_PHI, K.GO_LAMBDA)]
    for g in gs:
        m = g.matrix_rep()
        assert np.allclose(g.inv().matrix_rep() @ m, np.eye(m.shape[0]), atol=1e-8), g


# ---------------------------------------------------------------- sampling restatement
def test_alias_table_is_a_valid_alias_method():
    rng = np.random.default_rng(7)
    for n in (1, 2, 5, 64, 1000):
        p = rng.random(n) ** 3
        p /= p.sum()
        ap, al = oracle.alias_table(p)
        # reconstructed probabilities: p_i = (ap_i + sum_{j: alias j = i} (1 - ap_j)) / n
        rec = ap.copy()
        for j in range(n):
            if ap[j] < 1.0:
                rec[al[j]] += 1.0 - ap[j]
        assert np.allclose(rec / n, p, atol=1e-12)


def test_alias_draws_follow_reference_rule():
    p = np.array([0.1, 0.2, 0.3, 0.4])
    ap, al = oracle.alias_table(p)
    j = np.array([0, 1, 2, 3, 0, 3])
    u = np.array([0.05, 0.99, 0.5, 0.2, 0.9, 0.0])
    out = oracle.sample_alias(ap, al, j, u)
    exp = [jj if uu < ap[jj] else al[jj] for jj, uu in zip(j, u)]
    assert list(out) == exp


def test_direct_sampling_linear_scan():
    p = np.array([0.25, 0.0, 0.25, 0.5])
    u = np.array([0.0, 0.1, 0.25, 0.26, 0.5, 0.51, 0.999999])
    out = oracle.sample_direct(p, u, 1.0)
    # first index with running sum >= u * wsum
    exp = []
    for uu in u:
        cw, i = p[0], 0
        while cw < uu and i < 3:
            i += 1
            cw += p[i]
        exp.append(i)
    assert list(out) == exp
