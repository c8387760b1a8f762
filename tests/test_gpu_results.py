"""Probabilities, expectations, variances, marginals and sampling on the GPU."""
import math

import numpy as np
import pytest

import oracle
from conftest import bs, random_circuit, rel_err
from golden import reference_kats as K

pytestmark = pytest.mark.gpu
O = bs.observables


def _state_sim(kind):
    if kind == "sv":
        s = bs.StateVectorSimulator(4, 1000)
        s.state_vector = K.RT_STATE
    else:
        s = bs.DensityMatrixSimulator(4, 1000)
        s.density_matrix = np.outer(K.RT_STATE, K.RT_STATE.conj()).T   # stored matrix is rho^T
    return s


def _diag_expect(vec_or_rho, targets, evs, kind):
    p = np.abs(vec_or_rho) ** 2 if kind == "sv" else np.real(np.diag(vec_or_rho))
    m = bs.marginal_probability(p, 4, targets)
    return float(np.dot(m, evs))


OBS = [
    (O.TensorProduct([O.X(), O.H()]), (1, 2)),
    (O.TensorProduct([O.I(), O.Y()]), (0, 2)),
    (O.Y(), (2,)),
]


@pytest.mark.parametrize("kind", ["sv", "dm"])
@pytest.mark.parametrize("obs", OBS, ids=repr)
def test_expectation_and_variance_vs_diagonalisation(kind, obs):
    # test/test_result_types.jl:140-180
    sim = _state_sim(kind)
    sim.apply_observables([obs])
    rotated = sim.state_with_observables()
    evs = obs[0].eigvals()
    e = bs.calculate(bs.Expectation(*obs), sim)
    assert abs(e - _diag_expect(rotated, list(obs[1]), evs, kind)) < 1e-12
    v = bs.calculate(bs.Variance(*obs), sim)
    p = np.abs(rotated) ** 2 if kind == "sv" else np.real(np.diag(rotated))
    m = bs.marginal_probability(p, 4, list(obs[1]))
    assert abs(v - (np.dot(m, evs ** 2) - np.dot(m, evs) ** 2)) < 1e-12


@pytest.mark.parametrize("kind", ["sv", "dm"])
@pytest.mark.parametrize("obs", [O.X(), O.Y(), O.Z(), O.H(), O.I(), O.HermitianObservable([[0.0, 1.0], [1.0, 0.0]])], ids=repr)
def test_all_qubit_expectations(kind, obs):
    sim = _state_sim(kind)
    vals = bs.calculate(bs.Expectation(obs, (0, 1, 2, 3)), sim)
    for t, val in zip(range(4), vals):
        s2 = _state_sim(kind)
        s2.apply_observables([(obs, [t])])
        r = s2.state_with_observables()
        assert abs(val - _diag_expect(r, [t], obs.eigvals(), kind)) < 1e-12


@pytest.mark.parametrize("kind", ["sv", "dm"])
def test_probability_and_density_matrix_results(kind):
    sim = _state_sim(kind)
    p = np.abs(K.RT_STATE) ** 2
    assert rel_err(bs.calculate(bs.Probability((0, 1, 2, 3)), sim), p) < 1e-14
    m12 = [p[[0, 1, 8, 9]].sum(), p[[2, 3, 10, 11]].sum(), p[[4, 5, 12, 13]].sum(), p[[6, 7, 14, 15]].sum()]
    assert rel_err(bs.calculate(bs.Probability((1, 2)), sim), m12) < 1e-13
    assert rel_err(bs.calculate(bs.Probability((3, 2, 1, 0)), sim), p) < 1e-14
    if kind == "sv":
        amp = bs.calculate(bs.Amplitude(["0010", "0101", "1110"]), sim)
        assert abs(amp["0010"] - K.RT_STATE[2]) < 1e-15 and abs(amp["1110"] - K.RT_STATE[14]) < 1e-15
        assert np.allclose(bs.calculate(bs.DensityMatrix((3,)), sim), K.RT_DM_3, rtol=1e-6)
        assert np.allclose(bs.calculate(bs.DensityMatrix((0, 2, 1)), sim), K.RT_DM_021, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("n", [3, 9, 14])
def test_pauli_expectations_random(n):
    rng = np.random.default_rng(n)
    ops = random_circuit(n, 40, rng)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    psi = oracle.OracleSV(n).evolve(ops).psi
    for _ in range(12):
        x = int(rng.integers(0, 2 ** n))
        z = int(rng.integers(0, 2 ** n))
        xm = np.array([x], dtype=np.uint64)
        zm = np.array([z], dtype=np.uint64)
        out = np.empty(1)
        sim._h.call("bs_expectation_pauli", 1, bs._abi.u64ptr(xm), bs._abi.u64ptr(zm), bs._abi.dptr(np.ones(1)), bs._abi.dptr(out))
        assert abs(out[0] - oracle.expectation_pauli_sv(psi, n, x, z)) < 1e-12


@pytest.mark.parametrize("n", [2, 5])
def test_pauli_expectations_dm(n):
    rng = np.random.default_rng(n + 10)
    ops = random_circuit(n, 25, rng) + [bs.Instruction(bs.Depolarizing(0.1), [0])]
    sim = bs.DensityMatrixSimulator(n, 0).evolve(ops)
    rho = oracle.OracleDM(n).evolve(ops).rho
    for _ in range(10):
        x, z = int(rng.integers(0, 2 ** n)), int(rng.integers(0, 2 ** n))
        out = np.empty(1)
        sim._h.call("bs_expectation_pauli", 1, bs._abi.u64ptr(np.array([x], dtype=np.uint64)),
                    bs._abi.u64ptr(np.array([z], dtype=np.uint64)), bs._abi.dptr(np.ones(1)), bs._abi.dptr(out))
        assert abs(out[0] - oracle.expectation_pauli_dm(rho, n, x, z)) < 1e-12


def test_hermitian_multi_target_expectation():
    rng = np.random.default_rng(11)
    n = 6
    ops = random_circuit(n, 30, rng)
    a = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    h = a + a.conj().T
    for kind in ("sv", "dm"):
        sim = (bs.StateVectorSimulator if kind == "sv" else bs.DensityMatrixSimulator)(n, 0).evolve(ops)
        for t in ([4, 1, 2], [0, 5, 3]):
            e = sim.expectation(O.HermitianObservable(h), *t)
            # oracle: rotate into the eigenbasis and weight the marginal by eigenvalues
            w, v = np.linalg.eigh(h)
            if kind == "sv":
                psi = oracle.OracleSV(n).evolve(ops).psi
                phi = psi.copy()
                oracle.apply_gate(bs.Unitary(v.conj().T), phi, t)
                m = bs.marginal_probability(np.abs(phi) ** 2, n, t)
            else:
                r = oracle.OracleDM(n).evolve(ops)
                rr = r.rho.copy()
                oracle.apply_gate(bs.Unitary(v.conj().T), rr, t)
                oracle.apply_gate(bs.Unitary(v.conj().T), rr, [n + q for q in t], conj=True)
                d = 2 ** n
                m = bs.marginal_probability(np.real(rr[:: d + 1]), n, t)
            # eigenvalue order follows the sorted-target convention of both kernels
            assert abs(e - float(np.dot(m, w))) < 1e-10, (kind, t)


# ---------------------------------------------------------------- sampling
@pytest.mark.parametrize("n", [1, 4, 10, 16])
def test_alias_bit_exact_on_supplied_stream(n):
    rng = np.random.default_rng(n)
    p = rng.random(2 ** n) ** 4
    p /= p.sum()
    ws = oracle.pairwise_sum(p)
    shots = 5000
    j = rng.integers(0, 2 ** n, shots)
    u = rng.random(shots)
    sim = bs.StateVectorSimulator(n, shots)
    got = sim.samples_from_stream(j, u, wsum=ws, probabilities=p)
    ap, al = oracle.alias_table(p, ws)
    gap, gal = sim.alias_table()
    assert np.array_equal(gap, ap) and np.array_equal(gal, al)
    assert np.array_equal(got, oracle.sample_alias(ap, al, j, u))


def _represented(ap, al):
    """Distribution an alias table encodes (times n): bucket b keeps ap[b] for itself and gives
    1 - ap[b] to alias[b]."""
    w = np.array(ap, dtype=np.float64)
    give = np.where(al >= 0, 1.0 - ap, 0.0)
    np.add.at(w, np.where(al >= 0, al, 0), give)
    return w


@pytest.mark.parametrize("n,kind", [(1, "sv"), (6, "sv"), (12, "sv"), (20, "sv"), (6, "dm"), (16, "c64")])
def test_parallel_alias_table_is_valid_and_exact(n, kind):
    """BS_ALIAS_PARALLEL: a different table from the reference's serial one, for the same
    distribution.  Every bucket is a probability with a valid alias where it is below 1, and the
    distribution the table encodes equals the state's probabilities to rounding."""
    rng = np.random.default_rng(40 + n)
    if kind == "dm":
        sim = bs.DensityMatrixSimulator(n, 0).evolve(random_circuit(n, 20, rng))
    else:
        sim = bs.StateVectorSimulator(n, 0, precision="c64" if kind == "c64" else "c128")
        sim.evolve(random_circuit(n, 40, rng))
    p = sim.probabilities()
    N = p.size
    sim.alias_build(parallel=True)
    ap, al = sim.alias_table()
    assert np.all((ap >= 0) & (ap <= 1))
    low = ap < 1
    assert np.all((al[low] >= 0) & (al[low] < N) & (al[low] != np.arange(N)[low]))
    target = p * N / math.fsum(p)
    # the weights' own FP64 roundings leave at most ~2.2e-16 N of weight unbalanced (it stays with the
    # last bucket, as the serial algorithm's leftovers do); everything else is exact
    scale = max(1.0, float(np.max(target)))
    assert np.max(np.abs(_represented(ap, al) - target)) < 3e-16 * N + 1e-12 * scale
    # the serial table (float-float weight sum) encodes the same distribution
    sim.alias_build(parallel=False)
    sap, sal = sim.alias_table()
    assert np.max(np.abs(_represented(sap, sal) - target)) < 4e-15 * N + 1e-10 * scale


def test_parallel_alias_extreme_distributions():
    """One populated basis state; all weight equal; one state holding half of it."""
    for prep in ([bs.Instruction(bs.X(), [3])], [bs.Instruction(bs.H(), [q]) for q in range(8)],
                 [bs.Instruction(bs.H(), [0]), bs.Instruction(bs.CNot(), [0, 5])] +
                 [bs.Instruction(bs.Ry(0.3 * (q + 1)), [q]) for q in range(1, 5)]):
        sim = bs.StateVectorSimulator(8, 0).evolve(prep)
        p = sim.probabilities()
        sim.alias_build(parallel=True)
        ap, al = sim.alias_table()
        assert np.all((ap >= 0) & (ap <= 1))
        assert np.all(al[ap < 1] >= 0)
        assert np.max(np.abs(_represented(ap, al) - p * 256 / math.fsum(p))) < 1e-12 * 256


def test_parallel_alias_draws_follow_the_distribution():
    n, shots = 10, 400000
    rng = np.random.default_rng(5)
    sim = bs.StateVectorSimulator(n, 0).evolve(random_circuit(n, 40, rng))
    p = sim.probabilities()
    j = rng.integers(0, 2 ** n, shots)
    u = rng.random(shots)
    got = sim.samples_from_stream(j, u, parallel=True)
    ap, al = sim.alias_table()
    assert np.array_equal(got, oracle.sample_alias(ap, al, j, u))     # the draw rule on the same table
    counts = np.bincount(got, minlength=2 ** n)
    exp = p / p.sum() * shots
    keep = exp > 20
    chi2 = float(np.sum((counts[keep] - exp[keep]) ** 2 / exp[keep]))
    dof = int(keep.sum()) - 1
    assert chi2 < dof + 6 * np.sqrt(2 * dof)


@pytest.mark.parametrize("n", [6, 12, 18])
def test_direct_sampling_matches_linear_scan(n):
    rng = np.random.default_rng(n + 1)
    ops = random_circuit(n, 30, rng)
    sim = bs.StateVectorSimulator(n, 0).evolve(ops)
    p = sim.probabilities()
    u = rng.random(20000)
    got = sim.samples_direct(u, wsum=float(np.sum(p)))
    ref = oracle.sample_direct(p, u, float(np.sum(p)))
    mismatches = int(np.sum(got != ref))
    assert mismatches <= 2, mismatches      # only possible at FP boundaries of the running sum


def test_sample_statistics():
    # test/test_sv_simulator.jl:385-398 (Bell pair, 10000 shots)
    sim = bs.StateVectorSimulator(2, 10000).evolve([bs.Instruction(bs.H(), [0]), bs.Instruction(bs.CNot(), [0, 1])])
    s = sim.samples(seed=99)
    vals, counts = np.unique(s, return_counts=True)
    assert list(vals) == [0, 3] and counts.sum() == 10000 and 0.4 < counts[0] / 10000 < 0.6
    dm = bs.DensityMatrixSimulator(2, 10000).evolve([bs.Instruction(bs.H(), [0]), bs.Instruction(bs.CNot(), [0, 1])])
    s = dm.samples(seed=7)
    vals, counts = np.unique(s, return_counts=True)
    assert list(vals) == [0, 3] and 0.4 < counts[0] / 10000 < 0.6


def test_simulate_program_ghz_batch():
    # test/test_sv_simulator.jl:399-419
    prog = bs.Program([bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, 5)])
    res = bs.simulate(bs.StateVectorSimulator(5, 0), [prog] * 4, 1000, seed=5)
    for r in res:
        m = r["measurements"]
        assert m.shape == (1000, 5)
        assert 400 < np.sum(np.all(m == 0, axis=1)) < 600 and 400 < np.sum(np.all(m == 1, axis=1)) < 600


@pytest.mark.parametrize("n,keep", [(5, (3,)), (5, (0, 2, 1)), (9, (8, 0, 4, 2)), (11, (1, 3, 5, 7, 9, 10)),
                                    (13, tuple(range(0, 13, 2))), (14, tuple(range(2, 14)))])
def test_device_partial_trace_matches_host(n, keep):
    """The device partial trace (float-float sums) equals the host restatement of the reference's
    loops, for state vectors and density matrices, sorted and unsorted kept qubits."""
    rng = np.random.default_rng(n + len(keep))
    ops = random_circuit(n, 40, rng)
    sv = bs.StateVectorSimulator(n, 0)
    sv.evolve(ops)
    psi = sv.state_vector
    got = bs.calculate(bs.DensityMatrix(keep), sv)
    if len(keep) <= 8:
        ref = bs.partial_trace(psi, list(keep))   # the reference's loops, restated
    else:
        # many kept qubits: the same matrix by tensor contraction (kept qubits in descending order of
        # their endian bits, i.e. ascending qubit numbers, then the reference's reordering)
        t = psi.reshape([2] * n)
        kept = sorted(keep)
        tr = [q for q in range(n) if q not in kept]
        a = np.transpose(t, kept + tr).reshape(1 << len(kept), -1)
        nat = a @ a.conj().T
        ref = nat if list(keep) == kept else None
    if ref is not None:
        assert np.max(np.abs(got - ref)) < 1e-13
    if n <= 7:
        dm = bs.DensityMatrixSimulator(n, 0)
        dm.evolve(ops + [bs.Instruction(bs.Depolarizing(0.1), [0])])
        rho = dm.density_matrix
        assert np.max(np.abs(bs.calculate(bs.DensityMatrix(keep), dm) - bs.partial_trace(rho, list(keep)))) < 1e-13


@pytest.mark.parametrize("n,keep", [(17, tuple(range(1, 15))), (15, tuple(range(15))), (16, tuple(range(0, 16, 1))[2:])])
def test_device_partial_trace_wide(n, keep):
    """More than 12 kept qubits (and all of them: the state vector's density matrix) on the device,
    against the same matrix by tensor contraction of the oracle's state."""
    rng = np.random.default_rng(n + 3 * len(keep))
    ops = random_circuit(n, 30, rng)
    sv = bs.StateVectorSimulator(n, 0).evolve(ops)
    got = bs.calculate(bs.DensityMatrix(keep), sv)
    psi = oracle.OracleSV(n).evolve(ops).psi
    kept = sorted(keep)
    tr = [q for q in range(n) if q not in kept]
    a = np.transpose(psi.reshape([2] * n), kept + tr).reshape(1 << len(kept), -1)
    ref = a @ a.conj().T
    assert rel_err(got, ref) < 1e-12


def test_state_vector_density_matrix_on_device():
    n = 11
    ops = random_circuit(n, 40, np.random.default_rng(8))
    sv = bs.StateVectorSimulator(n, 0).evolve(ops)
    psi = oracle.OracleSV(n).evolve(ops).psi
    assert rel_err(sv.density_matrix(), np.outer(psi, psi.conj())) < 1e-12
    assert rel_err(bs.calculate(bs.DensityMatrix(()), sv), np.outer(psi, psi.conj())) < 1e-12


def test_density_matrix_keep_all_13_qubits_on_device():
    n = 13
    dm = bs.DensityMatrixSimulator(n, 0)
    dm.evolve([bs.Instruction(bs.H(), [q]) for q in range(n)] + [bs.Instruction(bs.CNot(), [0, 12]),
              bs.Instruction(bs.Depolarizing(0.2), [5]), bs.Instruction(bs.Ry(0.7), [12])])
    assert rel_err(dm.reduced_density_matrix(range(n)), dm.density_matrix) < 1e-13


@pytest.mark.parametrize("kind,n,k,precision", [("sv", 18, 13, "c128"), ("sv", 18, 16, "c128"), ("sv", 17, 17, "c128"),
                                                ("sv", 18, 14, "c64"), ("dm", 13, 13, "c128")])
def test_marginal_probabilities_wide(kind, n, k, precision):
    """Marginals over more than 12 targets on the device (no host fallback) against the oracle's
    probabilities summed over the other qubits."""
    rng = np.random.default_rng(n * 7 + k)
    ops = random_circuit(n, 30 if kind == "sv" else 12, rng)
    if kind == "sv":
        sim = bs.StateVectorSimulator(n, 0, precision=precision).evolve(ops)
        p = np.abs(oracle.OracleSV(n).evolve(ops).psi) ** 2
    else:
        sim = bs.DensityMatrixSimulator(n, 0).evolve(ops)
        p = oracle.OracleDM(n).evolve(ops).probabilities()
    targets = sorted(int(x) for x in rng.choice(n, k, replace=False))
    got = bs.calculate(bs.Probability(tuple(targets)), sim) if k < n else sim.marginal_probabilities(targets)
    traced = tuple(q for q in range(n) if q not in targets)
    ref = p.reshape([2] * n).sum(axis=traced).reshape(-1) if traced else p
    tol = 1e-12 if precision == "c128" else 1e-6
    assert np.max(np.abs(got - ref)) < tol * max(1.0, float(np.max(ref)))


def test_device_partial_trace_complex64():
    n = 12
    rng = np.random.default_rng(3)
    ops = random_circuit(n, 60, rng)
    s64 = bs.StateVectorSimulator(n, 0, precision="c64")
    s64.evolve(ops)
    ref = bs.partial_trace(oracle.OracleSV(n).evolve(ops).psi, [2, 7, 11])
    assert np.max(np.abs(s64.reduced_density_matrix([2, 7, 11]) - ref)) < 1e-5


def test_device_partial_trace_rejects_bad_qubits():
    sim = bs.StateVectorSimulator(5, 0)
    for bad in ([], [5], [1, 1], list(range(13)), [-1]):
        with pytest.raises(bs._abi.BraketGB300Error):
            sim.reduced_density_matrix(bad)
    assert np.allclose(sim.reduced_density_matrix([0]), [[1, 0], [0, 0]])   # the handle stays usable


def test_simulate_circuit_with_basis_rotations():
    """Sampling X, Y, Z eigenstates after the reference's basis rotations gives fixed outcomes."""
    O = bs.observables
    ixs = [bs.Instruction(bs.H(), [0]), bs.Instruction(bs.H(), [1]), bs.Instruction(bs.S(), [1]),
           bs.Instruction(bs.X(), [2])]
    c = bs.Circuit(ixs, [bs.Sample(O.X(), (0,)), bs.Sample(O.Y(), (1,)), bs.Sample(O.Z(), (2,))])
    for sim in (bs.StateVectorSimulator(3, 0), bs.DensityMatrixSimulator(3, 0)):
        res = bs.simulate(sim, c.to_program(200), 200, seed=1)
        m = res["measurements"]
        assert m.shape == (200, 3)
        assert (m[:, 0] == 0).all() and (m[:, 1] == 0).all() and (m[:, 2] == 1).all()


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_result_files_match_host_results(tmp_path, precision):
    """bs_write_result_file streams the state and probability vectors to files whose bytes are the
    host results' bytes (complex128 / float64, as the reference writes them)."""
    n = 12
    sim = bs.StateVectorSimulator(n, 0, precision=precision)
    sim.evolve(random_circuit(n, 60, np.random.default_rng(31)))
    sv, pr = sim.state_vector, sim.probabilities()
    assert sim.write_result_file("state", tmp_path / "sv.bin") == sv.nbytes
    assert sim.write_result_file("probabilities", tmp_path / "p.bin") == pr.nbytes
    assert (tmp_path / "sv.bin").read_bytes() == np.ascontiguousarray(sv, dtype=np.complex128).tobytes()
    assert (tmp_path / "p.bin").read_bytes() == pr.tobytes()
    dm = bs.DensityMatrixSimulator(5, 0, precision=precision)
    dm.evolve(random_circuit(5, 30, np.random.default_rng(32)))
    assert dm.write_result_file("probabilities", tmp_path / "d.bin") == 8 * 32
    assert (tmp_path / "d.bin").read_bytes() == dm.probabilities().tobytes()
    with pytest.raises(bs._abi.BraketGB300Error):
        dm.write_result_file("state", tmp_path / "x.bin")
    with pytest.raises(bs._abi.BraketGB300Error) as e:
        sim.write_result_file("state", tmp_path / "missing-dir" / "x.bin")
    assert e.value.code == bs._abi.BS_ERR_IO


def test_simulate_writes_large_results_to_files(tmp_path):
    """simulate(..., mmap_threshold) leaves values above the threshold empty and returns their files
    (the reference's mmap convention for external callers)."""
    n = 17   # state 2 MiB (to a file), probabilities 1 MiB (kept: not above 1 MiB)
    prog = bs.Program(random_circuit(n, 40, np.random.default_rng(33)), [bs.StateVector(), bs.Probability(()), bs.Probability((0, 1))])
    ref = bs.simulate(bs.StateVectorSimulator(n, 0), prog, 0)
    out = bs.simulate(bs.StateVectorSimulator(n, 0), prog, 0, mmap_threshold=bs.program.MMAP_THRESHOLD,
                      mmap_dir=tmp_path)
    assert out["mmapLengths"] == (1 << n,)
    (path,) = out["mmapPaths"]
    got = np.frombuffer(open(path, "rb").read(), dtype=np.complex128)
    assert np.array_equal(got, ref["resultTypes"][0][1])
    assert out["resultTypes"][0][1].size == 0
    assert np.array_equal(out["resultTypes"][1][1], ref["resultTypes"][1][1])
    assert np.array_equal(out["resultTypes"][2][1], ref["resultTypes"][2][1])
    # threshold 0: every value goes to a file, the small marginal from the host
    out0 = bs.simulate(bs.StateVectorSimulator(n, 0), prog, 0, mmap_threshold=0, mmap_dir=tmp_path)
    assert out0["mmapLengths"] == (1 << n, 1 << n, 4)
    for (rt, v), p, r in zip(out0["resultTypes"], out0["mmapPaths"], ref["resultTypes"]):
        assert v.size == 0
        assert open(p, "rb").read() == np.asarray(r[1]).tobytes()


def _splitmix64(x):
    m = (1 << 64) - 1
    x = (x + 0x9E3779B97F4A7C15) & m
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
    return x ^ (x >> 31)


@pytest.mark.parametrize("kind,n", [("sv", 10), ("sv", 14), ("dm", 5), ("dm", 7)])
def test_own_rng_samples_follow_the_inverse_cdf(kind, n):
    """bs_sample draws u_s = splitmix64(seed ^ splitmix64(s)) / 2^64 and returns the first index whose
    running probability sum reaches u_s * total: the one-launch path for states of one CDF block
    (2^n <= 4096) and the three-kernel path agree with the host inverse CDF (ties aside)."""
    shots, seed = 3000, 12345
    rng = np.random.default_rng(n)
    sim = bs.StateVectorSimulator(n, shots) if kind == "sv" else bs.DensityMatrixSimulator(n, shots)
    sim.evolve(random_circuit(n, 40, rng))
    p = sim.probabilities()
    c = np.cumsum(p)
    u = np.array([(_splitmix64(seed ^ _splitmix64(s)) >> 11) * 2.0 ** -53 for s in range(shots)])
    want = np.minimum(np.searchsorted(c, u * c[-1], side="left"), p.size - 1)
    got = sim.samples(seed=seed)
    assert np.mean(got == want) > 0.999
