"""Batched uneven circuits: one persistent launch for the small ones, stream pool for the rest."""
import numpy as np
import pytest

import oracle
from conftest import bs

pytestmark = pytest.mark.gpu


def random_batch(nc, nmin, nmax, rng, depth=(5, 15)):
    circuits, counts, obs = [], [], []
    for _ in range(nc):
        n = int(rng.integers(nmin, nmax + 1))
        ins = []
        for _ in range(int(rng.integers(*depth)) * max(1, n // 2)):
            r = int(rng.integers(8))
            q = [int(x) for x in rng.choice(n, min(n, 3), replace=False)]
            if r == 0 or n < 2:
                ins.append(bs.Instruction(bs.H(), [q[0]]))
            elif r in (1, 2, 3):
                ins.append(bs.Instruction([bs.Rx, bs.Ry, bs.Rz][r - 1](float(rng.uniform(-np.pi, np.pi))), [q[0]]))
            elif r == 4:
                ins.append(bs.Instruction(bs.CNot(), q[:2]))
            elif r == 5:
                ins.append(bs.Instruction(bs.CZ(), q[:2]))
            elif r == 6:
                ins.append(bs.Instruction(bs.Swap(), q[:2]))
            elif n >= 3:
                ins.append(bs.Instruction(bs.CCNot(), q[:3]))
        terms = [{int(t): "XYZ"[rng.integers(3)] for t in rng.choice(n, min(n, int(rng.integers(1, 4))), replace=False)}
                 for _ in range(4)]
        circuits.append(ins)
        counts.append(n)
        obs.append(terms)
    return circuits, counts, obs


def exact(ins, n, terms):
    psi = oracle.OracleSV(n).evolve(ins).psi
    out = []
    for t in terms:
        x = sum(1 << q for q, p in t.items() if p in "XY")
        z = sum(1 << q for q, p in t.items() if p in "YZ")
        out.append(oracle.expectation_pauli_sv(psi, n, x, z))
    return np.array(out), np.abs(psi) ** 2


@pytest.mark.parametrize("precision,tol", [("c64", 2e-5), ("c128", 1e-12)])
def test_batch_expectations_and_samples(precision, tol):
    rng = np.random.default_rng(11)
    circuits, counts, obs = random_batch(40, 2, 16, rng)
    shots = 4000
    exp, smp, st = bs.batch_simulate(circuits, counts, obs, shots=shots, seed=5, precision=precision)
    assert exp.shape == (40, 4) and smp.shape == (40, shots)
    for c in range(40):
        e, p = exact(circuits[c], counts[c], obs[c])
        assert np.max(np.abs(exp[c] - e)) < tol, (c, counts[c])
        assert np.all(p[smp[c]] > 1e-12)          # every shot lands on a populated basis state
        # <Z_0> from the samples agrees with the exact value within 6 sigma
        n = counts[c]
        z0 = 1.0 - 2.0 * ((smp[c] >> (n - 1)) & 1)
        exact_z0 = float(np.sum(p * (1.0 - 2.0 * ((np.arange(2 ** n) >> (n - 1)) & 1))))
        assert abs(z0.mean() - exact_z0) < 6.0 / np.sqrt(shots) + 1e-9


def test_batch_small_circuits_share_one_launch():
    rng = np.random.default_rng(3)
    circuits, counts, obs = random_batch(64, 3, 12, rng)
    exp, smp, st = bs.batch_simulate(circuits, counts, obs, shots=100, seed=1, precision="c64")
    assert st["kernel_launches"] == 1
    for c in range(64):
        e, _ = exact(circuits[c], counts[c], obs[c])
        assert np.max(np.abs(exp[c] - e)) < 2e-5


def rebind_angles(circuits, rng):
    """Same gate sequence, new rotation angles (a parameter sweep)."""
    out = []
    for ins in circuits:
        new = []
        for ix in ins:
            op = ix.operator
            if isinstance(op, (bs.Rx, bs.Ry, bs.Rz)):
                op = type(op)(float(rng.uniform(-np.pi, np.pi)))
            new.append(bs.Instruction(op, list(ix.target)))
        out.append(new)
    return out


@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_captured_batch_replays_the_one_shot_results(precision):
    rng = np.random.default_rng(21)
    circuits, counts, obs = random_batch(24, 3, 16, rng)
    shots = 500
    exp1, smp1, _ = bs.batch_simulate(circuits, counts, obs, shots=shots, seed=9, precision=precision)
    with bs.CapturedBatch(circuits, counts, obs, shots=shots, seed=9, precision=precision) as cb:
        for _ in range(3):
            exp2, smp2, st = cb.launch()
            # the same kernels on the same inputs: identical expectations and shots
            assert np.array_equal(exp1, exp2)
            assert np.array_equal(smp1, smp2)
            assert st["gpu_ms"] > 0


def test_captured_batch_parameter_update():
    rng = np.random.default_rng(5)
    circuits, counts, obs = random_batch(20, 2, 15, rng)
    with bs.CapturedBatch(circuits, counts, obs, shots=64, seed=2, precision="c128") as cb:
        for _ in range(2):
            circuits = rebind_angles(circuits, rng)
            cb.set_circuits(circuits)
            exp, smp, _ = cb.launch()
            ref, _, _ = bs.batch_simulate(circuits, counts, obs, shots=64, seed=2, precision="c128")
            assert np.array_equal(exp, ref)
            for c in range(len(circuits)):
                e, _ = exact(circuits[c], counts[c], obs[c])
                assert np.max(np.abs(exp[c] - e)) < 1e-12


def test_captured_batch_rejects_a_change_of_path():
    rng = np.random.default_rng(8)
    circuits, counts, obs = random_batch(6, 3, 8, rng)
    with bs.CapturedBatch(circuits, counts, obs, shots=0, seed=0, precision="c64") as cb:
        changed = [list(ins) for ins in circuits]
        # a 2-qubit dense gate moves a small circuit from the one-CTA kernel to the tile path
        changed[0].append(bs.Instruction(bs.XX(0.3), [0, 1]))
        with pytest.raises(bs._abi.BraketGB300Error):
            cb.set_circuits(changed)
        exp, _, _ = cb.launch()   # the batch is still usable
        ref, _, _ = bs.batch_simulate(circuits, counts, obs, shots=0, seed=0, precision="c64")
        assert np.array_equal(exp, ref)


def test_captured_batch_autotune_keeps_results():
    rng = np.random.default_rng(31)
    circuits, counts, obs = random_batch(12, 10, 16, rng)
    ref, smp_ref, _ = bs.batch_simulate(circuits, counts, obs, shots=200, seed=4, precision="c128")
    with bs.CapturedBatch(circuits, counts, obs, shots=200, seed=4, precision="c128") as cb:
        res = cb.autotune(repeats=1)
        assert res["setting"] in [t["setting"] for t in res["timings"]]
        exp, smp, _ = cb.launch()
        # every tuning computes the same state to 1e-12; shots may differ only at exact CDF ties
        assert np.max(np.abs(exp - ref)) < 1e-11
        assert np.mean(smp == smp_ref) > 0.99
