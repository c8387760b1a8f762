"""Per-handle tuning and the autotuner: every candidate setting (tile shape, threads, tensor-core
fusion width) gives the oracle's result, and autotune keeps one of them on the handle."""
import numpy as np
import pytest

import oracle
from conftest import bs, random_circuit, rel_err

pytestmark = pytest.mark.gpu
AT = __import__("braketsimulator_gb300.autotune", fromlist=["candidates"])


def test_tuning_round_trip_and_validation():
    sim = bs.StateVectorSimulator(14, 0)
    bs.set_tuning(sim, tile_bits=11, tile_threads=512, tc=0, tc_min_bits=18, tc_cost=3.5)
    assert bs.get_tuning(sim) == {"tile_bits": 11, "tile_threads": 512, "tc": 0, "tc_min_bits": 18, "tc_cost": 3.5,
                                  "adj_segments": -1}
    bs.set_tuning(sim, adj_segments=4)
    assert bs.get_tuning(sim)["adj_segments"] == 4
    bs.set_tuning(sim, tile_bits=None, tile_threads=None, tc=None, tc_min_bits=None, tc_cost=None)
    t = bs.get_tuning(sim)
    assert t["tile_bits"] == 12 and t["tile_threads"] in (256, 512)
    for bad in ({"tile_bits": 9}, {"tile_threads": 384}, {"tc": 2}, {"tile_bits": 11.5}):
        with pytest.raises(bs._abi.BraketGB300Error):
            bs.set_tuning(sim, **bad)
    with pytest.raises(KeyError):
        bs.set_tuning(sim, width=3)


@pytest.mark.parametrize("n,precision,tol", [(13, "c128", 1e-12), (15, "c128", 1e-12), (13, "c64", 2e-5)])
def test_every_candidate_matches_the_oracle(n, precision, tol):
    rng = np.random.default_rng(n)
    ops = random_circuit(n, 120, rng)
    ref = oracle.OracleSV(n).evolve(ops).psi
    sim = bs.StateVectorSimulator(n, 0, precision=precision)
    cands = AT.candidates(sim)
    assert len(cands) >= 4
    for cand in cands:
        bs.set_tuning(sim, tile_bits=None, tile_threads=None, tc=None, tc_min_bits=None, tc_cost=None)
        bs.set_tuning(sim, **cand)
        sim.reinit(n, 0)
        sim.evolve(ops)
        assert rel_err(sim.state_vector, ref) < tol, cand
        if cand.get("tc") == 1:
            assert sim.last_stats()["tc_gates"] > 0


def test_density_matrix_candidates_match_the_oracle():
    n = 6
    rng = np.random.default_rng(4)
    ops = random_circuit(n, 40, rng)
    ops += [bs.Instruction(bs.Depolarizing(0.05), [q]) for q in range(n)]
    ref = oracle.OracleDM(n).evolve(ops).matrix
    sim = bs.DensityMatrixSimulator(n, 0)
    for cand in AT.candidates(sim):
        bs.set_tuning(sim, tile_bits=None, tile_threads=None, tc=None, tc_min_bits=None, tc_cost=None)
        bs.set_tuning(sim, **cand)
        sim.reinit(n, 0)
        sim.evolve(ops)
        assert rel_err(sim.density_matrix, ref) < 1e-12, cand


def test_autotune_keeps_the_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("BRAKET_GB300_TUNING_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(AT, "_CACHE", {})
    n = 16
    rng = np.random.default_rng(2)
    ops = random_circuit(n, 200, rng)
    sim = bs.StateVectorSimulator(n, 0)
    res = bs.autotune(sim, ops, repeats=1)
    assert not res["cached"]
    assert res["setting"] in [t["setting"] for t in res["timings"]]
    assert res["seconds"] == min(t["seconds"] for t in res["timings"])
    now = bs.get_tuning(sim)
    for k, v in res["setting"].items():
        assert now[k] == v
    again = bs.autotune(sim, ops)
    assert again["cached"] and again["setting"] == res["setting"]
    sim.evolve(ops)
    assert rel_err(sim.state_vector, oracle.OracleSV(n).evolve(ops).psi) < 1e-12
