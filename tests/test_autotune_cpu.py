"""Autotuner host logic: candidate sets, circuit signatures, the on-disk cache (no GPU)."""
import json
import types

import pytest

from conftest import bs

at = pytest.importorskip("braketsimulator_gb300.autotune")


def fake_sim(n, kind=0, precision="c128"):
    return types.SimpleNamespace(qubit_count=n, kind=kind, precision=precision, shots=0)


def test_candidates_cover_tensor_core_and_float_float_paths():
    c = at.candidates(fake_sim(20))
    assert {x["tc"] for x in c} == {0, 1}
    assert sorted({x["tc_cost"] for x in c if x["tc"] == 1}) == [1.0, 2.0, 4.0]
    assert {x.get("tile_threads") for x in c if x["tc"] == 0} == {256, 512}


def test_candidates_complex64_and_small_states_vary_tile_shape():
    c = at.candidates(fake_sim(16, precision="c64"))
    assert all(x["tc"] == 0 for x in c)
    assert {x["tile_bits"] for x in c} == {10, 11, 12}
    small = at.candidates(fake_sim(6))
    assert {x["tile_bits"] for x in small} == {10}


def test_signature_buckets_gate_mix():
    ops1 = [bs.Instruction(bs.H(), [0])] * 10 + [bs.Instruction(bs.CNot(), [0, 1])] * 10
    ops2 = [bs.Instruction(bs.H(), [1])] * 11 + [bs.Instruction(bs.CZ(), [1, 2])] * 9
    ops3 = [bs.Instruction(bs.H(), [0])] * 20
    assert at.signature(ops1) == at.signature(ops2)
    assert at.signature(ops1) != at.signature(ops3)


def test_disk_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tuning.json"
    monkeypatch.setenv("BRAKET_GB300_TUNING_CACHE", str(path))
    monkeypatch.setattr(at, "_CACHE", {"k": {"setting": {"tc": 1, "tc_cost": 2.0}, "seconds": 0.5, "timings": []}})
    at._save_disk()
    assert json.loads(path.read_text())["k"]["setting"]["tc_cost"] == 2.0
    monkeypatch.setattr(at, "_CACHE", {})
    at._load_disk()
    assert at._CACHE["k"]["seconds"] == 0.5
