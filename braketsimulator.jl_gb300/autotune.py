"""The project's autotuner: chooses the sweep kernels' tile shape and the tensor-core fusion
settings for a simulator size and circuit family by timing candidates on the GPU.

Tunables (per handle, ``bs_set_tuning`` in the C ABI; no reference counterpart, the reference has
no tunable kernels):

* ``tile_bits`` (10..12): amplitude bits per shared-memory tile of the sweep kernels;
* ``tile_threads`` (256 / 512): threads per CTA of the float-float sweep kernel;
* ``tc`` (0 / 1): fused tensor-core sweeps;
* ``tc_min_bits``: vector bits from which fused tensor-core sweeps are used;
* ``tc_cost``: fusion width — a run of gates on at most 5 tile bits becomes one fused unitary when
  its float-float cost (in dense 1-qubit gates) exceeds this;
* ``adj_segments``: adjoint gradients' forward segments (checkpoints of psi + 1); not timed by
  ``autotune`` (it trades memory for accuracy, not speed).

``autotune(sim, instructions)`` re-initialises the simulator, times ``evolve`` of the instructions
(wall clock: host planning included) under each candidate, leaves the fastest set on the handle
and returns it.  Results are cached per (device, simulator kind, precision, qubits, circuit
signature) in memory and, when the environment variable ``BRAKET_GB300_TUNING_CACHE`` names a JSON
file, on disk.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time

from . import _abi

PARAMS = {"tile_bits": _abi.BS_TUNE_TILE_BITS, "tile_threads": _abi.BS_TUNE_TILE_THREADS,
          "tc": _abi.BS_TUNE_TC, "tc_min_bits": _abi.BS_TUNE_TC_MIN_BITS, "tc_cost": _abi.BS_TUNE_TC_COST,
          "adj_segments": _abi.BS_TUNE_ADJ_SEGMENTS}

_CACHE: dict = {}


def get_tuning(sim) -> dict:
    """The values in effect on the simulator's handle."""
    out = {}
    for name, pid in PARAMS.items():
        v = C.c_double()
        sim._h.call("bs_get_tuning", pid, C.byref(v))
        out[name] = v.value if name == "tc_cost" else int(v.value)
    return out


def set_tuning(sim, **values):
    """Set tunables on the handle; None restores the environment / default value."""
    for name, v in values.items():
        if name not in PARAMS:
            raise KeyError(f"unknown tunable {name!r}")
        sim._h.call("bs_set_tuning", PARAMS[name], C.c_double(-1.0 if v is None else float(v)))


def candidates(sim) -> list:
    """Default candidate set for the simulator's kind, precision and size."""
    bits = sim.qubit_count * (2 if sim.kind == _abi.BS_KIND_DM else 1)
    out = []
    if sim.precision == "c128" and bits >= 12:
        # fused tensor-core sweeps at three fusion widths, and the float-float path
        for cost in (1.0, 2.0, 4.0):
            out.append({"tile_bits": 12, "tc": 1, "tc_min_bits": 0, "tc_cost": cost})
        for thr in (256, 512):
            out.append({"tile_bits": 12, "tile_threads": thr, "tc": 0})
    else:
        for tb in [t for t in (10, 11, 12) if t <= max(10, bits)]:
            for thr in (256, 512):
                out.append({"tile_bits": tb, "tile_threads": thr, "tc": 0})
    return out


def signature(instructions) -> tuple:
    """Circuit family key: gate count and the share of multi-qubit and noise instructions, bucketed."""
    n = len(instructions)
    multi = sum(1 for ix in instructions if len(getattr(ix, "target", ())) > 1)
    noise = sum(1 for ix in instructions if type(ix.operator).__module__.endswith("noises"))
    b = lambda x: int(round(8.0 * x / max(1, n)))
    return (n.bit_length(), b(multi), b(noise))


def _device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "unknown"


def _key(sim, instructions) -> str:
    return json.dumps([_device_name(), sim.kind, sim.precision, sim.qubit_count, signature(instructions)])


def _disk_path():
    return os.environ.get("BRAKET_GB300_TUNING_CACHE")


def _load_disk():
    p = _disk_path()
    if p and os.path.exists(p):
        try:
            with open(p) as f:
                _CACHE.update(json.load(f))
        except (OSError, ValueError):
            pass


def _save_disk():
    p = _disk_path()
    if p:
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(_CACHE, f, indent=1, sort_keys=True)
        os.replace(tmp, p)


def autotune(sim, instructions, candidate_list=None, repeats: int = 2, warmup: int = 1, use_cache: bool = True) -> dict:
    """Time ``evolve(instructions)`` under each candidate setting and keep the fastest on ``sim``.

    Re-initialises the simulator (its state is |0...0> afterwards).  Returns the chosen setting with
    its time in seconds and the timings of every candidate (``{"setting": ..., "seconds": ...,
    "timings": [...], "cached": bool}``)."""
    key = _key(sim, instructions)
    if use_cache:
        if not _CACHE:
            _load_disk()
        hit = _CACHE.get(key)
        if hit is not None:
            set_tuning(sim, **hit["setting"])
            return {**hit, "cached": True}
    cands = candidates(sim) if candidate_list is None else list(candidate_list)
    if not cands:
        raise ValueError("no candidate settings")
    n, shots = sim.qubit_count, sim.shots
    timings = []
    for cand in cands:
        set_tuning(sim, **{k: None for k in PARAMS})
        set_tuning(sim, **cand)
        for _ in range(warmup):
            sim.reinit(n, shots)
            sim.evolve(instructions)
        best = float("inf")
        for _ in range(max(1, repeats)):
            sim.reinit(n, shots)
            t0 = time.perf_counter()
            sim.evolve(instructions)
            best = min(best, time.perf_counter() - t0)
        timings.append({"setting": cand, "seconds": best})
    win = min(timings, key=lambda r: r["seconds"])
    set_tuning(sim, **{k: None for k in PARAMS})
    set_tuning(sim, **win["setting"])
    sim.reinit(n, shots)
    rec = {"setting": win["setting"], "seconds": win["seconds"], "timings": timings}
    if use_cache:
        _CACHE[key] = rec
        _save_disk()
    return {**rec, "cached": False}
