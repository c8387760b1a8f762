"""Benchmark: 30-qubit complex128 state-vector gate layers on one GB300.

Workload (one "step"): the dense random circuit on 30 qubits — 20 layers of a
Haar-random SU(2) on every qubit followed by CZ on an alternating even/odd
brick, then 20 layers of SU(2) on every qubit followed by CZ at (q, q+s mod 30)
with s cycling through 1, 8, 16 — then <Z0 Z29> and 1e5 shots, run from |0...0>
through the public API.  Data are seeded synthetic circuits (no dataset exists).

value   : gate-layer HBM bytes of the workload (2*16*2^30 B per gate: the one pass
          over the state per gate that the reference makes, and that the reference arm
          measures) / device time of the evolution (CUDA events on the launching stream).
          The engine fuses gates, so it executes far fewer sweeps: their bytes per
          second are gate_layer.executed_sweep_GBps, and the dominant kernel's roofline
          (tensor-bound, with its HBM view) is in roofline.
e2e     : the same bytes / wall time of the whole step through the public API
          (circuit upload, evolution, expectation, shots copied to the host).
Side measurement: adjoint gradients of the 24-qubit, 720-parameter ansatz with a
48-term Hamiltonian, against parameter shift on the same GPU.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
LAYERS = 20
SHOTS = 100_000
STRIDES = (1, 8, 16)


def load():
    import __graft_entry__ as ge
    ge.build()
    return ge.load_package()


def haar_su2(rng):
    a = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    q, r = np.linalg.qr(a)
    q = q * (np.diag(r) / np.abs(np.diag(r)))
    return q / np.sqrt(np.linalg.det(q))


def dense_circuit(bs, n=N_QUBITS, layers=LAYERS, seed=0):
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(layers):
        for q in range(n):
            ops.append(bs.Instruction(bs.Unitary(haar_su2(rng)), [q]))
        for q in range(layer % 2, n - 1, 2):
            ops.append(bs.Instruction(bs.CZ(), [q, q + 1]))
    for layer in range(layers):
        s = STRIDES[layer % len(STRIDES)]
        for q in range(n):
            ops.append(bs.Instruction(bs.Unitary(haar_su2(rng)), [q]))
        used = set()
        for q in range(n):
            r = (q + s) % n
            if q in used or r in used:
                continue
            used.update((q, r))
            ops.append(bs.Instruction(bs.CZ(), [q, r]))
    return ops


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    """(HBM GB/s, sustained bf16 TFLOP/s, source): the measured values, else the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops_sustained", 1700.0), "measured"
    return 6800.0, 1700.0, "fallback"


# Tensor-core sweep (k_tile_sweep_tc): executed bf16 MMA work per fused gate per 2^12-amplitude tile
# (26 digit pairs x 4 k-steps, each M=128 N=64 K=16), and the DRAM bytes per amplitude per launch that
# ncu measured for it on the 27-qubit dense circuit (2.1488e9 read + 2.0865e9 written per launch).
TC_FLOP_PER_TILE_GATE = 104 * 2 * 128 * 64 * 16
TC_DRAM_BYTES_PER_AMP = (2.148804e9 + 2.086545e9) / 2 ** 27


def workload_name():
    return f"dense random circuit, {N_QUBITS} qubits, complex128, 2x20 layers, <Z0 Z{N_QUBITS - 1}> + 1e5 shots"


def l2_note():
    gib = 16 * 2 ** N_QUBITS / 2 ** 30
    return f"state ({gib:g} GiB) larger than L2 (129 MB)"


def step(bs, sim, ops, shots, seed):
    """One simulate-style pass through the public API; returns (evolve device ms, stats, result)."""
    sim.reinit(N_QUBITS, shots)
    sim.evolve(ops)
    st = sim.last_stats()
    zz = bs.observables.TensorProduct([bs.observables.Z(), bs.observables.Z()])
    e = sim.expectation(zz, 0, N_QUBITS - 1)
    s = sim.samples(seed)
    return st, e, s


def cpu_baseline_port(seconds_budget=20.0):
    """The oracle (C restatement of the reference's kernels, OpenMP over host cores) on a
    bounded sample of the workload: SU(2) sweeps and CZ sweeps of the 30-qubit state."""
    import oracle
    L = oracle.lib()
    n = N_QUBITS
    psi = np.zeros(2 ** n, dtype=np.complex128)
    psi[0] = 1.0
    rng = np.random.default_rng(1)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    sweeps = 0
    q = 0
    while time.perf_counter() - t0 < seconds_budget and sweeps < 64:
        u = np.ascontiguousarray(haar_su2(rng))
        L.orc_apply_1q(psi.ctypes.data, psi.size, u.ctypes.data, q)
        sweeps += 1
        if sweeps % 3 == 0:
            cz = np.ascontiguousarray(np.diag([1, 1, 1, -1]).astype(np.complex128))
            L.orc_apply_2q(psi.ctypes.data, psi.size, cz.ctypes.data, q, (q + 1) % n)
            sweeps += 1
        q = (q + 7) % n
    dt = time.perf_counter() - t0
    gbs = sweeps * 32.0 * 2 ** n / dt / 1e9
    return {"value": round(gbs, 2), "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{sweeps} reference-kernel gate sweeps (SU(2) and CZ) of the 30-qubit complex128 state, "
                      f"{dt:.1f} s on {cores} OpenMP threads"}, dt


def adjoint_bench(bs, n=24, layers=10, terms=48, shift_params=24, seed=3, ansatz="ry_rz_zz", c64=True):
    """ansatz "ry_rz_zz": per layer Ry(t) Rz(t) on every qubit and a ZZ(t) ring (720 parameters at 24
    qubits, 10 layers); "ry_cz": per layer Ry(t) on every qubit and a fixed CZ ring (240 parameters)."""
    from importlib import import_module
    adj = import_module("braketsimulator_gb300.adjoint")
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(layers):
        for q in range(n):
            ops.append(bs.Instruction(bs.Ry(float(rng.uniform(-np.pi, np.pi))), [q]))
            if ansatz == "ry_rz_zz":
                ops.append(bs.Instruction(bs.Rz(float(rng.uniform(-np.pi, np.pi))), [q]))
        for q in range(n):
            if ansatz == "ry_rz_zz":
                ops.append(bs.Instruction(bs.ZZ(float(rng.uniform(-np.pi, np.pi))), [q, (q + 1) % n]))
            else:
                ops.append(bs.Instruction(bs.CZ(), [q, (q + 1) % n]))
    h = []
    for _ in range(terms):
        w = int(rng.integers(1, 5))
        qs = rng.choice(n, w, replace=False)
        h.append((float(rng.normal()), {int(q): "XYZ"[rng.integers(3)] for q in qs}))
    sim = bs.StateVectorSimulator(n, 0)
    adj.adjoint_gradient(sim, ops, h)            # warm-up
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        e, g = adj.adjoint_gradient(sim, ops, h)
    torch.cuda.synchronize()
    t_adj = (time.perf_counter() - t0) / reps
    # parameter shift on a subset of parameters (cost is linear in the count)
    pidx = adj.parameterised(ops)
    pick = sorted(rng.choice(len(pidx), shift_params, replace=False))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    diffs = []
    for k in pick:
        i = pidx[k]
        ix = ops[i]
        plus = ops[:i] + [adj._with_angle(ix, math.pi / 2)] + ops[i + 1:]
        minus = ops[:i] + [adj._with_angle(ix, -math.pi / 2)] + ops[i + 1:]
        d = (adj.energy(sim, plus, h) - adj.energy(sim, minus, h)) / 2.0
        diffs.append(abs(d - g[k]))
    torch.cuda.synchronize()
    t_ps_per_param = (time.perf_counter() - t0) / shift_params
    P = len(pidx)
    base = {"qubits": n, "params": P, "terms": terms, "energy": e,
            "adjoint_s_per_gradient": round(t_adj, 4), "adjoint_grads_per_s": round(P / t_adj, 1),
            "param_shift_s_per_gradient_extrapolated": round(t_ps_per_param * P, 3),
            "param_shift_grads_per_s": round(1.0 / t_ps_per_param, 2),
            "speedup_vs_param_shift": round(t_ps_per_param * P / t_adj, 1),
            "max_abs_diff_vs_param_shift": float(max(diffs)),
            "param_shift_sample": f"{shift_params} of {P} parameters, 2 circuits each"}
    if not c64:
        return base
    # complex64 variant: same circuit and Hamiltonian on a complex64 state
    sim64 = bs.StateVectorSimulator(n, 0, precision="c64")
    adj.adjoint_gradient(sim64, ops, h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        e64, g64 = adj.adjoint_gradient(sim64, ops, h)
    torch.cuda.synchronize()
    t_adj64 = (time.perf_counter() - t0) / reps
    return {**base,
            "c64": {"adjoint_s_per_gradient": round(t_adj64, 4), "adjoint_grads_per_s": round(P / t_adj64, 1),
                    "max_abs_diff_vs_c128_gradient": float(np.max(np.abs(np.asarray(g64) - np.asarray(g)))),
                    "energy_diff_vs_c128": float(abs(e64 - e))}}


def ghz_bench(bs, reps=100, cpu=False):
    """GHZ-10 (H, CNOT(0,k)), full probabilities and 1000 shots per circuit: latency-bound."""
    import torch
    ops = [bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, 10)]
    sim = bs.StateVectorSimulator(10, 1000)
    for r in range(5):
        sim.reinit(10, 1000)
        sim.evolve(ops)
        sim.probabilities()
        sim.samples(r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in range(reps):
        sim.reinit(10, 1000)
        sim.evolve(ops)
        p = sim.probabilities()
        s = sim.samples(r)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    ok = abs(p[0] - 0.5) < 1e-15 and abs(p[-1] - 0.5) < 1e-15 and set(np.unique(s)) <= {0, 1023}
    out = {"us_per_circuit": round(dt * 1e6, 1), "circuits_per_s": round(1 / dt, 1), "checked": bool(ok)}
    if cpu:
        out["cpu_baseline"] = ghz_cpu_port(reps)
    return out


def ghz_cpu_port(reps=200):
    """The same GHZ-10 flow on the oracle port of the reference's CPU kernels, one host thread:
    H and nine CNOT sweeps, |psi|^2, the serial alias table and 1000 draws on a host stream."""
    import oracle
    L = oracle.lib()
    h = oracle._cm(oracle.FIXED["h"])
    x = oracle._cm(oracle.FIXED["x"])
    rng = np.random.default_rng(0)
    psi = np.zeros(1024, dtype=np.complex128)

    def one():
        psi[:] = 0
        psi[0] = 1
        L.orc_apply_1q(oracle._p(psi), 1024, oracle._p(h), 0)
        for k in range(1, 10):
            L.orc_apply_c1t1(oracle._p(psi), 1024, oracle._p(x), 1, 0, k)
        p = np.abs(psi) ** 2
        ap, al = oracle.alias_table(p)
        j = rng.integers(0, 1024, 1000)
        u = rng.random(1000)
        return oracle.sample_alias(ap, al, j, u)

    for _ in range(10):
        one()
    t0 = time.perf_counter()
    for _ in range(reps):
        s = one()
    dt = (time.perf_counter() - t0) / reps
    assert set(np.unique(s)) <= {0, 1023}
    return {"us_per_circuit": round(dt * 1e6, 1), "cores": 1, "kind": "port",
            "sample": f"{reps} circuits: the oracle's C kernels through ctypes, numpy |psi|^2 and RNG"}


def dm_circuit(bs, n=14, depth=12, seed=5):
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(depth):
        for q in range(n):
            g = [bs.Rx, bs.Ry, bs.Rz][rng.integers(3)](float(rng.uniform(0, 2 * np.pi)))
            ops += [bs.Instruction(g, [q]), bs.Instruction(bs.Depolarizing(1e-3), [q]),
                    bs.Instruction(bs.AmplitudeDamping(5e-3), [q])]
        for q in range(n - 1):
            ops += [bs.Instruction(bs.CNot(), [q, q + 1]), bs.Instruction(bs.TwoQubitDepolarizing(1e-2), [q, q + 1]),
                    bs.Instruction(bs.AmplitudeDamping(5e-3), [q]), bs.Instruction(bs.AmplitudeDamping(5e-3), [q + 1])]
    return ops


def dm_bench(bs, n=14, cpu=False):
    """Noisy density matrix, 14 qubits (4 GiB): diag + <X X X X> on qubits 0..3, both noise modes."""
    import torch
    ops = dm_circuit(bs, n)
    x4 = bs.observables.TensorProduct([bs.observables.X()] * 4)
    out = {}
    for mode in ("reference", "physical"):
        sim = bs.DensityMatrixSimulator(n, 0, noise_mode=mode)
        sim.evolve(ops)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.reinit(n, 0)
        sim.evolve(ops)
        st = sim.last_stats()
        diag = sim.probabilities()
        ex = sim.expectation(x4, 0, 1, 2, 3)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[mode] = {"s_per_circuit": round(dt, 3), "evolve_gpu_ms": round(st["gpu_ms"], 1), "sweeps": st["sweeps"],
                     "sweep_GBps": round(st["bytes_moved"] / (st["gpu_ms"] * 1e-3) / 1e9, 1),
                     "trace": round(float(np.sum(diag)), 12), "x4": ex}
    out["instructions"] = len(ops)
    if cpu:
        out["cpu_baseline"] = dm_cpu_port(ops, n)
    return out


def dm_cpu_port(ops, n=14, depth=12):
    """Reference noise mode on the oracle port of the reference's CPU kernels (all host threads):
    the first of the circuit's `depth` identical-shape layers is timed and scaled by `depth`."""
    import oracle
    oracle.lib()
    layer = len(ops) // depth
    sim = oracle.OracleDM(n)
    sim.rho[:] = 0
    sim.rho[0] = 1.0
    t0 = time.perf_counter()
    sim.evolve(ops[:layer])
    dt = time.perf_counter() - t0
    return {"s_per_circuit": round(dt * depth, 2), "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 of {depth} layers ({layer} instructions, {dt:.1f} s) timed, scaled by {depth}"}


def batch_circuits(bs, nc=512, seed=7):
    """512 circuits: qubits U{12..26}, depth U{10..60} layers of ceil(n/2) gates from
    {H, Rx, Ry, Rz, CNOT, CZ, Swap, CCNot} on seeded random qubits; 8 Pauli strings each."""
    rng = np.random.default_rng(seed)
    circuits, counts, obs = [], [], []
    for _ in range(nc):
        n = int(rng.integers(12, 27))
        depth = int(rng.integers(10, 61))
        ins = []
        for _ in range(depth * ((n + 1) // 2)):
            r = int(rng.integers(8))
            q = [int(x) for x in rng.choice(n, 3, replace=False)]
            if r == 0:
                ins.append(bs.Instruction(bs.H(), [q[0]]))
            elif r in (1, 2, 3):
                ins.append(bs.Instruction([bs.Rx, bs.Ry, bs.Rz][r - 1](float(rng.uniform(-np.pi, np.pi))), [q[0]]))
            elif r == 4:
                ins.append(bs.Instruction(bs.CNot(), q[:2]))
            elif r == 5:
                ins.append(bs.Instruction(bs.CZ(), q[:2]))
            elif r == 6:
                ins.append(bs.Instruction(bs.Swap(), q[:2]))
            else:
                ins.append(bs.Instruction(bs.CCNot(), q))
        terms = [{int(t): "XYZ"[rng.integers(3)] for t in rng.choice(n, int(rng.integers(1, 5)), replace=False)}
                 for _ in range(8)]
        circuits.append(ins)
        counts.append(n)
        obs.append(terms)
    return circuits, counts, obs


def batch_bench(bs, cpu=False):
    import torch
    circuits, counts, obs = batch_circuits(bs)
    bs.batch_simulate(circuits[:8], counts[:8], obs[:8], shots=1000, seed=1)      # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    exp, smp, st = bs.batch_simulate(circuits, counts, obs, shots=1000, seed=2, precision="c64")
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    # error of the complex64 run against complex128 on a few circuits (the smallest ones)
    small = sorted(range(len(counts)), key=lambda c: counts[c])[:4]
    e128, _, _ = bs.batch_simulate([circuits[c] for c in small], [counts[c] for c in small], [obs[c] for c in small],
                                   shots=0, precision="c128")
    err = float(np.max(np.abs(exp[small] - e128)))
    # the same batch captured once into a CUDA graph, then replayed (host work per replay: one
    # graph launch and the result copies)
    t0 = time.perf_counter()
    cb = bs.CapturedBatch(circuits, counts, obs, shots=1000, seed=2, precision="c64")
    t_cap = time.perf_counter() - t0
    cb.launch()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        exp2, _, st2 = cb.launch()
    t_rep = (time.perf_counter() - t0) / reps
    same = bool(np.array_equal(exp, exp2))
    cb.close()
    return {"circuits": len(circuits), "qubits": "12..26", "gates": int(sum(len(c) for c in circuits)),
            "shots_each": 1000, "expectations_each": 8, "precision": "c64 (FP64 reductions)",
            "s_per_batch": round(dt, 3), "circuits_per_s": round(len(circuits) / dt, 1),
            "device_ms": round(st["gpu_ms"], 1), "sweeps": st["sweeps"],
            "max_abs_err_c64_vs_c128_expectations": err,
            "graph": {"capture_s": round(t_cap, 3), "s_per_replay": round(t_rep, 3),
                      "circuits_per_s": round(len(circuits) / t_rep, 1), "device_ms": round(st2["gpu_ms"], 1),
                      "replay_equals_one_shot": same},
            **({"cpu_baseline": batch_cpu_port(circuits, counts)} if cpu else {})}


def batch_cpu_port(circuits, counts, budget_s=8.0):
    """The batch's gate sweeps on the oracle port of the reference's CPU kernels (complex128, all host
    threads; the reference has no complex64 path): circuits in batch order are evolved until the
    budget is spent, and the whole batch's time is scaled from the sample by gate-sweep bytes."""
    import oracle
    oracle.lib()
    total = sum(len(c) * 32.0 * 2 ** n for c, n in zip(circuits, counts))
    done_bytes, t_used, k = 0.0, 0.0, 0
    for c, n in zip(circuits, counts):
        if t_used > budget_s or n > 24:
            continue
        sim = oracle.OracleSV(n)
        t0 = time.perf_counter()
        sim.evolve(c)
        t_used += time.perf_counter() - t0
        done_bytes += len(c) * 32.0 * 2 ** n
        k += 1
    est = total / (done_bytes / t_used)
    return {"circuits_per_s": round(len(circuits) / est, 2), "s_per_batch": round(est, 1), "cores": os.cpu_count(),
            "kind": "port", "sample": f"{k} circuits of <=24 qubits evolved in {t_used:.1f} s; the batch scaled by "
                                      "gate-sweep bytes (2*16*2^n per gate); shots and expectations not included"}


def max_over_ranks(vals, world, device="cuda"):
    """The timed quantities' maximum over the replicas (one all_reduce; as is for one rank).  Each
    rank runs its own full workload, so the whole-job rate is the units of all ranks over this time."""
    if world <= 1:
        return [float(v) for v in vals]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in vals], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU kernels (oracle port; Julia is not installed)
    on the host cores, bounded sample of the same workload per step."""
    if rank != 0:
        return
    import oracle
    oracle.lib()
    vals = []
    for i in range(args.warmup + args.steps):
        res, dt = cpu_baseline_port(seconds_budget=8.0)
        if i >= args.warmup:
            vals.append((res, dt))
    v = float(np.mean([r["value"] for r, _ in vals]))
    line = {"impl": "reference", "metric": "30q SV gate-layer HBM GB/s", "value": round(v, 2), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * float(np.mean([dt for _, dt in vals])), 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64)", "data": "synthetic",
            "config": {"workload": workload_name(),
                       "qubits": N_QUBITS, "shots": SHOTS,
                       "bytes": "gate-layer bytes: 2*16*2^n per gate (one pass per gate, as the reference runs)",
                       "sample": "each step times a bounded run of the workload's gate sweeps (SU(2) and CZ "
                                 "passes of the reference kernels); GB/s per gate pass is the same unit"},
            "cpu_baseline": {**vals[-1][0], "value": round(v, 2)},
            "e2e": {"value": round(v, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--qubits", type=int, default=N_QUBITS, help="smaller cases for profiling")
    ap.add_argument("--precision", default="c128", choices=["c128", "c64"])
    args = ap.parse_args()
    globals()["N_QUBITS"] = args.qubits
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    bs = load()
    ops = dense_circuit(bs, n=N_QUBITS)
    sim = bs.StateVectorSimulator(N_QUBITS, SHOTS, precision=args.precision)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for i in range(args.warmup):
        step(bs, sim, ops, SHOTS, 100 + i)
    barrier()
    dev_ms, bytes_moved, sweeps, launches, tc_gates, tc_ms, tc_launches = 0.0, 0.0, 0, 0, 0, 0.0, 0
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            st, e, s = step(bs, sim, ops, SHOTS, 1000 + i)
            dev_ms += st["gpu_ms"]
            bytes_moved += st["bytes_moved"]
            sweeps += st["sweeps"]
            launches += st["kernel_launches"]
            tc_gates += st["tc_gates"]
            tc_ms += st["tc_ms"]
            tc_launches += st["tc_launches"]
        barrier()
        wall = time.perf_counter() - t0
    wall, dev_ms = max_over_ranks([wall, dev_ms], world)
    if rank != 0:
        return
    hbm, bf16, src = peaks()
    sweep_bytes = 32.0 * 2 ** N_QUBITS            # algorithmic HBM bytes of one sweep (read + write)
    if tc_launches:
        # dominant kernel: the tensor-core sweep, timed by the library with CUDA events around each launch
        tc_launch_s = tc_ms * 1e-3 / tc_launches
        flop_per_launch = tc_gates * 2 ** (N_QUBITS - 12) * TC_FLOP_PER_TILE_GATE / tc_launches
        tflops = flop_per_launch / tc_launch_s / 1e12
        hbm_gbs = sweep_bytes / tc_launch_s / 1e9
        roofline = {"bound": "tensor", "achieved": round(tflops, 1), "peak": bf16, "unit": "TFLOP/s",
                    "frac": round(tflops / bf16, 3), "traffic": round(TC_DRAM_BYTES_PER_AMP * 2 ** N_QUBITS),
                    "peak_source": f"{src} (bf16 sustained)", "kernel": "k_tile_sweep_tc",
                    "flop_per_launch": flop_per_launch, "launch_ms": round(tc_launch_s * 1e3, 2),
                    "launches_per_step": tc_launches // args.steps,
                    "hbm_view": {"achieved": round(hbm_gbs, 1), "peak": hbm, "unit": "GB/s",
                                 "frac": round(hbm_gbs / hbm, 3), "bytes_per_launch": sweep_bytes}}
    else:
        per_launch_ms = dev_ms / max(1, sweeps)
        achieved = sweep_bytes / (per_launch_ms * 1e-3) / 1e9
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved / hbm, 3), "traffic": None, "peak_source": src,
                    "kernel": "k_tile_sweep", "bytes_per_launch": sweep_bytes}
    # value: the workload's gate-layer bytes (2*16*2^n per gate: the one pass per gate the reference
    # makes) over the device time, so that it compares with the reference arm's number for the same
    # circuit; the bytes of the sweeps actually executed (fused) are in gate_layer / roofline
    n_gates = sum(1 for _ in ops)
    workload_bytes = n_gates * sweep_bytes * args.steps
    value = workload_bytes / (dev_ms * 1e-3) / 1e9 * world
    e2e = workload_bytes / wall / 1e9 * world
    executed = bytes_moved / (dev_ms * 1e-3) / 1e9
    line = {
        "metric": "30q SV gate-layer HBM GB/s", "value": round(value, 1), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * wall / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 state, float-float (FP32-pipe) arithmetic", "data": "synthetic (seeded Haar SU(2) + CZ)",
        "config": {"workload": workload_name(),
                   "qubits": N_QUBITS, "gates": n_gates, "shots": SHOTS,
                   "bytes": "gate-layer bytes: 2*16*2^n per gate (one pass per gate, as the reference runs)",
                   "l2": l2_note(), "parallelism": "replicas" if world > 1 else "1 GPU"},
        "e2e": {"value": round(e2e, 1), "unit": "GB/s", "h2d_bytes_per_step": int(n_gates * 64 + 200 * n_gates),
                "d2h_bytes_per_step": int(SHOTS * 8 + 8)},
        "roofline": roofline,
        "gate_layer": {"sweeps_per_step": sweeps // args.steps, "gates_per_step": n_gates,
                       "tensor_core_fused_unitaries_per_step": tc_gates // args.steps,
                       "executed_sweep_GBps": round(executed, 1),
                       "layer_ms": round(dev_ms / args.steps / (2 * LAYERS), 2)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        line["cpu_baseline"], _ = cpu_baseline_port()
    if not args.no_adjoint:
        line["adjoint"] = adjoint_bench(bs)
        line["adjoint240"] = adjoint_bench(bs, ansatz="ry_cz", c64=False)   # the 240-parameter ansatz
        line["ghz10"] = ghz_bench(bs, cpu=not args.no_cpu)
        line["dm14"] = dm_bench(bs, cpu=not args.no_cpu)
        line["batch512"] = batch_bench(bs, cpu=not args.no_cpu)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
