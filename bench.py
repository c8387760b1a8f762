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


def dense_circuit(bs, n=N_QUBITS, layers=LAYERS, seed=0, layers2=None, two_qubit="cz"):
    """The dense random circuit: `layers` layers of Haar SU(2) on every qubit and a 2-qubit gate on
    an alternating even/odd brick, then `layers2` (default `layers`) layers of SU(2) on every qubit
    and the 2-qubit gate at (q, q+s mod n), s cycling through 1, 8, 16.  two_qubit: "cz" (the
    headline workload) or "cnot" (a dense 2-qubit gate that fusion cannot fold into a phase)."""
    rng = np.random.default_rng(seed)
    gate = {"cz": bs.CZ, "cnot": bs.CNot}[two_qubit]
    ops = []
    for layer in range(layers):
        for q in range(n):
            ops.append(bs.Instruction(bs.Unitary(haar_su2(rng)), [q]))
        for q in range(layer % 2, n - 1, 2):
            ops.append(bs.Instruction(gate(), [q, q + 1]))
    for layer in range(layers if layers2 is None else layers2):
        s = STRIDES[layer % len(STRIDES)]
        for q in range(n):
            ops.append(bs.Instruction(bs.Unitary(haar_su2(rng)), [q]))
        used = set()
        for q in range(n):
            r = (q + s) % n
            if q in used or r in used:
                continue
            used.update((q, r))
            ops.append(bs.Instruction(gate(), [q, r]))
    return ops


def inverse_circuit(bs, ops):
    """The circuit's inverse: reversed order, each SU(2) daggered (CZ and CNOT are involutions)."""
    out = []
    for ix in reversed(ops):
        g = ix.operator
        if isinstance(g, bs.Unitary):
            out.append(bs.Instruction(bs.Unitary(np.conj(np.asarray(g.matrix)).T), list(ix.target)))
        else:
            out.append(bs.Instruction(type(g)(), list(ix.target)))
    return out


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


class ReferenceSampler:
    """The reference's CPU path for the headline workload, on the oracle port of its kernels
    (Julia is not installed: C restatements of src/gate_kernels.jl, OpenMP over the host cores
    as the reference's Threads.@threads), timed on bounded samples and extrapolated to a step.

    One step of the workload on the reference path is
      evolve!:       each of the circuit's instructions through the reference's dispatch (SU(2)
                     as a 1-qubit dense sweep, CZ as the 1-control-1-target kernel that touches
                     half of the amplitudes, src/gate_kernels.jl:489-537,579-606,720-732);
      expectation:   <Z0 Z29> = real(dot(psi, apply_observable(Z Z, copy(psi)))), a deep copy, two
                     Z sweeps and a dot (src/sv_simulator.jl:240-248);
      probabilities: abs2 of the state and the pairwise sum of Weights (src/result_types.jl:56-58);
      1e5 shots:     at 30 qubits the reference draws every shot by StatsBase's linear scan of the
                     running sum (src/result_types.jl:73-77), about 2^29 weights per shot for the
                     circuit's flat (Porter-Thomas) output distribution.
    Each sample evolves the next contiguous slice of the instruction list on a persistent 30-qubit
    oracle state (so over the steps the oracle runs the circuit from its start), and times one of
    the other three parts in rotation; the step estimate is n_SU(2) * t_SU(2) + n_CZ * t_CZ +
    t_expectation + t_probabilities + 1e5 * t_shot from the running means."""

    def __init__(self, bs, ops):
        import oracle
        self.oracle = oracle
        oracle.lib()
        self.ops = ops
        self.unitary = bs.Unitary
        self.n_su2 = sum(1 for ix in ops if isinstance(ix.operator, bs.Unitary))
        self.n_2q = len(ops) - self.n_su2
        self.sv = oracle.OracleSV(N_QUBITS)
        self.cursor = 0
        self.t = {"su2": [], "2q": [], "expectation": [], "probabilities": [], "shot": []}
        self.flat = None
        self.part = 0
        self.cores = os.cpu_count() or 1

    def _time(self, key, fn):
        t0 = time.perf_counter()
        r = fn()
        self.t[key].append(time.perf_counter() - t0)
        return r

    def expectation(self):
        zz = (1 << 0) | (1 << (N_QUBITS - 1))
        self._time("expectation", lambda: self.oracle.expectation_pauli_sv(self.sv.psi, N_QUBITS, 0, zz))

    def probabilities(self):
        self._time("probabilities", lambda: self.oracle.pairwise_sum(np.abs(self.sv.psi) ** 2))

    def shot(self):
        if N_QUBITS >= 30:
            # one draw at u = 1/2 on a flat weight vector: the scan covers half of the 2^n weights,
            # the mean over uniform draws for a flat cumulative distribution
            if self.flat is None:
                self.flat = np.full(2 ** N_QUBITS, 2.0 ** -N_QUBITS)
            self._time("shot", lambda: self.oracle.sample_direct(self.flat, np.array([0.5]), 1.0))
        else:
            # below 30 qubits the reference builds the alias table and draws from it
            # (src/result_types.jl:62-72): its cost per step, spread over the shots
            p = np.abs(self.sv.psi) ** 2
            rng = np.random.default_rng(0)

            def draw():
                ap, al = self.oracle.alias_table(p)
                self.oracle.sample_alias(ap, al, rng.integers(0, p.size, SHOTS), rng.random(SHOTS))

            t0 = time.perf_counter()
            draw()
            self.t["shot"].append((time.perf_counter() - t0) / SHOTS)

    def sample(self, n_gates=8, parts=None):
        """Evolve the next n_gates instructions; time the parts named (default: the next in rotation)."""
        for _ in range(n_gates):
            ix = self.ops[self.cursor]
            self._time("su2" if isinstance(ix.operator, self.unitary) else "2q", lambda: self.sv.evolve([ix]))
            self.cursor = (self.cursor + 1) % len(self.ops)
            if self.cursor == 0:
                self.sv = self.oracle.OracleSV(N_QUBITS)
        rot = ("expectation", "probabilities", "shot")
        if parts is None:
            parts = [rot[self.part % 3]]
            self.part += 1
        for p in parts:
            getattr(self, p)()

    def estimate(self):
        """Seconds per step of the whole workload on the reference path, and its parts."""
        m = {k: (float(np.mean(v)) if v else float("nan")) for k, v in self.t.items()}
        parts = {"evolve": self.n_su2 * m["su2"] + self.n_2q * m["2q"], "expectation": m["expectation"],
                 "probabilities": m["probabilities"], "shots": SHOTS * m["shot"]}
        return sum(parts.values()), parts

    def describe(self):
        c = {k: len(v) for k, v in self.t.items()}
        return (f"oracle port of the reference kernels on {self.cores} OpenMP threads: {c['su2']} SU(2) and {c['2q']} "
                f"CZ instructions of the workload timed one by one through the reference dispatch, "
                f"{c['expectation']} <Z0 Z{N_QUBITS - 1}> evaluations, {c['probabilities']} probability passes and "
                f"{c['shot']} " + (f"direct-sampling scans (2^{N_QUBITS - 1} weights each)" if N_QUBITS >= 30 else
                                   f"alias-table builds with {SHOTS} draws") +
                f" of the {N_QUBITS}-qubit state; the step "
                f"({self.n_su2} SU(2) + {self.n_2q} CZ, <Z0 Z{N_QUBITS - 1}>, probabilities, {SHOTS} shots) "
                f"extrapolated from "
                f"their means")


def headline_check(bs, sim, ops, zz):
    """Checks of the benchmarked 30-qubit result itself, after the timed region (the FP64 oracle
    runs this circuit in the test suite at 28 qubits and a shortened one at 30; at full size it
    would take minutes of host time):
      mirror: the inverse circuit applied to the benchmarked state must give back |0...0>;
      paths:  <Z0 Z29> from the tensor-core sweeps against the float-float sweeps alone (BS_TC off),
              two independent arithmetic paths of the engine on the same circuit."""
    sim.evolve(inverse_circuit(bs, ops))
    psi = sim.state_vector
    mirror = float(np.sqrt(abs(psi[0] - 1.0) ** 2 + np.vdot(psi[1:], psi[1:]).real))
    del psi
    ff = bs.StateVectorSimulator(N_QUBITS, 0)
    bs.set_tuning(ff, tc=0)
    ff.evolve(ops)
    zz_ff = ff.expectation(bs.observables.TensorProduct([bs.observables.Z(), bs.observables.Z()]), 0, N_QUBITS - 1)
    del ff
    return {"zz": zz, "zz_float_float_path": zz_ff, "zz_abs_diff": abs(zz - zz_ff),
            "mirror_err": mirror, "tol": 1e-12, "checked": bool(mirror < 1e-12 and abs(zz - zz_ff) < 1e-12)}


def dense_cnot_bench(bs, reps=2):
    """Side measurement: the same 30-qubit circuit with CNOT in place of CZ, a dense 2-qubit gate
    that fusion cannot fold into a parity phase (strides 8 and 16 included), timed like the headline
    evolution, with the mirror check (the inverse circuit gives back |0...0>)."""
    import torch
    ops = dense_circuit(bs, n=N_QUBITS, two_qubit="cnot")
    sim = bs.StateVectorSimulator(N_QUBITS, 0)
    sim.evolve(ops)
    torch.cuda.synchronize()
    ms, st = [], None
    for _ in range(reps):
        sim.reinit(N_QUBITS, 0)
        sim.evolve(ops)
        st = sim.last_stats()
        ms.append(st["gpu_ms"])
    hbm, _, _ = peaks()
    sweep_bytes = 32.0 * 2 ** N_QUBITS
    dev = float(np.median(ms))
    out = {"gates": len(ops), "evolve_ms": round(dev, 1), "sweeps": st["sweeps"],
           "tensor_core_fused_unitaries": st["tc_gates"], "gate_layer_GBps": round(len(ops) * sweep_bytes / dev / 1e6, 1),
           "executed_sweep_GBps": round(st["bytes_moved"] / dev / 1e6, 1)}
    if st["tc_launches"]:
        launch_s = st["tc_ms"] * 1e-3 / st["tc_launches"]
        out["k_tile_sweep_tc"] = {"launch_ms": round(launch_s * 1e3, 2), "launches": st["tc_launches"],
                                  "hbm_frac": round(sweep_bytes / launch_s / 1e9 / hbm, 3)}
    sim.evolve(inverse_circuit(bs, ops))
    psi = sim.state_vector
    out["mirror_err"] = float(np.sqrt(abs(psi[0] - 1.0) ** 2 + np.vdot(psi[1:], psi[1:]).real))
    out["checked"] = bool(out["mirror_err"] < 1e-12)
    return out


def cpu_baseline_reference(bs, ops, budget_s=25.0):
    """cpu_baseline for the headline line: a bounded sample (about budget_s of host work)."""
    rs = ReferenceSampler(bs, ops)
    rs.sample(n_gates=4, parts=("expectation", "probabilities", "shot"))
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s * 0.5:
        rs.sample(n_gates=4, parts=())
    t_step, parts = rs.estimate()
    workload_bytes = len(ops) * 32.0 * 2 ** N_QUBITS
    out = {"value": round(workload_bytes / t_step / 1e9, 3), "unit": "GB/s", "cores": rs.cores, "kind": "port",
           "sample": rs.describe(),
           "extrapolated_s_per_step": round(t_step, 1), "parts_s": {k: round(v, 2) for k, v in parts.items()},
           "evolve_only_GBps": round(workload_bytes / parts["evolve"] / 1e9, 2)}
    del rs
    return out


def adjoint_workload(bs, n=24, layers=10, terms=48, seed=3, ansatz="ry_rz_zz"):
    """(instructions, hamiltonian) of the adjoint-gradient workload.  ansatz "ry_rz_zz": per layer
    Ry(t) Rz(t) on every qubit and a ZZ(t) ring (720 parameters at 24 qubits, 10 layers); "ry_cz":
    per layer Ry(t) on every qubit and a fixed CZ ring (240 parameters).  Angles U(-pi, pi); the
    Hamiltonian has `terms` Pauli strings of weight <= 4 with N(0, 1) coefficients."""
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
    return ops, h


def adjoint_bench(bs, n=24, layers=10, terms=48, shift_params=24, seed=3, ansatz="ry_rz_zz", c64=True):
    """ansatz "ry_rz_zz": per layer Ry(t) Rz(t) on every qubit and a ZZ(t) ring (720 parameters at 24
    qubits, 10 layers); "ry_cz": per layer Ry(t) on every qubit and a fixed CZ ring (240 parameters)."""
    from importlib import import_module
    adj = import_module("braketsimulator_gb300.adjoint")
    ops, h = adjoint_workload(bs, n, layers, terms, seed, ansatz)
    rng = np.random.default_rng(seed + 1)
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


def ghz_bench(bs, reps=2000, cpu=False):
    """GHZ-10 (H, CNOT(0,k)), full probabilities and 1000 shots per circuit: latency-bound.
    run(): simulate in one round trip (one upload, one CTA for the whole circuit, the sampler, one
    copy back); four_calls: reinit, evolve, probabilities and samples as separate calls."""
    import torch
    ops = [bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, 10)]
    sim = bs.StateVectorSimulator(10, 1000)
    for r in range(300):   # host caches and the GPU's clocks settle
        sim.run(ops, 1000, seed=r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in range(reps):
        p, s = sim.run(ops, 1000, seed=r)
    dt = (time.perf_counter() - t0) / reps
    ok = abs(p[0] - 0.5) < 1e-15 and abs(p[-1] - 0.5) < 1e-15 and set(np.unique(s)) <= {0, 1023}
    # a different circuit every call (GHZ-10 then Rz with a fresh angle on qubit 9): nothing of the
    # previous call's plan can be reused
    angles = np.random.default_rng(3).uniform(0, 2 * np.pi, reps // 4)
    variants = [ops + [bs.Instruction(bs.Rz(float(a)), [9])] for a in angles]
    t0 = time.perf_counter()
    for r, v in enumerate(variants):
        pv, sv = sim.run(v, 1000, seed=r)
    dt_distinct = (time.perf_counter() - t0) / len(variants)
    ok = ok and abs(pv[0] - 0.5) < 1e-13 and abs(pv[-1] - 0.5) < 1e-13   # float-float phases: ~2^-46
    for r in range(50):
        sim.reinit(10, 1000)
        sim.evolve(ops)
        sim.probabilities()
        sim.samples(r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in range(reps // 4):
        sim.reinit(10, 1000)
        sim.evolve(ops)
        p4 = sim.probabilities()
        s4 = sim.samples(r)
    dt4 = (time.perf_counter() - t0) / (reps // 4)
    # both flows give the same probabilities and, for the same seed, the same shots
    p, s = sim.run(ops, 1000, seed=reps)
    sim.reinit(10, 1000)
    sim.evolve(ops)
    ok = ok and np.array_equal(sim.probabilities(), p) and np.array_equal(sim.samples(reps), s)
    out = {"us_per_circuit": round(dt * 1e6, 1), "circuits_per_s": round(1 / dt, 1),
           "api": "StateVectorSimulator.run (bs_run_small)",
           "us_per_circuit_distinct": round(dt_distinct * 1e6, 1),
           "note": "us_per_circuit: the same circuit every call (its plan is reused); distinct: a new "
                   "Rz angle every call (planned every call)",
           "four_calls_us_per_circuit": round(dt4 * 1e6, 1),
           "checked": bool(ok)}
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
                     "trace": float(np.sum(diag)), "x4": ex}
    out["instructions"] = len(ops)
    if cpu:
        out["cpu_baseline"] = cb = dm_cpu_port(ops, n)
        if "oracle_x4" in cb:
            out["reference"]["x4_abs_diff_vs_oracle"] = abs(out["reference"]["x4"] - cb["oracle_x4"])
            out["reference"]["trace_abs_diff_vs_oracle"] = abs(out["reference"]["trace"] - cb["oracle_trace"])
    return out


def dm_cpu_port(ops, n=14, depth=12, budget_s=40.0):
    """Reference noise mode on the oracle port of the reference's CPU kernels (all host threads),
    layer by layer: the whole circuit when it fits the budget (then the oracle's trace and <X X X X>
    are returned beside the time, as the checker of the GPU values), else the layers done, scaled."""
    import oracle
    oracle.lib()
    layer = len(ops) // depth
    sim = oracle.OracleDM(n)
    sim.rho[:] = 0
    sim.rho[0] = 1.0
    t0 = time.perf_counter()
    done = 0
    while done < depth:
        sim.evolve(ops[done * layer:(done + 1) * layer])
        done += 1
        el = time.perf_counter() - t0
        if el / done * depth > budget_s:
            break
    dt = time.perf_counter() - t0
    out = {"s_per_circuit": round(dt * depth / done, 2), "cores": os.cpu_count(), "kind": "port",
           "sample": f"{done} of {depth} layers ({done * layer} instructions, {dt:.1f} s) timed"
                     + ("" if done == depth else f", scaled by {depth}/{done}")}
    if done == depth:
        out["oracle_trace"] = float(np.real(np.sum(sim.probabilities())))
        out["oracle_x4"] = oracle.expectation_pauli_dm(sim.rho, n, 0b1111, 0)
    return out


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
    hbm, _, src = peaks()
    # the batch's roofline: the sweeps' algorithmic bytes (one read and one write of a circuit's state
    # per sweep, 8 B per complex64 amplitude) over the batch's device time, against the HBM copy rate
    gbps = st2["bytes_moved"] / (st2["gpu_ms"] * 1e-3) / 1e9 if st2["gpu_ms"] > 0 else None
    roof = {"sweep_bytes": st2["bytes_moved"], "executed_sweep_GBps": round(gbps, 1) if gbps else None,
            "hbm_frac": round(gbps / hbm, 3) if gbps else None, "peak_GBps": hbm, "peak_source": src}
    return {"circuits": len(circuits), "qubits": "12..26", "gates": int(sum(len(c) for c in circuits)),
            "roofline": roof,
            "shots_each": 1000, "expectations_each": 8, "precision": "c64 (FP64 reductions)",
            "s_per_batch": round(dt, 3), "circuits_per_s": round(len(circuits) / dt, 1),
            "device_ms": round(st["gpu_ms"], 1), "sweeps": st["sweeps"],
            "max_abs_err_c64_vs_engine_c128_expectations": err,
            "graph": {"capture_s": round(t_cap, 3), "s_per_replay": round(t_rep, 3),
                      "circuits_per_s": round(len(circuits) / t_rep, 1), "device_ms": round(st2["gpu_ms"], 1),
                      "replay_equals_one_shot": same},
            **({"cpu_baseline": batch_cpu_port(circuits, counts, obs, exp)} if cpu else {})}


def batch_cpu_port(circuits, counts, obs=None, exp=None, budget_s=8.0):
    """The batch's gate sweeps on the oracle port of the reference's CPU kernels (complex128, all host
    threads; the reference has no complex64 path): circuits in batch order are evolved until the
    budget is spent, and the whole batch's time is scaled from the sample by gate-sweep bytes.  With
    the GPU's complex64 expectations (exp) the oracle's complex128 values of the sampled circuits
    check them."""
    import oracle
    oracle.lib()
    total = sum(len(c) * 32.0 * 2 ** n for c, n in zip(circuits, counts))
    done_bytes, t_used, k, errs = 0.0, 0.0, 0, []
    for ci, (c, n) in enumerate(zip(circuits, counts)):
        if t_used > budget_s or n > 24:
            continue
        sim = oracle.OracleSV(n)
        t0 = time.perf_counter()
        sim.evolve(c)
        t_used += time.perf_counter() - t0
        done_bytes += len(c) * 32.0 * 2 ** n
        k += 1
        if obs is not None and exp is not None:
            for t, term in enumerate(obs[ci]):
                x = sum(1 << q for q, pp in term.items() if pp in "XY")
                z = sum(1 << q for q, pp in term.items() if pp in "YZ")
                errs.append(abs(float(exp[ci, t]) - oracle.expectation_pauli_fast(sim.psi, n, x, z)))
    est = total / (done_bytes / t_used)
    out = {"circuits_per_s": round(len(circuits) / est, 2), "s_per_batch": round(est, 1), "cores": os.cpu_count(),
           "kind": "port", "sample": f"{k} circuits of <=24 qubits evolved in {t_used:.1f} s; the batch scaled by "
                                     "gate-sweep bytes (2*16*2^n per gate); shots and expectations not included"}
    if errs:
        out["max_abs_err_gpu_c64_vs_oracle_c128"] = float(max(errs))
        out["checked_expectations"] = len(errs)
    return out


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


class OracleCircuit:
    """Circuit objects for the reference arm, read by the oracle by attribute (name, angle,
    pow_exponent, matrix): the reference arm never imports the engine."""

    class Instruction:
        def __init__(self, operator, target):
            self.operator, self.target = operator, list(target)

    class Unitary:
        name = "unitary"
        angle = ()
        pow_exponent = 1.0

        def __init__(self, matrix):
            self.matrix = np.asarray(matrix, dtype=np.complex128)

    class CZ:
        name = "cz"
        angle = ()
        pow_exponent = 1.0

    class CNot:
        name = "cnot"
        angle = ()
        pow_exponent = 1.0


def workload_config(world, n_gates):
    """The config both arms report (identical dicts: same circuit, same outputs, same bytes)."""
    return {"workload": workload_name(), "qubits": N_QUBITS, "gates": n_gates, "shots": SHOTS,
            "outputs": f"<Z0 Z{N_QUBITS - 1}> and {SHOTS} shots",
            "bytes": "gate-layer bytes: 2*16*2^n per gate (one pass per gate, as the reference runs)",
            "l2": l2_note(), "parallelism": "replicas" if world > 1 else "1 GPU"}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (oracle port of its kernels, all host cores;
    Julia is not installed) on the same workload; each step times a bounded sample (the next
    slice of the instruction list plus one of expectation / probabilities / one shot) and the
    line reports the whole-step rate extrapolated from the running means."""
    if rank != 0:
        return
    ops = dense_circuit(OracleCircuit, n=N_QUBITS)
    rs = ReferenceSampler(OracleCircuit, ops)
    workload_bytes = len(ops) * 32.0 * 2 ** N_QUBITS
    rs.sample(n_gates=8, parts=("expectation", "probabilities", "shot"))
    vals, dts = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rs.sample(n_gates=8)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            t_step, parts = rs.estimate()
            vals.append(workload_bytes / t_step / 1e9)
            dts.append(dt)
    t_step, parts = rs.estimate()
    v = float(vals[-1])
    line = {"impl": "reference", "metric": "30q SV gate-layer HBM GB/s", "value": round(v, 3), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * float(np.mean(dts)), 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64)", "data": "synthetic (seeded Haar SU(2) + CZ)",
            "config": workload_config(world, len(ops)),
            "extrapolated_s_per_step": round(t_step, 1),
            "parts_s": {k: round(x, 2) for k, x in parts.items()},
            "evolve_only_GBps": round(workload_bytes / parts["evolve"] / 1e9, 2),
            "ms_per_step_note": "host time of each step's bounded sample; value uses extrapolated_s_per_step",
            "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": rs.cores, "kind": "port",
                             "sample": rs.describe()},
            "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _only_adjoint(bs):
    from importlib import import_module
    adj = import_module("braketsimulator_gb300.adjoint")
    ops, h = adjoint_workload(bs, n=24, layers=4)
    sim = bs.StateVectorSimulator(24, 0)
    for _ in range(3):
        e, g = adj.adjoint_gradient(sim, ops, h)
    return {"energy": e, "params": len(g)}


def _only_expect(bs):
    n = 26
    sim = bs.StateVectorSimulator(n, 0).evolve(dense_circuit(bs, n=n, layers=2, layers2=0))
    _, h = adjoint_workload(bs, n=n, layers=1, terms=48)
    from importlib import import_module
    adj = import_module("braketsimulator_gb300.adjoint")
    xm = np.array([adj.pauli_masks(t)[0] for _, t in h], dtype=np.uint64)
    zm = np.array([adj.pauli_masks(t)[1] for _, t in h], dtype=np.uint64)
    co = np.array([c for c, _ in h])
    out = np.empty(len(co))
    for _ in range(3):
        sim._h.call("bs_expectation_pauli", len(co), bs._abi.u64ptr(xm), bs._abi.u64ptr(zm), bs._abi.dptr(co),
                    bs._abi.dptr(out))
    return {"energy": float(out.sum())}


def _only_sample(bs):
    n = 26
    sim = bs.StateVectorSimulator(n, SHOTS).evolve(dense_circuit(bs, n=n, layers=2, layers2=0))
    for r in range(3):
        s = sim.samples(r)
    return {"distinct": int(np.unique(s).size)}


def _only_batch_small(bs):
    circuits, counts, obs = batch_circuits(bs, nc=256, seed=11)
    keep = [c for c in range(len(counts)) if counts[c] <= 12] or [0]
    for _ in range(3):
        exp, smp, st = bs.batch_simulate([circuits[c] for c in keep], [counts[c] for c in keep], [obs[c] for c in keep],
                                         shots=1000, seed=1, precision="c64")
    return {"circuits": len(keep)}


def _only_ghz(bs):
    ops = [bs.Instruction(bs.H(), [0])] + [bs.Instruction(bs.CNot(), [0, k]) for k in range(1, 10)]
    sim = bs.StateVectorSimulator(10, 1000)
    for r in range(50):
        sim.run(ops, 1000, seed=r)
    return {"kernel_us": sim.last_stats()["gpu_ms"] * 1e3}


def _only_dense(bs):
    n = 27
    sim = bs.StateVectorSimulator(n, 0)
    ops = dense_circuit(bs, n=n)
    for _ in range(2):
        sim.reinit(n, 0)
        sim.evolve(ops)
    return sim.last_stats()


# side workloads for kernel profiles: (what runs, the kernel it exercises)
PROFILE_WORKLOADS = {
    "adjoint24": (_only_adjoint, "k_adjoint_sweep: 24-qubit Ry/Rz/ZZ ansatz, 4 layers, 48 terms (256 MiB state)"),
    "expect26": (_only_expect, "k_pauli_sv: 48 Pauli terms on a 26-qubit state (1 GiB)"),
    "sample26": (_only_sample, "k_block_sums / k_sample_rng: 1e5 shots of a 26-qubit state"),
    "batch_small": (_only_batch_small, "k_batch_small: the <= 12-qubit circuits of a 256-circuit batch"),
    "dense27": (_only_dense, "k_tile_sweep_tc: the dense circuit at 27 qubits (2 GiB state)"),
    "ghz10": (_only_ghz, "k_small_run: GHZ-10 with 1000 shots through StateVectorSimulator.run, 50 times"),
}


def run_only(name):
    bs = load()
    fn, what = PROFILE_WORKLOADS[name]
    out = fn(bs)
    import torch
    torch.cuda.synchronize()
    print(json.dumps({"only": name, "what": what, **{k: v for k, v in out.items() if isinstance(v, (int, float))}}))


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
    ap.add_argument("--only", default=None, choices=sorted(PROFILE_WORKLOADS),
                    help="run one side workload a few times and exit (the small cases the kernel profiles use)")
    args = ap.parse_args()
    globals()["N_QUBITS"] = args.qubits
    if args.only:
        return run_only(args.only)
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
        # on the stream it is launched on.  Its roofline is the sweep's algorithmic HBM bytes (one read and
        # one write of the state, 2*16*2^n B per launch); the tensor work it executes is reported beside it.
        tc_launch_s = tc_ms * 1e-3 / tc_launches
        hbm_gbs = sweep_bytes / tc_launch_s / 1e9
        flop_per_launch = tc_gates * 2 ** (N_QUBITS - 12) * TC_FLOP_PER_TILE_GATE / tc_launches
        alg_flop_per_launch = tc_gates * 2 ** N_QUBITS * 256.0 / tc_launches
        roofline = {"bound": "hbm", "achieved": round(hbm_gbs, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(hbm_gbs / hbm, 3), "traffic": round(TC_DRAM_BYTES_PER_AMP * 2 ** N_QUBITS),
                    "peak_source": f"{src} (HBM copy)", "kernel": "k_tile_sweep_tc",
                    "bytes_per_launch": sweep_bytes, "launch_ms": round(tc_launch_s * 1e3, 2),
                    "launches_per_step": tc_launches // args.steps,
                    "fused_unitaries_per_launch": round(tc_gates / tc_launches, 2),
                    "tensor_view": {
                        "executed_bf16_TFLOPs": round(flop_per_launch / tc_launch_s / 1e12, 1),
                        "executed_frac_of_bf16_sustained": round(flop_per_launch / tc_launch_s / 1e12 / bf16, 3),
                        "algorithmic_TFLOPs": round(alg_flop_per_launch / tc_launch_s / 1e12, 2),
                        "note": "executed = 26 bf16 digit-pair MMAs per complex128 product (exact split); "
                                "algorithmic = 256 flop per amplitude per fused 5-qubit unitary"}}
    else:
        per_launch_ms = dev_ms / max(1, sweeps)
        achieved = sweep_bytes / (per_launch_ms * 1e-3) / 1e9
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved / hbm, 3), "traffic": None, "peak_source": f"{src} (HBM copy)",
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
        "config": workload_config(world, n_gates),
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
    line["check"] = headline_check(bs, sim, ops, e)
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_reference(OracleCircuit, dense_circuit(OracleCircuit, n=N_QUBITS))
    if not args.no_adjoint:
        line["dense_cnot"] = dense_cnot_bench(bs)
        line["adjoint"] = adjoint_bench(bs)
        line["adjoint240"] = adjoint_bench(bs, ansatz="ry_cz", c64=False)   # the 240-parameter ansatz
        line["ghz10"] = ghz_bench(bs, cpu=not args.no_cpu)
        line["dm14"] = dm_bench(bs, cpu=not args.no_cpu)
        line["batch512"] = batch_bench(bs, cpu=not args.no_cpu)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
