#!/usr/bin/env python3
"""Benchmark: 30-qubit FP64 brickwork circuit on one GB300 (+ adjoint gradients).

Workload (BASELINE config 2): 30 qubits FP64 (16 GiB state), from |0...0>,
20 layers of U(theta, phi, lambda) on every qubit (angles uniform in [0, 2 pi)
from the seeded splitmix64 stream, seed 2), then CX on (0,1),(2,3),...,(28,29)
and (1,2),...,(27,28): 1180 gates.  One step = reset to |0...0> + execute the
whole circuit through the fused executor, state resident in HBM.  The state
(16 GiB) is far larger than L2 (129 MB), so no L2 flush is needed.

metric value = unfused algorithmic bytes of the gates (sum of 32N / 16N per
gate) / step time, in GB/s ("gate-apply GB/s"); gates/s is reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU path as restated by the oracle
(the Rust reference cannot be built here) on the host cores, one brickwork
layer per step (59 of the 1180 gates), same metric and unit.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q FP64 gate-apply GB/s vs HBM peak; adjoint grads/s vs plain-GPU FD (1e-9)"
UNIT = "GB/s"


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def brickwork_ops(n: int, layers: int, seed: int = 2):
    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import rng

    ang = rng.uniforms(seed, 3 * n * layers) * (2.0 * math.pi)
    rows = []
    k = 0
    for _ in range(layers):
        for q in range(n):
            rows.append(((nat.U, 0, 0, 0, (ang[k], ang[k + 1], ang[k + 2])), q, nat.CONTROLS_NONE, 0, 0))
            k += 3
        for q in list(range(0, n - 1, 2)) + list(range(1, n - 1, 2)):
            rows.append(((nat.X, 0, 0, 0, (0.0, 0.0, 0.0)), q + 1, nat.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops


def algorithmic_bytes(ops, n: int) -> int:
    from spinoza_gb300 import circuit

    return circuit.plan_stats(n, ops, fused=False)["algorithmic_bytes"]


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap",
              "clocks_event_reasons.hw_power_brake_slowdown", "utilization.gpu", "temperature.gpu"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={','.join(self.FIELDS)}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        else:
            self.lines = []

    def summary(self) -> dict:
        sm, mx, reasons, masks, power, util, temp = [], None, set(), set(), [], [], []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap", "hw_power_brake"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 12:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
                util.append(float(f[10]))
                temp.append(float(f[11]))
            except ValueError:
                continue
            masks.add(f[4])
            for name, val in zip(names, f[5:10]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        med = (lambda v: statistics.median(v) if v else None)
        return {"sm_mhz": med(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "active_masks": sorted(masks), "power_w_median": med(power), "util_pct_median": med(util),
                "temp_c_max": max(temp) if temp else None}


def profile_traffic(kernel_file: str):
    """DRAM bytes per launch recorded by ncu in profiles/<kernel_file> (or None)."""
    p = ROOT / "profiles" / kernel_file
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("dram_bytes_per_full_launch:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- CPU arms
def cpu_sample(n: int, layers_sample: int, reps: int = 1, warmup: int = 0) -> dict:
    """The oracle (restated reference CPU path, OpenMP over all host cores) on
    `layers_sample` brickwork layers at n qubits; returns GB/s over the
    sample's algorithmic bytes."""
    import oracle

    ops = brickwork_ops(n, layers_sample)
    abytes = algorithmic_bytes(ops, n)
    re, im = oracle.zero_state(n)
    times = []
    for r in range(warmup + reps):
        re[:] = 0.0
        im[:] = 0.0
        re[0] = 1.0
        t0 = time.perf_counter()
        oracle.execute(ops, re, im)
        dt = time.perf_counter() - t0
        if r >= warmup:
            times.append(dt)
    del re, im
    return {"bytes": abytes, "times": times, "gates": len(ops), "threads": oracle.num_threads()}


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n, layers = args.qubits, args.layers
    res = cpu_sample(n, 1, reps=args.steps, warmup=args.warmup)
    t = sum(res["times"])
    value = res["bytes"] * len(res["times"]) / t / 1e9
    sample = (f"1 of {layers} brickwork layers per step ({res['gates']} of {layers * (2 * n - 1)} gates) at {n} "
              f"qubits, oracle restatement of the reference CPU path (reference Rust crate not buildable here)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(res["times"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"brickwork-{n}q-{layers}layers (U on every qubit + CX even/odd, from |0...0>)",
                   "qubits": n, "layers": layers, "sample_layers_per_step": 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["threads"], "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def adjoint_bench(n: int = 24, layers: int = 8, fd_sample: int = 4) -> dict:
    """Config 4: adjoint gradient of the 384-parameter ansatz vs central FD
    (768 forward circuits) with the plain per-gate kernels, same GPU."""
    import torch

    from spinoza_gb300 import adjoint, core, rng
    from spinoza_gb300.circuit import QuantumCircuit
    from spinoza_gb300.core import State

    ops, pidx = adjoint.hardware_efficient_ansatz(n, layers)
    theta = (rng.uniforms(6, len(pidx)) * 2 - 1) * math.pi
    u = rng.uniforms(7, 4 * n)
    a = np.sqrt(-2 * np.log1p(-u[:n - 1])) * np.cos(2 * math.pi * u[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-u[2 * n:3 * n])) * np.cos(2 * math.pi * u[3 * n:4 * n])
    H = core.ising_hamiltonian(a, b)
    opsv = adjoint.set_params(ops, pidx, theta)
    s = State(n)
    adjoint.adjoint_gradient(s, opsv, pidx, H)  # warm-up (allocates the work vectors)
    torch.cuda.synchronize()
    reps = 2
    t0 = time.perf_counter()
    for _ in range(reps):
        s.reset_zero()
        adjoint.adjoint_gradient(s, opsv, pidx, H)
    t_adj = (time.perf_counter() - t0) / reps
    # FD baseline: forward circuits with the plain per-gate kernels + <H>.
    f = State(n)
    qc = QuantumCircuit.from_state(f, fused=False)
    qc.execute_ops(opsv)
    core.pauli_expectation(f, H)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(fd_sample):
        f.reset_zero()
        qc.execute_ops(opsv)
        core.pauli_expectation(f, H)
    t_fwd = (time.perf_counter() - t0) / fd_sample
    t_fd = 2 * len(pidx) * t_fwd
    return {"qubits": n, "params": int(len(pidx)), "adjoint_s": t_adj, "grads_per_s": len(pidx) / t_adj,
            "fd_forward_s": t_fwd, "fd_s_extrapolated": t_fd, "fd_grads_per_s": len(pidx) / t_fd,
            "speedup_vs_fd": t_fd / t_adj, "fd_sample": f"{fd_sample} of {2 * len(pidx)} forward circuits"}


def gpu_arm(args) -> None:
    import torch

    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import core
    from spinoza_gb300.circuit import QuantumCircuit
    from spinoza_gb300.core import State

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    n, layers = args.qubits, args.layers
    ops = brickwork_ops(n, layers)
    abytes = algorithmic_bytes(ops, n)
    state = State(n)
    stream = torch.cuda.current_stream()
    nat.check(nat.lib().spz_state_set_stream(state.handle, nat.c_void_p(stream.cuda_stream)))
    qc = QuantumCircuit.from_state(state)

    def step(flags=nat.EXEC_DEFAULT):
        state.reset_zero()
        st = nat.spz_exec_stats()
        nat.check(nat.lib().spz_circuit_execute(state.handle, nat.ptr(ops), len(ops), nat.byref(qc.qubit_tracker.c),
                                                flags, nat.byref(st)))
        return st

    fma_rate_before = core.fp64_fma_rate()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tile_ms, tile_launches, fp64_ops, launches, plain_ms = 0.0, 0, 0, 0, 0.0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            st = step(nat.EXEC_TIME_PASSES)
            tile_ms += st.tile_ms
            plain_ms += st.plain_ms
            tile_launches += st.tile_passes
            fp64_ops += st.fp64_ops
            launches += 1 + st.passes  # reset kernel + one kernel per pass
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = abytes * world * args.steps / (ms / 1e3) / 1e9
    peaks = measured_peaks()
    N = 1 << n
    tile_avg_ms = tile_ms / max(1, tile_launches)
    achieved = (32 * N) / (tile_avg_ms / 1e3) / 1e9
    traffic = profile_traffic("tile_kernel_brickwork30.txt")
    fma_rate_after = core.fp64_fma_rate()
    fma_rate = max(fma_rate_before, fma_rate_after)
    fp64_achieved = fp64_ops / ((tile_ms + plain_ms) / 1e3)

    # end to end: host (pinned) |0...0> in, execute, host result out
    e2e = None
    if not args.no_e2e:
        hin_re = torch.zeros(N, dtype=torch.float64, pin_memory=True)
        hin_im = torch.zeros(N, dtype=torch.float64, pin_memory=True)
        hin_re[0] = 1.0
        hout_re = torch.empty(N, dtype=torch.float64, pin_memory=True)
        hout_im = torch.empty(N, dtype=torch.float64, pin_memory=True)

        def e2e_step():
            nat.check(nat.lib().spz_state_upload(state.handle, nat.c_void_p(hin_re.data_ptr()),
                                                 nat.c_void_p(hin_im.data_ptr())))
            nat.check(nat.lib().spz_circuit_execute(state.handle, nat.ptr(ops), len(ops),
                                                    nat.byref(qc.qubit_tracker.c), nat.EXEC_DEFAULT, None))
            nat.check(nat.lib().spz_state_download(state.handle, nat.c_void_p(hout_re.data_ptr()),
                                                   nat.c_void_p(hout_im.data_ptr())))

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        t_e2e = (time.perf_counter() - t0) / args.steps
        e2e = {"value": abytes * world / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": 16 * N + ops.nbytes,
               "d2h_bytes_per_step": 16 * N, "ms_per_step": 1e3 * t_e2e,
               "api": "spz_state_upload + spz_circuit_execute + spz_state_download (pinned host buffers)"}
        del hin_re, hin_im, hout_re, hout_im

    adj = None if args.no_adjoint or rank != 0 else adjoint_bench()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        del state, qc
        torch.cuda.synchronize()
        res = cpu_sample(n, 1)
        cpu = {"value": res["bytes"] / res["times"][0] / 1e9, "unit": UNIT, "cores": res["threads"], "kind": "port",
               "sample": f"1 of {layers} brickwork layers ({res['gates']} gates) at {n} qubits, oracle restatement of "
                         f"the reference CPU path, OpenMP over {res['threads']} host threads"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"brickwork-{n}q-{layers}layers (U(theta,phi,lambda) on every qubit, angles "
                                   f"U[0,2pi) seed 2, + CX even/odd ladders; from |0...0>)",
                       "qubits": n, "layers": layers, "gates": int(len(ops)), "state_bytes": 16 * N,
                       "l2": "inputs larger than L2 (16 GiB state vs 129 MB L2); no flush",
                       "executor": "fused shared-memory tile passes, exact reference arithmetic",
                       "parallelism": "replicas" if world > 1 else "single-gpu"},
            "gates_per_s": len(ops) * world * args.steps / (ms / 1e3),
            "passes_per_step": int(launches / args.steps) - 1,
            "roofline": {"bound": "hbm", "kernel": "tile_kernel", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                         "peak_source": peaks["source"],
                         "note": "achieved = 32 N bytes (one read + one write of the state) per tile pass / mean "
                                 "tile-pass time; the tile passes are FP64-issue bound, see fp64"},
            "fp64": {"achieved": fp64_achieved, "peak": fma_rate, "unit": "FP64 instr/s", "frac": fp64_achieved / fma_rate,
                     "peak_before": fma_rate_before, "peak_after": fma_rate_after,
                     "note": "FP64-pipe instructions the gates need / device time of the passes; peak = DFMA issue "
                             "rate measured live on this GPU before and after the timed region "
                             "(spz_probe_fp64_fma_rate), the larger of the two"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "adjoint": adj,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
