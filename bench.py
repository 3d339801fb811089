#!/usr/bin/env python3
"""Benchmark: 30-qubit FP64 brickwork circuit on one GB300 (+ adjoint gradients).

Workload (the brickwork circuit): 30 qubits FP64 (16 GiB state), from |0...0>,
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


def brickwork_ops(n: int, layers: int, seed: int = 2, source: str = "product"):
    """The brickwork circuit as a flat op array (the C ABI's spz_op records).

    source "product" builds it with the library's own record layout and seeded
    stream; source "oracle" with the oracle's numpy restatements of both, so
    that the reference arm never loads the product library.  Both give the
    same bytes (checked by tests/test_host.py)."""
    if source == "product":
        from spinoza_gb300 import _native as mod
        from spinoza_gb300 import rng

        uniforms = rng.uniforms
    else:
        import oracle as mod

        uniforms = mod.uniforms
    ang = uniforms(seed, 3 * n * layers) * (2.0 * math.pi)
    rows = []
    k = 0
    for _ in range(layers):
        for q in range(n):
            rows.append(((mod.U, 0, 0, 0, (ang[k], ang[k + 1], ang[k + 2])), q, mod.CONTROLS_NONE, 0, 0))
            k += 3
        for q in list(range(0, n - 1, 2)) + list(range(1, n - 1, 2)):
            rows.append(((mod.X, 0, 0, 0, (0.0, 0.0, 0.0)), q + 1, mod.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=mod.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops


def workload_config(n: int, layers: int) -> dict:
    """The `config` object of the headline line, identical in both arms."""
    return {"workload": f"brickwork-{n}q-{layers}layers (U(theta,phi,lambda) on every qubit, angles U[0,2pi) seed 2, "
                        f"+ CX even/odd ladders; from |0...0>)",
            "qubits": n, "layers": layers, "gates": layers * (2 * n - 1), "state_bytes": 16 << n,
            "l2": "inputs larger than L2 (16 GiB state vs 129 MB L2); no flush"}


def replica_throughput(ms_local: float, units_per_replica: float, steps: int, dist=None, device=None):
    """Replicas only: every rank runs the whole workload on its own GPU, no
    data-path collective.  Returns (ms, value): the slowest rank's time (max
    over ranks, the only collective) and the whole job's units per second
    (units of all ranks / that time)."""
    import torch

    world = 1
    if dist is not None:
        world = dist.get_world_size()
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_local = float(t.item())
    return ms_local, units_per_replica * world * steps / (ms_local / 1e3)


def algorithmic_bytes(ops, n: int) -> int:
    """Unfused algorithmic bytes as the library's planner counts them."""
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
        ln = ln.strip()
        if ln.startswith("dram_bytes_per_full_launch:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- CPU arms
def cpu_sample(n: int, layers_sample: int, reps: int = 1, warmup: int = 0, keep_state: bool = False) -> dict:
    """The oracle (restated reference CPU path, OpenMP over all host cores) on
    `layers_sample` brickwork layers at n qubits; returns the sample's
    algorithmic bytes and times.  Touches only the oracle: the ops, the seeded
    angles and the byte count all come from its numpy restatements."""
    import oracle

    ops = brickwork_ops(n, layers_sample, source="oracle")
    abytes = oracle.algorithmic_bytes(ops, n)
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
    out = {"bytes": abytes, "times": times, "gates": len(ops), "threads": oracle.num_threads()}
    if keep_state:
        out["state"] = (re, im)
    return out


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n, layers = args.qubits, args.layers
    res = cpu_sample(n, 1, reps=args.steps, warmup=args.warmup)
    t = sum(res["times"])
    value = res["bytes"] * len(res["times"]) / t / 1e9
    ms_layer = 1e3 * t / len(res["times"])
    sample = (f"1 of {layers} brickwork layers per step ({res['gates']} of {layers * (2 * n - 1)} gates) at {n} "
              f"qubits: the layers have identical structure, so GB/s over one layer is the full circuit's rate and "
              f"a full step takes {layers} x the layer time; oracle restatement of the reference CPU path "
              f"(reference Rust crate not buildable here), OpenMP over {res['threads']} host threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_layer,
        "ms_per_full_circuit_extrapolated": ms_layer * layers,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, layers),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["threads"], "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def adjoint_bench(n: int = 24, layers: int = 8, fd_sample: int = 4) -> dict:
    """Adjoint gradient of the 24-qubit, 384-parameter ansatz vs central FD
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
    reps = 3

    def timed(fast):
        s.reset_zero()
        adjoint.adjoint_gradient(s, opsv, pidx, H, fast=fast)  # warm-up (allocates the work vectors)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            s.reset_zero()
            e, g = adjoint.adjoint_gradient(s, opsv, pidx, H, fast=fast)
        return (time.perf_counter() - t0) / reps, e, g

    t_exact, e_exact, g_exact = timed(False)
    t_adj, e_fast, g_fast = timed(True)  # the headline: fast mode
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
    return {"qubits": n, "params": int(len(pidx)), "mode": "fast", "adjoint_s": t_adj,
            "grads_per_s": len(pidx) / t_adj, "adjoint_exact_s": t_exact,
            "max_abs_grad_diff_fast_vs_exact": float(np.max(np.abs(g_fast - g_exact))),
            "energy_diff_fast_vs_exact": float(abs(e_fast - e_exact)),
            "fd_forward_s": t_fwd, "fd_s_extrapolated": t_fd, "fd_grads_per_s": len(pidx) / t_fd,
            "speedup_vs_fd": t_fd / t_adj, "fd_sample": f"{fd_sample} of {2 * len(pidx)} forward circuits"}


def sweep_single_qubit(state, n: int, peak_gbs: float, fma_rate: float, reps: int = 3) -> dict:
    """Every single-qubit gate kind on every target at n qubits, through
    spz_apply: the reference's arithmetic (default) and the opt-in lazy mode
    (H, RX, RY as the gate over a scalar; RZ as P on the 1 half times a
    carried phase).  Per gate: CUDA-event time on the state's stream (mean of
    `reps` back-to-back applications), GB/s over the algorithmic 32 N bytes,
    the fraction of the measured HBM copy rate and of the live DFMA rate."""
    import torch

    from spinoza_gb300 import gates
    from spinoza_gb300.gates import Gate

    N = 1 << n
    kinds = [("H", Gate.H, 8, 4), ("RX", Gate.RX(0.7), 12, 4), ("RY", Gate.RY(0.7), 12, 4),
             ("RZ", Gate.RZ(0.7), 8, 4), ("U", Gate.U(0.3, 0.4, 0.5), 14, None), ("X", Gate.X, 0, None)]
    stream = torch.cuda.current_stream()
    rows = []
    for lazy in (False, True):
        state.set_lazy(lazy)
        for name, g, fp_exact, fp_lazy in kinds:
            if lazy and fp_lazy is None:
                continue
            for t in range(n):
                gates.apply(g, state, t)  # warm-up
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    gates.apply(g, state, t)
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1) / reps
                fp = (fp_lazy if lazy else fp_exact) * (N // 2)
                gbs = 32 * N / (ms / 1e3) / 1e9
                rows.append({"gate": name, "mode": "lazy" if lazy else "exact", "target": t, "ms": ms, "gbs": gbs,
                             "hbm_frac": gbs / peak_gbs, "fp64_frac": fp / (ms / 1e3) / fma_rate})
            state.settle()
    state.set_lazy(False)
    summary = {}
    for name, _, _, _ in kinds:
        for mode in ("exact", "lazy"):
            r = [x for x in rows if x["gate"] == name and x["mode"] == mode]
            if not r:
                continue
            summary[f"{name}_{mode}"] = {
                "ms_median": statistics.median(x["ms"] for x in r),
                "gbs_median": statistics.median(x["gbs"] for x in r),
                "hbm_frac_median": statistics.median(x["hbm_frac"] for x in r),
                "hbm_frac_min": min(x["hbm_frac"] for x in r),
                "fp64_frac_median": statistics.median(x["fp64_frac"] for x in r)}
    return {"qubits": n, "reps": reps, "peak_gbs": peak_gbs, "fma_rate": fma_rate, "summary": summary,
            "rows": rows,
            "note": "GB/s = 32 N algorithmic bytes per gate / time (the lazy RZ moves only the 1 half, 16 N); "
                    "exact = the reference's arithmetic, bit-identical; lazy = spz_state_set_lazy, within rounding"}


def numa_bind_to_gpu(device: int) -> dict:
    """Run this thread on the host cores of the GPU's NUMA node, so that pinned
    host buffers allocated afterwards are first touched (placed) there."""
    info = {"nproc": os.cpu_count(), "node": None, "cpus": None}
    try:
        import torch

        pr = torch.cuda.get_device_properties(device)
        bus = f"{int(getattr(pr, 'pci_domain_id', 0)):04x}:{int(pr.pci_bus_id):02x}:{int(pr.pci_device_id):02x}.0"
        info["pci"] = bus
        node = int(Path(f"/sys/bus/pci/devices/{bus}/numa_node").read_text().strip())
        info["node"] = node
        if node >= 0:
            cpus = set()
            for part in Path(f"/sys/devices/system/node/node{node}/cpulist").read_text().strip().split(","):
                lo, _, hi = part.partition("-")
                cpus.update(range(int(lo), int(hi or lo) + 1))
            if cpus:
                os.sched_setaffinity(0, cpus)
                info["cpus"] = len(cpus)
    except (OSError, ValueError, AttributeError, RuntimeError) as e:
        info["error"] = str(e)
    return info


def gpu_arm(args) -> None:
    import torch

    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import circuit, core
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
    N = 1 << n
    mode = nat.EXEC_DEFAULT if args.exact else nat.EXEC_FAST
    mode |= {"threads": 0, "tma": nat.EXEC_TMA, "tma-prefetch": nat.EXEC_TMA_PREFETCH,
             "shuffle": nat.EXEC_SHUFFLE}[args.staging]
    re_t = torch.empty(N, dtype=torch.float64, device="cuda")
    im_t = torch.empty(N, dtype=torch.float64, device="cuda")
    state = State.from_torch(re_t, im_t)
    stream = torch.cuda.current_stream()
    state.set_stream(stream)  # events on torch's stream bracket the kernels
    qc = QuantumCircuit.from_state(state, fast=not args.exact)

    def step(flags=0):
        flags |= mode
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
    ms, value = replica_throughput(e0.elapsed_time(e1), abytes / 1e9, args.steps, dist, "cuda")
    ms_step = ms / args.steps
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
        numa = numa_bind_to_gpu(local)
        hin_re = torch.zeros(N, dtype=torch.float64, pin_memory=True)
        hin_im = torch.zeros(N, dtype=torch.float64, pin_memory=True)
        hin_re[0] = 1.0
        hout_re = torch.empty(N, dtype=torch.float64, pin_memory=True)
        hout_im = torch.empty(N, dtype=torch.float64, pin_memory=True)

        hin = (hin_re.numpy(), hin_im.numpy())
        hout = (hout_re.numpy(), hout_im.numpy())
        tr = circuit.QubitTracker()

        def e2e_step():
            # the reference's setting: a host State in, the executed State out
            circuit.execute_host(ops, hin[0], hin[1], hout, state=state, tracker=tr, fast=not args.exact)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        t_e2e = (time.perf_counter() - t0) / args.steps
        # upload / download alone, for the record (not part of the timed region):
        # the library's calls, best of 3, and torch's own copies of the same
        # pinned buffers (a slow host link shows in both)
        up, down, tup = [], [], []
        for _ in range(3):
            t1 = time.perf_counter()
            nat.check(nat.lib().spz_state_upload(state.handle, nat.ptr(hin[0]), nat.ptr(hin[1])))
            t2 = time.perf_counter()
            nat.check(nat.lib().spz_state_download(state.handle, nat.ptr(hout[0]), nat.ptr(hout[1])))
            t3 = time.perf_counter()
            re_t.copy_(hin_re, non_blocking=True)
            im_t.copy_(hin_im, non_blocking=True)
            torch.cuda.synchronize()
            t4 = time.perf_counter()
            up.append(t2 - t1)
            down.append(t3 - t2)
            tup.append(t4 - t3)
        t1, t2, t3 = 0.0, min(up), min(up) + min(down)
        e2e = {"value": abytes * world / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": 16 * N + ops.nbytes,
               "d2h_bytes_per_step": 16 * N, "ms_per_step": 1e3 * t_e2e,
               "upload_alone_ms": 1e3 * (t2 - t1), "download_alone_ms": 1e3 * (t3 - t2),
               "h2d_gbs": 16 * N / (t2 - t1) / 1e9, "d2h_gbs": 16 * N / (t3 - t2) / 1e9,
               "h2d_gbs_torch_copy": 16 * N / min(tup) / 1e9, "host": numa,
               "api": "spz_circuit_execute_host (pinned host arrays in and out; the copies overlap the leading "
                      "and trailing tile passes, slab by slab)"}
        del hin_re, hin_im, hout_re, hout_im

    # Parity at full size: the exact (reference-arithmetic, bit-identical to the
    # oracle's sequence) mode on a second state; max |difference| of the amplitudes.
    parity = None
    if not args.exact and not args.no_parity:
        re2 = torch.empty(N, dtype=torch.float64, device="cuda")
        im2 = torch.empty(N, dtype=torch.float64, device="cuda")
        s2 = State.from_torch(re2, im2)
        s2.reset_zero()
        q2 = QuantumCircuit.from_state(s2)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        q2.execute_ops(ops)
        t1.record()
        torch.cuda.synchronize()
        state.reset_zero()
        qc.execute_ops(ops)  # a fresh fast run to compare against
        torch.cuda.synchronize()
        d = max(float((re_t - re2).abs().max()), float((im_t - im2).abs().max()))
        parity = {"max_abs_diff_fast_vs_exact": d, "bound": 1e-12, "ok": d <= 1e-12,
                  "exact_ms_per_step": t0.elapsed_time(t1),
                  "exact_gbs": abytes / (t0.elapsed_time(t1) / 1e3) / 1e9,
                  "max_abs_amplitude": max(float(re_t.abs().max()), float(im_t.abs().max()))}
        del s2, q2, re2, im2
    sweep = None
    if rank == 0 and not args.no_sweep:
        sweep = sweep_single_qubit(state, n, peaks["hbm_gbs"], fma_rate)
    adj = None if args.no_adjoint or rank != 0 else adjoint_bench()
    bat = None if args.no_batch or rank != 0 else batch_bench(args)
    qft = mea = None
    if rank == 0 and not args.no_configs:
        qft = qft20_bench(args)
        mea = measure28_bench(args)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        torch.cuda.synchronize()
        res = cpu_sample(n, 1, keep_state=True)
        cpu = {"value": res["bytes"] / res["times"][0] / 1e9, "unit": UNIT, "cores": res["threads"], "kind": "port",
               "sample": f"1 of {layers} brickwork layers ({res['gates']} gates) at {n} qubits, oracle restatement of "
                         f"the reference CPU path, OpenMP over {res['threads']} host threads"}
        # Parity of the timed workload against the oracle at full size, on the
        # same one-layer prefix (outside the timed region): the oracle's state
        # is uploaded and compared on the device.
        ore = torch.from_numpy(res["state"][0]).to("cuda")
        oim = torch.from_numpy(res["state"][1]).to("cuda")
        del res
        ops1 = brickwork_ops(n, 1)
        out = {"prefix": f"first 1 of {layers} layers ({len(ops1)} gates), {n} qubits, from |0...0>"}
        for mode, fast in (("fast", True), ("exact", False)):
            state.reset_zero()
            QuantumCircuit.from_state(state, fast=fast).execute_ops(ops1)
            torch.cuda.synchronize()
            d = max(float((re_t - ore).abs().max()), float((im_t - oim).abs().max()))
            out[f"max_abs_diff_{mode}_vs_oracle"] = d
            if not fast:
                out["exact_bit_identical"] = bool(torch.equal(re_t, ore) and torch.equal(im_t, oim))
        out["bound"] = 1e-12
        out["ok"] = out["max_abs_diff_fast_vs_oracle"] <= 1e-12 and out["exact_bit_identical"]
        del ore, oim
        if parity is None:
            parity = {}
        parity["vs_oracle"] = out
    sw33 = None
    if rank == 0 and not args.no_sweep33:
        torch.cuda.empty_cache()
        sw33 = sweep33_bench(33, steps=2, warmup=1)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(n, layers),
            "staging": args.staging,
            "executor": ("fused shared-memory tile passes, exact reference arithmetic" if args.exact else
                         "fused shared-memory tile passes, fast arithmetic (lazy scaling, U = P RY P, phases pushed "
                         "through permutations); equal to exact up to rounding"),
            "parallelism": "replicas" if world > 1 else "single-gpu",
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
            "parity": parity,
            "sweep30": sweep,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "adjoint": adj,
            "batch": bat,
            "qft20": qft,
            "measure28": mea,
            "sweep33": sw33,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------------------ other configs
def _line(metric: str, value: float, unit: str, args, **extra) -> None:
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "dtype": "f64", "data": "synthetic"}
    d.update(extra)
    print(json.dumps(d), flush=True)


def _event_time(fn, steps: int, warmup: int) -> float:
    """Mean seconds per call, CUDA events on torch's current stream, synchronised around."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps


def narrow_ops(n: int, layers: int, seed: int = 3):
    """A circuit on qubits 0-4 of an n-qubit state: per layer U on each of the
    five, then CX(0,1) CX(2,3) CX(1,2) CX(3,4)."""
    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import rng

    ang = rng.uniforms(seed, 15 * layers) * (2.0 * math.pi)
    rows, k = [], 0
    for _ in range(layers):
        for q in range(5):
            rows.append(((nat.U, 0, 0, 0, (ang[k], ang[k + 1], ang[k + 2])), q, nat.CONTROLS_NONE, 0, 0))
            k += 3
        for q in (0, 2, 1, 3):
            rows.append(((nat.X, 0, 0, 0, (0.0, 0.0, 0.0)), q + 1, nat.CONTROLS_SINGLE, 1 << q, 0))
    ops = np.zeros(len(rows), dtype=nat.OP_DTYPE)
    for i, r in enumerate(rows):
        ops[i] = r
    return ops


def workload_narrow(args) -> None:
    """The narrow circuit (every gate on qubits 0-4; one fused pass) on an
    n-qubit state, fast and exact mode, with the chosen tile staging: device
    time of the pass, FP64 rate against the live DFMA probe."""
    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import core
    from spinoza_gb300.core import State

    n, layers = args.qubits, args.layers
    ops = narrow_ops(n, layers)
    staging = {"threads": 0, "tma": nat.EXEC_TMA, "tma-prefetch": nat.EXEC_TMA_PREFETCH,
               "shuffle": nat.EXEC_SHUFFLE}[args.staging]
    s = State(n)
    rate = core.fp64_fma_rate()
    out = {}
    for mode, base in (("fast", nat.EXEC_FAST), ("exact", nat.EXEC_DEFAULT)):
        ms = []
        for i in range(args.warmup + args.steps):
            s.reset_zero()
            tr, st = nat.spz_tracker(0, 0), nat.spz_exec_stats()
            nat.check(nat.lib().spz_circuit_execute(s.handle, nat.ptr(ops), len(ops), nat.byref(tr),
                                                    base | staging | nat.EXEC_TIME_PASSES, nat.byref(st)))
            if i >= args.warmup:
                ms.append(st.tile_ms + st.plain_ms)
        t = sum(ms) / len(ms)
        out[mode] = {"ms": t, "passes": int(st.passes), "tile_passes": int(st.tile_passes),
                     "ops_in_shuffle_runs": int(st.shuffle_gates), "fp64_per_s": st.fp64_ops / (t / 1e3),
                     "fp64_frac": st.fp64_ops / (t / 1e3) / rate, "gb_s": st.algorithmic_bytes / (t / 1e3) / 1e9}
    _line(f"narrow circuit ({layers} layers on qubits 0-4) FP64 gate-apply GB/s", out["fast"]["gb_s"], "GB/s", args,
          config={"workload": f"narrow-{n}q-{layers}layers (U on qubits 0-4, CX(0,1) CX(2,3) CX(1,2) CX(3,4) per "
                              f"layer; from |0...0>)", "qubits": n, "layers": layers, "gates": len(ops)},
          staging=args.staging, modes=out, dfma_rate=rate, higher_is_better=True)


def qft20_bench(args) -> dict:
    """QFT with swaps on a seeded N(0,1) normalised 20-qubit state: the fused
    executor, the unfused per-gate path and compiled programs (graph replay),
    exact and fast, against the oracle."""
    import oracle
    from spinoza_gb300 import _native as nat
    from spinoza_gb300 import circuit, rng
    from spinoza_gb300.circuit import QuantumCircuit
    from spinoza_gb300.core import State

    n = 20
    qc = QuantumCircuit.__new__(QuantumCircuit)
    qc.transformations = []
    for j in range(n - 1, -1, -1):
        qc.h(j)
        for k in range(j - 1, -1, -1):
            qc.cp(math.pi / 2 ** (j - k), j, k)
    for i in range(n // 2):
        qc.swap(i, n - 1 - i)
    ops = circuit._ops_array(qc.transformations, lambda: 0.0)
    import torch

    init = rng.normal_state(n, 1)
    src, s = State.from_arrays(*init), State(n)
    src.set_stream(torch.cuda.current_stream())
    s.set_stream(torch.cuda.current_stream())
    runner = QuantumCircuit.from_state(s)
    out = {}
    for name, fused in (("fused", True), ("unfused", False)):
        runner.fused = fused

        def step():
            nat.check(nat.lib().spz_state_copy(s.handle, src.handle))
            runner.execute_ops(ops)

        out[name] = _event_time(step, args.steps * 20, args.warmup)
    # the same circuit compiled once and replayed as a CUDA graph
    progs = {"program": circuit.Program(n, ops), "program_fast": circuit.Program(n, ops, fast=True)}
    for name, prog in progs.items():
        def pstep(prog=prog):
            nat.check(nat.lib().spz_state_copy(s.handle, src.handle))
            prog.run(s)

        out[name] = _event_time(pstep, args.steps * 20, args.warmup)
        if name == "program":
            pre, pim = s.to_numpy()
    re, im = init[0].copy(), init[1].copy()
    t0 = time.perf_counter()
    oracle.execute(ops, re, im)
    t_cpu = time.perf_counter() - t0
    gre, gim = s.to_numpy()  # the fast program's result
    d_fast = float(max(np.max(np.abs(gre - re)), np.max(np.abs(gim - im))))
    d = float(max(np.max(np.abs(pre - re)), np.max(np.abs(pim - im))))
    abytes = algorithmic_bytes(ops, n)
    return {"workload": "QFT with swaps, 20 qubits, N(0,1) normalised state seed 1", "gates": len(ops),
            "program_fast_ms": out["program_fast"] * 1e3, "program_ms": out["program"] * 1e3,
            "execute_ms": out["fused"] * 1e3, "unfused_ms": out["unfused"] * 1e3,
            "effective_gbs": abytes / out["program_fast"] / 1e9, "passes": circuit.plan_stats(n, ops)["passes"],
            "cpu_baseline_ms": t_cpu * 1e3, "cpu_threads": oracle.num_threads(),
            "max_abs_diff_vs_oracle": d, "bit_identical": bool(d == 0.0), "max_abs_diff_fast_vs_oracle": d_fast,
            "note": "program_fast: the fast-mode program (planned once, replayed as a CUDA graph); execute: the "
                    "bit-exact spz_circuit_execute (plans each run); program: the bit-exact program; every run "
                    "includes a device copy of the input state; cpu_baseline: the oracle, one run"}


def workload_qft20(args) -> None:
    r = qft20_bench(args)
    _line("QFT-20 circuit time", r["program_fast_ms"], "ms", args, higher_is_better=False,
          config={"workload": r.pop("workload"), "gates": r.pop("gates")}, **r)


def measure28_bench(args, oracle_check: bool = True) -> dict:
    """28 qubits: 1e6 seeded shots (bit-exact rule) and <H> = sum a ZZ + b X,
    with the oracle's shots and <H> on the same downloaded state."""
    from spinoza_gb300 import core, rng
    from spinoza_gb300.core import State

    n = 28
    s = State(n)
    s.fill_random(3, "normal", normalise=True)
    u = rng.uniforms(4, 1_000_000)
    t_shots = _event_time(lambda: core.sample(s, u), args.steps, 1)
    ab = rng.uniforms(5, 4 * n)
    a = np.sqrt(-2 * np.log1p(-ab[:n - 1])) * np.cos(2 * math.pi * ab[n:2 * n - 1])
    b = np.sqrt(-2 * np.log1p(-ab[2 * n:3 * n])) * np.cos(2 * math.pi * ab[3 * n:4 * n])
    H = core.ising_hamiltonian(a, b)
    t_h = _event_time(lambda: core.pauli_expectation(s, H), args.steps, 1)
    N = 1 << n
    energy = core.pauli_expectation(s, H)
    out = {"workload": "28-qubit N(0,1) normalised state, 1e6 shots (uniform seed 4), <H> with a_i, b_i ~ N(0,1) "
                       "(seed 5)", "terms": int(len(H)), "shots_per_s": 1e6 / t_shots, "sample_ms": t_shots * 1e3,
           "sample_gbs": (24 * N) / t_shots / 1e9, "expectation_ms": t_h * 1e3,
           "expectation_gbs": (16 * N) / t_h / 1e9, "energy": energy}
    if oracle_check:
        import oracle

        shots = core.sample(s, u)
        re, im = s.to_numpy()
        del s
        t0 = time.perf_counter()
        want = oracle.sample(re, im, u)
        t_cpu = time.perf_counter() - t0
        e_orc = oracle.pauli_expectation(re, im, H)
        out.update({"shots_bit_identical_vs_oracle": bool(np.array_equal(shots, want)),
                    "energy_abs_diff_vs_oracle": abs(energy - e_orc), "cpu_sample_ms": t_cpu * 1e3,
                    "cpu_threads": oracle.num_threads()})
    return out


def workload_measure28(args) -> None:
    r = measure28_bench(args, oracle_check=False)
    _line("shots/s at 28 qubits", r["shots_per_s"], "shots/s", args, higher_is_better=True,
          config={"workload": r.pop("workload"), "terms": r.pop("terms")}, **r)


def batch_bench(args) -> dict:
    """4096 variational instances, qubits 10..22, depth 2..10, forward <H> and
    adjoint gradients of all of them per graph launch, against a loop of the
    single-instance path (spz_adjoint_gradient, one instance at a time) on a
    stratified sample, and against the oracle's parameter shift on sampled
    instances and parameters."""
    import oracle
    from spinoza_gb300 import adjoint, batch
    from spinoza_gb300.core import State

    t0 = time.perf_counter()
    insts = batch.hea_workload(args.instances, qmin=args.batch_qmin, qmax=args.batch_qmax)
    t_build = time.perf_counter() - t0
    explicit = args.batch_tile or args.batch_threads or args.batch_tpi
    t0 = time.perf_counter()
    tune = ({"tile_qubits": args.batch_tile, "threads": args.batch_threads, "tiles_per_item": args.batch_tpi}
            if explicit or args.no_autotune else batch.autotune(insts, reps=1))
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = batch.Batch(insts, tile_qubits=tune["tile_qubits"], threads=tune["threads"], wide_qubits=args.batch_wide,
                    fast=args.batch_fast, tiles_per_item=tune.get("tiles_per_item", 0),
                    wide_apart=args.batch_apart)
    t_plan = time.perf_counter() - t0
    b.run()
    steps = max(1, args.batch_steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        e, g = b.run()
    t_batch = (time.perf_counter() - t0) / steps
    # the loop: the single-instance path on a stratified sample, extrapolated
    order = sorted(range(len(insts)), key=lambda i: insts[i][0] * 1000 + len(insts[i][1]))
    sample = order[:: max(1, len(order) // args.loop_sample)]
    t_loop_sample = 0.0
    max_e, max_g = 0.0, 0.0
    for i in sample:
        n, ops, pidx, theta, terms = insts[i]
        t1 = time.perf_counter()
        e1, g1 = adjoint.adjoint_gradient(State(n), adjoint.set_params(ops, pidx, theta), pidx, terms,
                                          fast=args.batch_fast)
        t_loop_sample += time.perf_counter() - t1
        max_e = max(max_e, abs(e1 - e[i]))
        max_g = max(max_g, float(np.max(np.abs(g1 - b.split(g)[i]))))
    t_loop = t_loop_sample * len(insts) / len(sample)
    # the oracle's parameter shift (exact for RY / RZ) on sampled instances
    checks, max_ps = 0, 0.0
    picks = [order[0], order[len(order) // 3], order[-1]]
    for i in picks:
        n, ops, pidx, theta, terms = insts[i]
        gi = b.split(g)[i]

        def energy(th):
            re, im = oracle.zero_state(n)
            oracle.execute(adjoint.set_params(ops, pidx, th).view(oracle.OP_DTYPE), re, im)
            return oracle.pauli_expectation(re, im, terms)

        for j in (0, len(pidx) // 2, len(pidx) - 1):
            tp, tm = theta.copy(), theta.copy()
            tp[j] += math.pi / 2
            tm[j] -= math.pi / 2
            max_ps = max(max_ps, abs(gi[j] - 0.5 * (energy(tp) - energy(tm))))
            checks += 1
    nparams = int(b.theta.size)
    qs = [x[0] for x in insts]
    return {"workload": f"{len(insts)} HEA instances (RY/RZ layers + CZ ring), qubits U{{{args.batch_qmin}..{args.batch_qmax}}}, "
                        f"depth U{{2..10}}, seeds 8+k", "instances": len(insts), "params": nparams,
            "qubits_min": min(qs), "qubits_max": max(qs), "launch": tune,
            "wide_qubits": args.batch_wide or 18, "wide_adjoint": "fast" if args.batch_fast else "exact",
            "wide_path": ("one at a time across the GPU" if args.batch_fast or args.batch_apart else
                          "work items inside the persistent launch"),
            "seconds_per_batch": t_batch, "instances_per_s": len(insts) / t_batch, "grads_per_s": nparams / t_batch,
            "loop_seconds_extrapolated": t_loop, "loop_sample": len(sample), "speedup_vs_loop": t_loop / t_batch,
            "max_abs_energy_diff_vs_loop": max_e, "max_abs_grad_diff_vs_loop": max_g,
            "max_abs_grad_diff_vs_oracle_parameter_shift": max_ps, "oracle_checks": checks,
            "oracle_instances": [int(insts[i][0]) for i in picks],
            "build_seconds": t_build, "plan_seconds": t_plan, "autotune_seconds": t_tune, "info": b.info(),
            "note": "loop = spz_adjoint_gradient per instance (fused executor, one instance at a time), timed on a "
                    "stratified sample and extrapolated; the batch is one graph launch (coefficients, the persistent "
                    "kernel with every instance, the fold of the wide instances' partial sums)"}


def workload_batch(args) -> None:
    d = batch_bench(args)
    _line("batched forward+adjoint instances/s", d["instances_per_s"], "instances/s", args,
          higher_is_better=True, config={"workload": d["workload"], "params": d["params"], "launch": d["launch"]},
          batch=d)


def workload_gate(args) -> None:
    """One gate kind on one target through spz_apply, exact or lazy, repeated:
    the case the per-gate kernels' profiles are taken on."""
    import torch

    from spinoza_gb300 import gates
    from spinoza_gb300.core import State
    from spinoza_gb300.gates import Gate

    n = args.qubits
    N = 1 << n
    s = State(n)
    s.fill_random(11, "uniform", normalise=True)
    s.set_stream(torch.cuda.current_stream())
    s.set_lazy(args.lazy)
    g = {"H": Gate.H, "X": Gate.X, "RX": Gate.RX(0.7), "RY": Gate.RY(0.7), "RZ": Gate.RZ(0.7),
         "U": Gate.U(0.3, 0.4, 0.5)}[args.gate]
    dt = _event_time(lambda: gates.apply(g, s, args.target), args.steps, args.warmup)
    s.settle()
    peaks = measured_peaks()
    gbs = 32 * N / dt / 1e9
    _line(f"{args.gate} gate at {n} qubits ({'lazy' if args.lazy else 'exact'})", gbs, "GB/s", args,
          higher_is_better=True, config={"workload": f"{args.gate} on target {args.target}, {n} qubits",
                                         "mode": "lazy" if args.lazy else "exact"},
          ms=dt * 1e3, hbm_frac=gbs / peaks["hbm_gbs"], peak_gbs=peaks["hbm_gbs"])


def sweep33_bench(n: int = 33, steps: int = 3, warmup: int = 3) -> dict:
    """Per-gate sweep: H, RZ, CX and 3-control X on every target at n qubits
    (33: 128 GiB), the reference's arithmetic through the per-gate entry points."""
    import torch

    from spinoza_gb300 import gates as G
    from spinoza_gb300.core import State
    from spinoza_gb300.gates import Gate

    N = 1 << n
    re = torch.empty(N, dtype=torch.float64, device="cuda")
    im = torch.empty(N, dtype=torch.float64, device="cuda")
    s = State.from_torch(re, im)
    s.fill_random(11, "uniform", normalise=False)
    peaks = measured_peaks()
    rows = []
    kinds = [("H", lambda t: G.apply(Gate.H, s, t), 32),
             ("RZ", lambda t: G.apply(Gate.RZ(0.7), s, t), 32),
             ("CX", lambda t: G.c_apply(Gate.X, s, (t + 1) % n, t), 16),
             ("MCX3", lambda t: G.mc_apply(Gate.X, s, [(t + 1) % n, (t + 2) % n, (t + 3) % n], None, t), 4)]
    for name, fn, bpn in kinds:
        for t in range(n):
            dt = _event_time(lambda: fn(t), steps, warmup)
            gbs = bpn * N / dt / 1e9
            rows.append({"gate": name, "target": t, "ms": dt * 1e3, "gbs": gbs, "frac": gbs / peaks["hbm_gbs"]})
    del s, re, im
    summary = {}
    for name, _, _ in kinds:
        r = [x for x in rows if x["gate"] == name]
        summary[name] = {"ms_median": statistics.median(x["ms"] for x in r),
                         "gbs_median": statistics.median(x["gbs"] for x in r),
                         "frac_median": statistics.median(x["frac"] for x in r),
                         "frac_min": min(x["frac"] for x in r)}
    return {"workload": f"H, RZ(0.7), CX(control (t+1) mod n), X with 3 controls (t+1..t+3 mod n), targets "
                        f"0..{n - 1}, {n} qubits ({16 * N >> 30} GiB)", "qubits": n, "steps": steps, "warmup": warmup,
            "summary": summary, "rows": rows, "peak_gbs": peaks["hbm_gbs"],
            "note": "GB/s = algorithmic bytes (32 N for H and RZ, 16 N for CX, 4 N for 3-control X) / CUDA-event "
                    "time per application; the reference's arithmetic (exact kernels)"}


def workload_sweep33(args) -> None:
    r = sweep33_bench(args.qubits if args.qubits != 30 else 33, args.steps, args.warmup)
    _line(f"per-gate sweep at {r['qubits']} qubits", r["summary"]["H"]["gbs_median"], "GB/s", args,
          higher_is_better=True, config={"workload": r.pop("workload")}, **r)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="brickwork",
                    choices=["brickwork", "qft20", "measure28", "batch", "sweep33", "gate", "narrow"])
    ap.add_argument("--gate", default="H", choices=["H", "X", "RX", "RY", "RZ", "U"], help="gate workload: kind")
    ap.add_argument("--target", type=int, default=5, help="gate workload: target qubit")
    ap.add_argument("--lazy", action="store_true", help="gate workload: the lazy per-gate mode")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--loop-sample", type=int, default=64)
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch: the library's default launch shape instead of the cached autotuner's choice")
    ap.add_argument("--no-batch", action="store_true", help="headline line without the 4096-instance batch object")
    ap.add_argument("--no-configs", action="store_true",
                    help="headline line without the QFT-20 and 28-qubit measurement objects")
    ap.add_argument("--batch-steps", type=int, default=1, help="timed runs of the 4096-instance batch")
    ap.add_argument("--batch-tpi", type=int, default=0, help="batch workload: tiles per work item of a wide instance")
    ap.add_argument("--batch-apart", action="store_true", help="batch workload: wide instances one at a time")
    ap.add_argument("--batch-tile", type=int, default=0,
                    help="batch workload: tile qubits, resident up to this n (0: the library default)")
    ap.add_argument("--batch-threads", type=int, default=0, help="batch workload: threads per block (0: default)")
    ap.add_argument("--batch-qmax", type=int, default=22, help="batch workload: largest instance (small profiling cases)")
    ap.add_argument("--batch-qmin", type=int, default=10, help="batch workload: smallest instance (profiling cases)")
    ap.add_argument("--batch-fast", action="store_true", help="batch workload: fast adjoint for the wide instances")
    ap.add_argument("--batch-wide", type=int, default=0,
                    help="batch workload: instances of at least this many qubits run across the whole GPU "
                         "(0: the library default, 31: never)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the per-gate sweep at the headline's qubit count")
    ap.add_argument("--no-sweep33", action="store_true", help="skip the per-gate sweep at 33 qubits (128 GiB)")
    ap.add_argument("--exact", action="store_true", help="time the bit-exact executor mode instead of fast mode")
    ap.add_argument("--staging", default="threads", choices=["threads", "tma", "tma-prefetch", "shuffle"],
                    help="how fused passes stage their tiles: thread loads (default), TMA gathers, or "
                         "thread loads with warp-shuffle runs for gates on the five lowest tile qubits")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "brickwork":
        gpu_arm(args)
    else:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        {"qft20": workload_qft20, "measure28": workload_measure28, "batch": workload_batch,
         "sweep33": workload_sweep33, "gate": workload_gate, "narrow": workload_narrow}[args.workload](args)


if __name__ == "__main__":
    main()
