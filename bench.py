"""Benchmark of the qibo state-vector hot path on one GB300.

Workload (one "step"): the 30-qubit random circuit of depth 20 — per layer
U3(theta, phi, lambda) on every qubit with angles uniform in [0, 2 pi) from a
seeded generator, then CZ on brickwork pairs — started from |0...0>, in
complex128, followed by 1e6 shots on all 30 qubits drawn from |psi|^2.

``value`` is the state-vector bandwidth of the step: the algorithmic bytes
of every pass (dense 1q/2q/fused/blocked pass: read+write of every
amplitude, 2 * 2^n * 16 B; CZ: 2 * 2^(n-2) * 16 B; probabilities: read
2^n * 16 B + write 2^n * 8 B; CDF/sampling: read 2^n * 8 B twice) divided by
the device time of the step, with the state already resident.  The state
(17.2 GB) is far larger than L2 (129 MB), so no L2 flush is needed.

``e2e`` is the same metric through the public API with host buffers:
``backend.execute_circuit(circuit, nshots=1e6)`` and the 1e6 samples read
back to the host every step.

``--impl reference`` times the reference's CPU algorithm (the numpy
restatement in ``oracle/``, OpenBLAS threads = all host cores) on a bounded
sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
DEPTH = 20
SEED = 30
NSHOTS = 1_000_000
METRIC = "state-vector GB/s vs HBM peak at n=30; circuits/s + p99 at <=1e-6 infidelity"


def brickwork_gates(n, depth, seed):
    from qibo_gb300 import gates

    ang = np.random.default_rng(seed).uniform(0, 2 * np.pi, (depth, n, 3))
    out = []
    for l in range(depth):
        for q in range(n):
            out.append(gates.U3(q, *ang[l, q]))
        for q in range(l % 2, n - 1, 2):
            out.append(gates.CZ(q, q + 1))
    return out


def algorithmic_bytes(n, ngates_dense, ngates_cz, dtype_bytes):
    N = 2**n
    gates_b = ngates_dense * 2 * N * dtype_bytes + ngates_cz * 2 * (N // 4) * dtype_bytes
    probs_b = N * dtype_bytes + N * 8
    sample_b = 2 * N * 8
    return gates_b, probs_b + sample_b


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", "0", "-lms", "200"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline_sample(n=28, ngates=9, dtype="complex128"):
    """The reference algorithm (oracle port: transpose, zgemm, transpose per
    gate, backends/abstract.py:2350-2355) on the first ``ngates`` gates of
    layer 0 of the brickwork circuit at ``n`` qubits.  Returns GB/s with the
    same byte accounting as the GPU metric."""
    from oracle import numpy_ref as ref

    ops = ref.brickwork_ops(n, 1, SEED)
    u3 = [o for o in ops if o[0] == "U3"][: (2 * ngates) // 3]
    cz = [o for o in ops if o[0] == "CZ"][: ngates - len(u3)]
    sample = u3 + cz
    st = ref.zero_state(n, dtype)
    st[:] = 1 / np.sqrt(2**n)
    t0 = time.perf_counter()
    for name, q, p in sample:
        st = ref.apply_gate(st, ref.gate_matrix(name, p, dtype), q, n)
    dt = time.perf_counter() - t0
    S = np.dtype(dtype).itemsize
    b = len(u3) * 2 * 2**n * S + len(cz) * 2 * 2**(n - 2) * S
    return {"value": b / dt / 1e9, "unit": "GB/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{len(u3)} U3 + {len(cz)} CZ of layer 0, n={n}, {dtype}, numpy/OpenBLAS "
                      f"(reference NumpyBackend algorithm), {dt:.2f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_baseline_sample(n=24, ngates=6)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline_sample(n=26, ngates=9))
    dt = time.perf_counter() - t0
    v = statistics.median([x["value"] for x in vals])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic",
            "config": {"workload": "random U3+CZ brickwork, depth 20, seed 30 (sampled gates)", "nqubits": 26},
            "cpu_baseline": {k: vals[-1][k] for k in ("kind", "cores", "sample")} | {"value": v, "unit": "GB/s"},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nqubits", type=int, default=N_QUBITS)
    ap.add_argument("--dtype", default="complex128")
    ap.add_argument("--mode", default="auto", choices=["auto", "gates", "blocked", "fused"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")

    from qibo_gb300 import Circuit
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend, describe_gate
    from qibo_gb300.device import DeviceState

    n, dtype = args.nqubits, args.dtype
    S = 16 if dtype == "complex128" else 8
    backend = GB300Backend(dtype)
    rt, eng, lib = backend.rt, backend.engine_gb, backend.rt.lib
    gates = brickwork_gates(n, DEPTH, SEED)
    circ = Circuit(n)
    circ.add(gates)
    mode = args.mode if args.mode != "auto" else "blocked"
    run_circ = circ.fuse(5) if mode == "fused" else circ
    descs = [describe_gate(g, backend) for g in run_circ.queue]
    backend.blocked = mode in ("blocked", "fused")
    ndense = sum(1 for g in gates if type(g).__name__ == "U3")
    ncz = len(gates) - ndense
    # effective bytes: what the unfused gate-by-gate passes of this circuit move
    gbytes, mbytes = algorithmic_bytes(n, ndense, ncz, S)
    npasses = eng.count_passes(n, 1 if dtype == "complex128" else 0, descs) if backend.blocked else len(descs)
    pass_bytes = (npasses * 2 * 2**n * S) if backend.blocked else gbytes
    state = DeviceState(n, dtype)
    allq = list(range(n))

    # device-resident sampler output (no D2H inside the device-timed step)
    from qibo_gb300.device import DeviceArray
    samp = DeviceArray((NSHOTS,), np.int64, rt)

    def device_step(seed):
        check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
        eng.apply_many(state, descs, blocked=backend.blocked)
        probs = eng.probabilities(state, allq)
        check(lib.qgb_sample(probs.ptr, n, NSHOTS, seed, samp.ptr, None, rt.scratch(lib.qgb_sample_scratch_bytes(n)),
                             rt.stream))
        return probs

    ev = []
    for _ in range(2):
        import ctypes as C
        e = C.c_void_p()
        check(lib.qgb_event_create(C.byref(e)))
        ev.append(e)
    for w in range(args.warmup):
        device_step(1000 + w)
    rt.synchronize()
    if world > 1:
        dist.barrier()
    launches0 = lib.qgb_launch_count()
    clocks = Clocks()
    clocks.start()
    check(lib.qgb_event_record(ev[0], rt.stream))
    for s in range(args.steps):
        device_step(s)
    check(lib.qgb_event_record(ev[1], rt.stream))
    rt.synchronize()
    import ctypes as C
    ms = C.c_float()
    check(lib.qgb_event_elapsed_ms(ev[0], ev[1], C.byref(ms)))
    clk = clocks.stop()
    launches = lib.qgb_launch_count() - launches0
    ms_step = ms.value / args.steps
    if world > 1:
        import torch
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    total_bytes = gbytes + mbytes
    value = total_bytes / (ms_step * 1e-3) / 1e9 * world

    # dominant kernel, CUDA events on the launch stream: the gate passes of one
    # circuit (k_pass launches in blocked mode, per-gate kernels otherwise)
    check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
    check(lib.qgb_event_record(ev[0], rt.stream))
    eng.apply_many(state, descs, blocked=backend.blocked)
    check(lib.qgb_event_record(ev[1], rt.stream))
    check(lib.qgb_event_elapsed_ms(ev[0], ev[1], C.byref(ms)))
    gate_ms = ms.value
    k_ms = gate_ms / max(1, npasses)
    k_bytes = pass_bytes / max(1, npasses)
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    roof = {"bound": "hbm", "achieved": k_bytes / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": k_bytes / (k_ms * 1e-3) / 1e9 / peak, "traffic": None,
            "kernel": "k_pass (shared-memory multi-gate pass)" if backend.blocked else "per-gate kernels",
            "per_launch_bytes": k_bytes, "launches": npasses,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback"}

    # end to end through the public API: host circuit in, 1e6 samples out
    e2e_times = []
    for s in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        res = backend.execute_circuit(run_circ if mode == "fused" else circ, nshots=NSHOTS)
        p = eng.probabilities(res.state(), allq)
        smp = eng.sample(p, NSHOTS, 77 + s, counts=False)
        e2e_times.append(time.perf_counter() - t0)
        del res, p
    e2e_s = statistics.median(e2e_times)
    coef_bytes = sum(16 * d[2].size for d in descs)

    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128" if dtype == "complex128" else "c64", "data": "synthetic",
            "config": {"workload": f"random U3+CZ brickwork n={n} depth {DEPTH} seed {SEED} + {NSHOTS} shots",
                       "mode": mode, "gates": len(gates), "state_passes": npasses,
                       "bytes": "effective: per-gate algorithmic bytes of the unfused circuit + probabilities + CDF",
                       "l2": "state 2^n*S >> L2 (no flush needed)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "circuits_per_s": 1e3 / ms_step, "gpu_launches": launches,
            "gate_ms": gate_ms, "pass_gbs": pass_bytes / (gate_ms * 1e-3) / 1e9,
            "roofline": roof, "clocks": clk,
            "e2e": {"value": total_bytes / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": coef_bytes,
                    "d2h_bytes_per_step": NSHOTS * 8, "seconds": e2e_s}}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
