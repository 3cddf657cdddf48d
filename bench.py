"""Benchmark of the qibo state-vector hot path on one GB300.

Default workload (one "step"): the 30-qubit random circuit of depth 20 — per
layer U3(theta, phi, lambda) on every qubit with angles uniform in [0, 2 pi)
from a seeded generator, then CZ on brickwork pairs — from |0...0> in
complex128, followed by 1e6 shots on all 30 qubits drawn from |psi|^2.

``value`` is the state-vector bandwidth of the step: the algorithmic bytes
of the launches the plan makes -- zeroing (2^n * 16 B), every state pass (a
fused 5-qubit block reads and writes every amplitude once, 2 * 2^n * 16 B),
the complex128 fixed-point chain's norm and two conversions (5 * 2^n * 16
B), probabilities (read 2^n * 16 B, write 2^n * 8 B) and the CDF (2 * 2^n *
8 B) -- divided by the device time of the step with the state resident.
``effective_gbs`` counts instead the bytes a gate-by-gate execution of the
unfused circuit would move (dense 1-qubit gate 2 * 2^n * 16 B, CZ 2 *
2^(n-2) * 16 B).  The state (17.2 GB) is far larger than L2 (129 MB), so no
L2 flush is needed between steps.

``e2e`` is the same metric through the public API with host buffers:
``backend.execute_circuit(circuit, nshots=1e6)`` with the 1e6 samples read
back to the host every step.  The line also carries the complex64 run of the
same circuit with its infidelity against the complex128 state, and a
bounded sample of the serving stream (circuits/s, p50/p99).

Other workloads (``--workload``): ``qft20``, ``vqe24``, ``serving``, ``tc5``,
``memlimit``, ``kernels`` (every hot-path call alone, with its roofline).
``--impl reference`` times the reference's CPU algorithm (the numpy
restatement in ``oracle/``, all host cores) on one layer of the same circuit,
gate by gate, with the per-gate bytes of the passes it runs.
"""

from __future__ import annotations

import argparse
import collections
import ctypes as C
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
                                          "-i", os.environ.get("LOCAL_RANK", "0"), "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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


def reference_nqubits():
    """Qubits of the CPU reference runs: the circuit's 30 when the host has
    room for the reference algorithm's state copies (about 3 x 17.2 GB in
    complex128; 100 GB free asked), else 28."""
    try:
        free = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError):
        free = 0
    return N_QUBITS if free >= 100 * 2**30 else 28


class ReferenceLayer:
    """The reference algorithm (oracle port: transpose, zgemm, transpose per
    gate, backends/abstract.py:2350-2355) on layer 0 of the brickwork circuit
    (n U3 then CZ on pairs (0,1), (2,3), ...: 30 + 15 gates at n = 30), gate
    by gate on a uniform state, with the per-gate algorithmic bytes of the
    passes it runs (one per gate: U3 2 * 2^n * 16 B, CZ 2 * 2^(n-2) * 16 B).
    ``run(k)`` applies the next k gates of the layer, wrapping around."""

    def __init__(self, n, dtype="complex128"):
        from oracle import numpy_ref as ref

        self.ref, self.n, self.dtype = ref, n, dtype
        self.ops = ref.brickwork_ops(n, 1, SEED)
        self.mats = [ref.gate_matrix(nm, p, dtype) for nm, _, p in self.ops]
        self.st = np.full(2**n, 1 / np.sqrt(2**n), dtype=dtype)
        self.pos = 0
        self.seconds = 0.0
        self.bytes = 0
        self.counts = collections.Counter()

    def run(self, k):
        S = np.dtype(self.dtype).itemsize
        n = self.n
        for _ in range(k):
            nm, q, _ = self.ops[self.pos]
            t0 = time.perf_counter()
            self.st = self.ref.apply_gate(self.st, self.mats[self.pos], q, n)
            self.seconds += time.perf_counter() - t0
            self.bytes += 2 * 2**n * S if nm == "U3" else 2 * 2**(n - 2) * S
            self.counts[nm] += 1
            self.pos = (self.pos + 1) % len(self.ops)

    def gbs(self):
        return self.bytes / self.seconds / 1e9

    def describe(self):
        return (f"{self.counts['U3']} U3 + {self.counts['CZ']} CZ of layer 0 ({len(self.ops)} gates), n={self.n}, "
                f"{self.dtype}, numpy/OpenBLAS (reference NumpyBackend algorithm), {self.seconds:.2f} s")


def cpu_baseline_sample(n=None, ngates=6):
    """A bounded sample (about 10-30 s) of the reference algorithm on the
    circuit's layer 0: its first ``ngates`` gates."""
    lay = ReferenceLayer(n or reference_nqubits())
    lay.run(ngates)
    return {"value": lay.gbs(), "unit": "GB/s", "cores": os.cpu_count(), "kind": "port", "sample": lay.describe()}


def run_reference(args):
    """The reference's own CPU algorithm for this path on the same circuit:
    layer 0 of the random U3+CZ brickwork at n = 30 (28 if the host lacks
    memory), three gates per step in layer order, the steps wrapping around
    the layer (15 steps cover it).  value = sum of bytes over sum of seconds
    of the timed steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = reference_nqubits()
    warm = ReferenceLayer(24)
    warm.run(max(1, args.warmup))
    lay = ReferenceLayer(n)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lay.run(3)
    dt = time.perf_counter() - t0
    v = lay.gbs()
    per_gate_s = lay.seconds / max(1, sum(lay.counts.values()))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic",
            "config": {"workload": f"one layer (layer 0: {n} U3 + {n // 2} CZ) of the random U3+CZ brickwork "
                                   f"n={n} depth {DEPTH} seed {SEED}, gate by gate, 3 gates per step in layer order",
                       "nqubits": n, "gates_timed": 3 * args.steps, "layer_gates": len(lay.ops),
                       "bytes": "per-gate algorithmic bytes of the passes this algorithm runs, one per gate "
                                "(U3 2*2^n*16 B, CZ 2*2^(n-2)*16 B)",
                       "difference": "the GPU arm runs all 20 layers and 1e6 shots; this arm times layer 0 (the "
                                     "per-gate rate is the same in every layer) as a bounded sample",
                       "seconds_per_circuit_estimate": per_gate_s * 890},
            "cpu_baseline": {"kind": "port", "cores": os.cpu_count(), "sample": lay.describe(), "value": v,
                             "unit": "GB/s"},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


class Events:
    def __init__(self, lib):
        from qibo_gb300._lib import check

        self.lib, self.check = lib, check
        self.a, self.b = C.c_void_p(), C.c_void_p()
        check(lib.qgb_event_create(C.byref(self.a)))
        check(lib.qgb_event_create(C.byref(self.b)))

    def start(self, stream):
        self.check(self.lib.qgb_event_record(self.a, stream))

    def stop_ms(self, stream) -> float:
        self.check(self.lib.qgb_event_record(self.b, stream))
        ms = C.c_float()
        self.check(self.lib.qgb_event_elapsed_ms(self.a, self.b, C.byref(ms)))
        return ms.value


def serving_sample(nreq: int, rates, baseline: bool = True, nbase: int = 120, c64: bool = True):
    """Bounded sample of the serving stream: ``nreq`` requests with qubits
    uniform in [10, 28], depth uniform in [5, 30], mixed complex64/complex128
    tags and outputs (state, 1e4 shots, Z-string expectation), served at each
    Poisson arrival rate in ``rates`` (the same requests; only the arrival
    times scale with the rate).  The highest rate is a burst: every request is
    waiting at once, so circuits/s there is the server's throughput.  Then the
    same requests tagged complex64 (engine fusion, 3xTF32 tensor-core blocks),
    and the one-at-a-time complex128 per-gate path on the first ``nbase`` of
    them (tagged complex128) as the baseline; the infidelity of the complex64
    states against the baseline's complex128 states is the largest over the
    state outputs of <= 24 qubits among those."""
    from qibo_gb300.serving import Request, Server, make_stream

    def retag(reqs, dtype):
        return [Request(r.rid, r.nqubits, dtype, r.ops, r.coefs, r.shape, r.output, r.nshots, r.zmask, r.seed,
                        r.arrival) for r in reqs]

    def keep_states(reqs):
        return {r.rid: r.result for r in reqs if r.output == "state" and r.nqubits <= 24}

    srv = Server(keep_states=c64)  # a long stream's states reach the host and are dropped there
    out = {"requests": nreq, "by_rate": [], "states_kept_on_host": c64}
    try:
        warm = make_stream(16, 0.0, seed=7, nmin=10, nmax=18, dmin=5, dmax=6)
        srv.run(warm + retag(warm, "complex64"), realtime=False)
        for rate in rates:
            srv.stats.clear()
            st = srv.run(make_stream(nreq, rate, seed=2026), realtime=True)
            out["by_rate"].append({"arrival_rate_per_s": rate, "circuits_per_s": st["circuits_per_s"],
                                   "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                                   "batched": st.get("batched_requests", 0), "fused": st.get("fused", 0),
                                   "graph_replays": st.get("graph_replays", 0)})
        c64_states = {}
        if c64:
            c64r = retag(make_stream(nreq, max(rates), seed=2026), "complex64")
            srv.stats.clear()
            st = srv.run(c64r, realtime=True)
            out["complex64_only"] = {"arrival_rate_per_s": max(rates), "circuits_per_s": st["circuits_per_s"],
                                     "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"]}
            c64_states = keep_states(c64r[:nbase])
            del c64r
    finally:
        srv.close()
    best = max(out["by_rate"], key=lambda d: d["circuits_per_s"])
    out.update({"circuits_per_s": best["circuits_per_s"], "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"],
                "arrival_rate_per_s": best["arrival_rate_per_s"]})
    if baseline:
        base = retag(make_stream(nreq, max(rates), seed=2026)[:nbase], "complex128")  # same requests, all waiting
        srv = Server(one_at_a_time=True)
        try:
            bst = srv.run(base, realtime=False)
        finally:
            srv.close()
        inf = 0.0
        for r in base:
            if r.rid in c64_states:
                a = r.result.astype(np.complex128)
                b = c64_states[r.rid].astype(np.complex128)
                inf = max(inf, 1.0 - abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real))
        out["baseline_one_at_a_time_c128_per_gate"] = {"requests": len(base), "circuits_per_s": bst["circuits_per_s"],
                                                        "p50_ms": bst["p50_ms"], "p99_ms": bst["p99_ms"],
                                                        "note": f"the first {len(base)} requests of the same stream"}
        out["speedup_vs_baseline"] = out["circuits_per_s"] / bst["circuits_per_s"]
        if c64:
            out["complex64_only"]["speedup_vs_baseline"] = out["complex64_only"]["circuits_per_s"] / bst["circuits_per_s"]
            out["complex64_only"]["max_infidelity_vs_c128"] = inf
    return out


def analytic_check(backend, n, dtype, depth=DEPTH, seed=SEED):
    """Max-abs error of the engine against a closed-form answer at the
    benchmark's size: U3 on every qubit (a product state), the depth-20
    brickwork and its inverse, with engine fusion; the product state must
    come back.  Checked at 4096 random indices plus both ends."""
    from qibo_gb300 import Circuit, gates

    ang = np.random.default_rng(seed + 1).uniform(0, 2 * np.pi, (n, 3))
    u = np.array([gates.U3(0, *a).matrix()[:, 0] for a in ang])
    layer = [gates.U3(q, *ang[q]) for q in range(n)]
    bw = brickwork_gates(n, depth, seed)
    inv = []
    for g in reversed(bw):
        if type(g).__name__ == "U3":
            th, ph, la = g.parameters
            inv.append(gates.U3(g.target_qubits[0], -th, -la, -ph))
        else:
            inv.append(g)
    c = Circuit(n)
    c.add(layer + bw + inv)
    st = backend.execute_circuit(c).state()
    rng = np.random.default_rng(3)
    idx = np.unique(np.concatenate([rng.integers(0, 2**n, 4096, dtype=np.int64), [0, 2**n - 1]]))
    bits = (idx[:, None] >> (n - 1 - np.arange(n))[None, :]) & 1
    want = np.prod(u[np.arange(n)[None, :], bits], axis=1)
    err = float(np.max(np.abs(st.take(idx) - want)))
    del st
    return {"circuit": f"U3 on every qubit, the depth-{depth} brickwork (seed {seed}) and its inverse, engine fusion",
            "answer": "the product state of the U3 layer (closed form)", "indices": int(idx.size),
            "max_abs_error": err, "tolerance": 1e-12 if dtype == "complex128" else 1e-5}


def complex64_legs(args, n, circ, descs, state, backend, ev, ndense, ncz, runs=8):
    """complex64 legs of the brickwork circuit against complex128.

    ``passes``: the unfused gate list in shared-memory passes.  ``fused_tc``:
    the gate list fused by the engine (QGB_PLAN_FUSE), whose uncontrolled
    5-qubit blocks run on the tensor cores (3xTF32) and the rest in passes; ``runs`` device-timed circuits give
    p50/p99.  Both results are renormalised in FP64 and compared with the
    complex128 blocked result (infidelity 1 - |<psi128|psi64>|^2).
    ``c128_per_gate_ms`` is one run of the plain complex128 per-gate path
    (IEEE FP64, one kernel per gate), the comparison point of the fused leg;
    ``c128_per_gate_double_float`` the same passes with dense gates in
    double-float, with the per-gate-pass bandwidth (algorithmic bytes of
    the gates over the device time)."""
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend, describe_gate
    from qibo_gb300.device import DeviceArray, DeviceState

    rt, eng, lib = backend.rt, backend.engine_gb, backend.rt.lib
    b64 = GB300Backend("complex64")
    st64 = DeviceState(n, "complex64")
    out = DeviceArray((2,), np.float64, rt)
    fdescs = [describe_gate(g, b64) for g in circ.fuse(5).queue]  # for one representative 5-qubit block
    nfused, n5 = b64.engine_gb.fuse_stats(descs, n if n >= 12 else 0)  # the engine's fusion of the gate list

    def infidelity():
        check(lib.qgb_inner_mixed(state.ptr, state.code, st64.ptr, st64.code, n, out.ptr,
                                  rt.scratch(lib.qgb_inner_scratch_bytes()), rt.stream))
        re, im = out.to_numpy()
        return 1.0 - (re * re + im * im)

    def timed(dl, reps, fuse=False):
        ms = []
        for _ in range(reps):
            check(lib.qgb_state_zero(st64.ptr, n, st64.code, rt.stream))
            ev.start(rt.stream)
            b64.engine_gb.apply_many(st64, dl, blocked=True, fuse=fuse)
            ms.append(ev.stop_ms(rt.stream))
        return ms

    # complex128 reference state: the unfused gate list in double-float passes
    check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
    ev.start(rt.stream)
    eng.apply_many(state, descs, blocked=True)
    ms_128b = ev.stop_ms(rt.stream)
    timed(descs, 2)
    ms_p = timed(descs, 1)[0]
    norm_p = b64.engine_gb.renormalize(st64)  # FP64 renormalisation of the complex64 result
    inf_p = infidelity()
    timed(descs, 2, fuse=True)
    ms_f = sorted(timed(descs, runs, fuse=True))
    norm_f = b64.engine_gb.renormalize(st64)
    inf_f = infidelity()
    # the tensor-core kernel alone: 10 launches of the first 5-qubit block
    tc_gbs = tc_kernel = None
    blk = next((d for d in fdescs if len(d[0]) == 5 and not d[1]), None)
    if blk is not None:
        from qibo_gb300 import _lib

        qs = _lib.int_array(blk[0])
        mat = np.ascontiguousarray(np.asarray(blk[2], dtype=np.complex128)).view(np.float64).ravel()
        mp = mat.ctypes.data_as(_lib.dp)
        check(lib.qgb_apply_fused5_tc(st64.ptr, n, st64.code, qs, mp, rt.stream))
        ev.start(rt.stream)
        for _ in range(10):
            check(lib.qgb_apply_fused5_tc(st64.ptr, n, st64.code, qs, mp, rt.stream))
        tc_ms = ev.stop_ms(rt.stream) / 10
        tc_gbs = 2 * 2**n * 8 / (tc_ms * 1e-3) / 1e9
        tc_kernel = tc64_kernel(n, blk[0])
    tc_timeout = C.c_int(0)
    check(lib.qgb_tc_status(C.byref(tc_timeout)))
    # plain complex128 per-gate path: IEEE FP64, one kernel per gate (state
    # reused: the references above are done)
    check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
    ev.start(rt.stream)
    eng.apply_many(state, descs, blocked=False, strict_fp64=True)
    ms_g = ev.stop_ms(rt.stream)
    del st64
    st2 = DeviceState(n, "complex128")

    def inf_vs_per_gate():  # 1 - |<psi_per_gate|psi>|^2 in FP64
        check(lib.qgb_inner(state.ptr, st2.ptr, n, state.code, out.ptr, rt.scratch(lib.qgb_inner_scratch_bytes()),
                            rt.stream))
        re2, im2 = out.to_numpy()
        return 1.0 - (re2 * re2 + im2 * im2)

    # the same gates one pass each, dense gates in double-float
    check(lib.qgb_state_zero(st2.ptr, n, st2.code, rt.stream))
    ev.start(rt.stream)
    eng.apply_many(st2, descs, blocked=False)
    ms_df = ev.stop_ms(rt.stream)
    inf_df = inf_vs_per_gate()
    # the fused complex128 result (tensor-core blocks)
    check(lib.qgb_state_zero(st2.ptr, n, st2.code, rt.stream))
    eng.apply_many(st2, descs, blocked=True, fuse=True)
    inf_128 = inf_vs_per_gate()
    del st2
    g128, _ = algorithmic_bytes(n, ndense, ncz, 16)
    g64, _ = algorithmic_bytes(n, ndense, ncz, 8)
    p50 = statistics.median(ms_f)
    p99 = ms_f[min(len(ms_f) - 1, int(np.ceil(0.99 * len(ms_f))) - 1)]
    return {"passes": {"gate_ms": ms_p, "value": g64 / (ms_p * 1e-3) / 1e9, "unit": "GB/s",
                       "infidelity_vs_c128": inf_p, "norm_before_renormalisation": norm_p},
            "fused_tc": {"fusion": "engine (QGB_PLAN_FUSE)", "fused_ops": nfused, "tc_blocks_5q": n5, "runs": runs,
                         "p50_ms": p50, "p99_ms": p99,
                         "circuits_per_s": 1e3 / p50, "infidelity_vs_c128": inf_f,
                         "norm_before_renormalisation": norm_f, "tc_wait_timeouts": tc_timeout.value,
                         "k_fused5_tc_gbs": tc_gbs, "k_fused5_tc_bytes_per_launch": 2 * 2**n * 8,
                         "k_fused5_tc_note": f"first 5-qubit block of the circuit, 10 launches ({tc_kernel})",
                         "p99_note": "p99 of 8 runs is the slowest run"},
            "c128_per_gate_ms": ms_g, "c128_unfused_passes_ms": ms_128b,
            "c128_per_gate_double_float": {
                "ms": ms_df, "GB/s": g128 / (ms_df * 1e-3) / 1e9,
                "frac_of_hbm_peak": g128 / (ms_df * 1e-3) / 1e9 / measured_peaks().get("hbm_gbs", 6800.0),
                "infidelity_vs_per_gate_fp64": inf_df,
                "note": "one pass per gate; dense 1-qubit gates with 2 of every 8 warps per scheduler in IEEE "
                        "FP64 and 6 in double-float, loads staged through shared memory by cp.async; dense "
                        "2-qubit gates in double-float; CZ by sign flips"},
            "c128_fused_infidelity_vs_per_gate_fp64": inf_128,
            "fused_tc_speedup_vs_c128_per_gate": ms_g / p50}


def run_brickwork(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")

    from qibo_gb300 import Circuit
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend, describe_gate
    from qibo_gb300.device import DeviceArray, DeviceState

    n, dtype = args.nqubits, args.dtype
    S = 16 if dtype == "complex128" else 8
    backend = GB300Backend(dtype)
    rt, eng, lib = backend.rt, backend.engine_gb, backend.rt.lib
    gates = brickwork_gates(n, DEPTH, SEED)
    circ = Circuit(n)
    circ.add(gates)
    mode = args.mode if args.mode != "auto" else ("engine" if n >= 12 else "blocked")
    t0 = time.perf_counter()
    run_circ = circ.fuse(5) if mode == "fused" else circ
    fuse_s = time.perf_counter() - t0
    descs = [describe_gate(g, backend) for g in run_circ.queue]
    udescs = descs if run_circ is circ else [describe_gate(g, backend) for g in circ.queue]
    backend.blocked = mode in ("blocked", "fused", "engine")
    backend.fuse = mode == "engine"
    efuse = mode == "engine"
    ndense = sum(1 for g in gates if type(g).__name__ == "U3")
    ncz = len(gates) - ndense
    gbytes, mbytes = algorithmic_bytes(n, ndense, ncz, S)
    code = 1 if dtype == "complex128" else 0
    # state passes the engine makes: tensor-core blocks (uncontrolled 5-qubit
    # dense ops) one each, the ops between them planned into shared-memory passes
    is_tc = [mode == "fused" and len(d[0]) == 5 and not d[1] for d in descs]
    n_tc, npasses, seg = sum(is_tc), 0, []
    for d, tc in zip(descs + [None], is_tc + [True]):
        if tc:
            npasses += eng.count_passes(n, code, seg) if (seg and backend.blocked) else len(seg)
            seg = []
        else:
            seg.append(d)
    npasses += n_tc
    if efuse:  # the engine's own fusion: its 5-qubit blocks and other ops
        nfused, n_tc = eng.fuse_stats(descs, n if n >= 12 else 0)
        npasses = nfused
    pass_bytes = (npasses * 2 * 2**n * S) if backend.blocked else gbytes
    state = DeviceState(n, dtype)
    allq = list(range(n))
    samp = DeviceArray((NSHOTS,), np.int64, rt)

    def device_step(seed):
        check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
        eng.apply_many(state, descs, blocked=backend.blocked, fuse=efuse)
        probs = eng.probabilities(state, allq)
        check(lib.qgb_sample(probs.ptr, n, NSHOTS, seed, samp.ptr, None, rt.scratch(lib.qgb_sample_scratch_bytes(n)),
                             rt.stream))
        return probs

    ev = Events(lib)
    for w in range(args.warmup):
        device_step(1000 + w)
    rt.synchronize()
    if dist is not None:
        dist.barrier()
    launches0 = lib.qgb_launch_count()
    clocks = Clocks()
    clocks.start()
    ev.start(rt.stream)
    for s in range(args.steps):
        device_step(s)
    ms_total = ev.stop_ms(rt.stream)
    rt.synchronize()
    clk = clocks.stop()
    launches = lib.qgb_launch_count() - launches0
    ms_step = ms_total / args.steps
    if dist is not None:
        import torch

        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    # physical algorithmic bytes of the plan that runs, every launch of the
    # step: zeroing, the state passes (each fused op reads and writes the
    # state once), for a complex128 run of tensor-core blocks the fixed-point
    # chain's norm and two conversions, then probabilities and the CDF
    N = 2**n
    nchains = 1 if (efuse and S == 16 and n_tc >= 2) else 0
    plan_bytes = N * S + pass_bytes + nchains * 5 * N * S + mbytes
    value = plan_bytes / (ms_step * 1e-3) / 1e9 * world
    # the per-gate bytes of the unfused circuit over the same time
    effective_gbs = (gbytes + mbytes) / (ms_step * 1e-3) / 1e9 * world

    # the gate passes of one circuit, CUDA events on the launch stream
    check(lib.qgb_state_zero(state.ptr, n, state.code, rt.stream))
    ev.start(rt.stream)
    eng.apply_many(state, descs, blocked=backend.blocked, fuse=efuse)
    gate_ms = ev.stop_ms(rt.stream)
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_source = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"
    if n_tc:
        # dominant kernel: the tensor-core block kernel, 10 launches of the
        # circuit's first block, CUDA events on the launch stream
        from qibo_gb300 import _lib

        # a representative 5-qubit block of the circuit (the Python packer's
        # first one; the kernel's cost does not depend on which)
        blk = next(d for d in (describe_gate(g, backend) for g in circ.fuse(5).queue) if len(d[0]) == 5 and not d[1])
        qs = _lib.int_array(blk[0])
        mat = np.ascontiguousarray(np.asarray(blk[2], dtype=np.complex128)).view(np.float64).ravel()
        mp = mat.ctypes.data_as(_lib.dp)
        if S == 16:
            # the circuit runs its complex128 blocks as fixed-point chains: a
            # chain of 10 minus a chain of 2, over 8, cancels the norm and the
            # two conversion passes
            def chain_ms(k):
                eng.apply_many(state, [blk] * k, blocked=True)
                ev.start(rt.stream)
                eng.apply_many(state, [blk] * k, blocked=True)
                return ev.stop_ms(rt.stream)

            k_ms = (chain_ms(10) - chain_ms(2)) / 8
        else:
            check(lib.qgb_apply_fused5_tc(state.ptr, n, state.code, qs, mp, rt.stream))
            ev.start(rt.stream)
            for _ in range(10):
                check(lib.qgb_apply_fused5_tc(state.ptr, n, state.code, qs, mp, rt.stream))
            k_ms = ev.stop_ms(rt.stream) / 10
        k_bytes = 2 * 2**n * S
        # dram bytes of one launch at n=28 from ncu, scaled by 2^(n-28)
        traffic28 = (4.295e9 + 4.233e9) if S == 16 else (2.148e9 + 2.086e9)
        kname = "k_fused5_oz<fixed-point> (complex128 Ozaki scheme on BF16 tensor cores)" if S == 16 else \
            "k_fused5_tc (complex64 3xTF32 tensor cores)"
        roof = {"bound": "hbm", "achieved": k_bytes / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": k_bytes / (k_ms * 1e-3) / 1e9 / peak, "traffic": traffic28 * 2 ** (n - 28),
                "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one launch from ncu at n=28, "
                                "scaled by 2^(n-28); equals the algorithmic bytes",
                "kernel": kname, "per_launch_bytes": k_bytes, "launches": n_tc, "ms_per_launch": k_ms,
                "share_of_gate_time": n_tc * k_ms / gate_ms, "peak_source": peak_source}
    else:
        k_ms = gate_ms / max(1, npasses)
        k_bytes = pass_bytes / max(1, npasses)
        roof = {"bound": "hbm", "achieved": k_bytes / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": k_bytes / (k_ms * 1e-3) / 1e9 / peak,
                "traffic": 2.09e9 * (2 ** (n - 26)) if n >= 26 else None,
                "traffic_note": "dram bytes per k_pass launch from ncu at n=26 (1.075 GB read + 1.014 GB write), "
                                "scaled by 2^(n-26); equals the algorithmic bytes",
                "kernel": "k_pass (shared-memory multi-gate pass)" if backend.blocked else "per-gate kernels",
                "per_launch_bytes": k_bytes, "launches": npasses, "peak_source": peak_source}

    # end to end through the public API: host circuit in, 1e6 samples out
    e2e_times = []
    for s in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        res = backend.execute_circuit(run_circ, nshots=NSHOTS)
        p = eng.probabilities(res.state(), allq)
        eng.sample(p, NSHOTS, 77 + s, counts=False)
        e2e_times.append(time.perf_counter() - t0)
        del res, p
    e2e_s = statistics.median(e2e_times)
    coef_bytes = sum(16 * d[2].size for d in descs)

    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128" if dtype == "complex128" else "c64", "data": "synthetic",
            "config": {"workload": f"random U3+CZ brickwork n={n} depth {DEPTH} seed {SEED} + {NSHOTS} shots",
                       "mode": mode, "gates": len(gates), "state_passes": npasses, "tensor_core_blocks": n_tc,
                       "fusion": ("qibo Circuit.fuse(max_qubits=5), once before timing "
                                  f"({fuse_s:.2f} s, {len(descs)} blocks)") if mode == "fused" else
                                 (f"engine (QGB_PLAN_FUSE, inside every qgb_apply_circuit call): {len(descs)} gates -> "
                                  f"{npasses} ops, {n_tc} 5-qubit blocks") if efuse else "none",
                       "arithmetic": (("5-qubit blocks: Ozaki scheme on BF16 tensor cores (47-bit fixed point, "
                                       "exact level sums, IEEE doubles out); " if n_tc and S == 16 else "")
                                      + ("double-float (FP32 pipe) in passes, IEEE FP64 reductions"
                                         if dtype == "complex128" and backend.blocked and not backend.strict_fp64
                                         else "native")),
                       "bytes": (f"physical: the plan's launches -- zeroing (2^n*S), {npasses} state passes "
                                 f"(2*2^n*S each), {nchains} fixed-point chain(s) (norm + two conversions, "
                                 "5*2^n*S), probabilities (2^n*S + 2^n*8) and CDF (2*2^n*8); S = "
                                 f"{S} B; {plan_bytes / 1e9:.1f} GB per step"),
                       "l2": "state 2^n*S >> L2 (no flush needed)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "circuits_per_s": 1e3 / ms_step, "gpu_launches": launches,
            "effective_gbs": effective_gbs,
            "effective_note": "per-gate algorithmic bytes of the unfused 890-gate circuit (what a gate-by-gate "
                              "run would move) + probabilities + CDF, over the same time; above the HBM peak "
                              "because fusion moves far fewer bytes",
            "gate_ms": gate_ms, "pass_gbs": pass_bytes / (gate_ms * 1e-3) / 1e9,
            "roofline": roof, "clocks": clk,
            "e2e": {"value": plan_bytes / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": coef_bytes,
                    "d2h_bytes_per_step": NSHOTS * 8, "seconds": e2e_s}}

    if rank == 0 and not args.quick:
        line["analytic_check"] = analytic_check(backend, n, dtype)
    if dtype == "complex128" and rank == 0 and not args.quick:
        line["complex64"] = complex64_legs(args, n, circ, udescs, state, backend, ev, ndense, ncz)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
    if rank == 0 and world == 1 and args.serving_requests > 0:
        del state
        line["serving"] = serving_sample(args.serving_requests, args.serving_rates)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_qft20(args):
    """QFT(20) in complex128 on a seeded complex Gaussian state + 1e5 shots."""
    from qibo_gb300 import QFT
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    n = 20
    psi = np.random.default_rng(20).normal(size=2**n) + 1j * np.random.default_rng(21).normal(size=2**n)
    psi /= np.linalg.norm(psi)
    backend = GB300Backend("complex128")
    c = QFT(n)
    backend.set_seed(1234)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        res = backend.execute_circuit(c, psi)
        p = backend.calculate_probabilities(res.state(), list(range(n)), n)
        backend.sample_frequencies(p, 100_000)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    s = statistics.median(times)
    print(json.dumps({"workload": "QFT(20) complex128 + 1e5 shots, through the public API", "seconds": s,
                      "reference_published_v100_s": 0.03881, "unit": "s", "higher_is_better": False}))


def run_vqe24(args):
    """24-qubit hardware-efficient ansatz (10 layers RY+RZ + CNOT ladder, 480
    parameters), periodic TFIM h=1: energy and all 480 adjoint gradients."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.adjoint import adjoint_gradient
    from qibo_gb300.backend import GB300Backend

    n, layers = 24, 10
    p = np.random.default_rng(24).uniform(-np.pi, np.pi, 2 * n * layers)
    # periodic TFIM, h = 1 (hamiltonians/models.py:649-662): -sum Z_i Z_i+1 - sum X_i
    ham = (["ZZ"] * n + ["X"] * n, [(i, (i + 1) % n) for i in range(n)] + [(i,) for i in range(n)],
           [-1.0] * (2 * n))
    out = {}
    for dtype in ("complex128", "complex64"):
        b = GB300Backend(dtype)
        c = Circuit(n)
        k = 0
        for _ in range(layers):  # RY then RZ on every qubit, then a CNOT ladder
            for q in range(n):
                c.add(gates.RY(q, float(p[k])))
                c.add(gates.RZ(q, float(p[k + 1])))
                k += 2
            for q in range(n - 1):
                c.add(gates.CNOT(q, q + 1))
        times = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            e, g = adjoint_gradient(b, c, ham)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        out[dtype] = {"energy": e, "grad_norm": float(np.linalg.norm(g)), "seconds": statistics.median(times)}
    print(json.dumps({"workload": "VQE24: energy + 480 adjoint gradients", **out}))


def run_serving(args):
    """The serving stream at the size given (``--serving-requests``; the
    configuration's full stream is 20,000) at each rate of
    ``--serving-rates``, with the complex64 retag and the one-at-a-time
    complex128 per-gate baseline on the first 120 requests."""
    big = args.serving_requests > 2000
    print(json.dumps({"workload": f"serving stream, {args.serving_requests} requests",
                      **serving_sample(args.serving_requests, args.serving_rates, c64=not big)}))


def tc64_kernel(n, qubits):
    """The complex64 block kernel and lane layout the launcher picks for a
    block on ``qubits`` (tcm_plan in qgb_tc.cu)."""
    if n < 12:
        return "k_fused5_tc"
    bits = sorted(n - 1 - q for q in qubits)
    low4 = sum(b < 4 for b in bits)
    strided = 0.45 if {0, 1} <= set(bits) or low4 > 2 else (0.945, 0.94, 0.84)[low4]
    grp = [b for b in range(n) if b not in bits][:5]
    k = sum(b in bits[:4] for b in sorted(grp + bits[:4])[:5])
    shfl = 0.955 if k <= 1 else 0.895 if k == 2 else 0.78 if k == 3 else 0.72
    if max(strided, shfl) <= 0.74:
        return "k_fused5_tc"
    return "k_fused5_tcm (coalesced lanes)" if shfl > strided else "k_fused5_tcm (strided lanes)"


def run_tc5(args):
    """The tensor-core block kernels alone: a random 5-qubit unitary applied to
    a state of ``--nqubits`` qubits (default 30; 8.6 GB in complex64, 17.2 GB
    in complex128, inputs >> L2), one launch per step, for three placements
    of the block qubits (lowest index bits, highest, spread), in complex64
    (k_fused5_tc, 3xTF32) and complex128 (k_fused5_oz, Ozaki scheme on BF16;
    single launches on IEEE doubles, and a chain of 10 blocks in the
    fixed-point format through qgb_apply_circuit), on a dense state.
    Algorithmic bytes per launch: 2 * 2^n * S."""
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    n = args.nqubits
    b = GB300Backend("complex64")
    rt, lib = b.rt, b.rt.lib
    rng = np.random.default_rng(5)
    z = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    u, _ = np.linalg.qr(z)
    mat = np.ascontiguousarray(u.astype(np.complex128)).view(np.float64).ravel()
    mp = mat.ctypes.data_as(_lib.dp)
    peak = measured_peaks().get("hbm_gbs", 6800.0)
    ev = Events(lib)
    out = {}
    for dtype, kernel, S, flops in (("complex64", "k_fused5_tc", 8, 3 * 2 * 64 * 64),
                                     ("complex128", "k_fused5_oz", 16, 26 * 2 * 64 * 64)):
        st = DeviceState(n, dtype)
        check(lib.qgb_state_zero(st.ptr, n, st.code, rt.stream))
        # a dense state (the kernels' cost depends on the data: zero tiles are
        # cheaper): the random unitary on qubits 5k..5k+4 for every k
        for k in range(n // 5):
            check(lib.qgb_apply_fused5_tc(st.ptr, n, st.code, _lib.int_array(range(5 * k, 5 * k + 5)), mp,
                                          rt.stream))
        nbytes = 2 * 2**n * S
        res = {"kernel": kernel, "bytes_per_launch": nbytes}
        for name, qs in (("high_bits", [0, 1, 2, 3, 4]), ("low_bits", [n - 1, n - 2, n - 3, n - 4, n - 5]),
                         ("spread", [1, n // 3, n // 2, n - 3, n - 1])):
            qa = _lib.int_array(qs)
            for _ in range(args.warmup):
                check(lib.qgb_apply_fused5_tc(st.ptr, n, st.code, qa, mp, rt.stream))
            ev.start(rt.stream)
            for _ in range(args.steps):
                check(lib.qgb_apply_fused5_tc(st.ptr, n, st.code, qa, mp, rt.stream))
            ms = ev.stop_ms(rt.stream) / args.steps
            gbs = nbytes / (ms * 1e-3) / 1e9
            kname = kernel
            if dtype == "complex64":
                kname = tc64_kernel(n, qs)
            res[name] = {"qubits": qs, "kernel": kname, "ms": ms, "GB/s": gbs, "frac_of_hbm_peak": gbs / peak,
                         "tensor_tflops": flops * 2 ** (n - 5) / (ms * 1e-3) / 1e12}
        if dtype == "complex64" and n >= 12:
            # both complex64 kernels on placements with 0-5 block qubits on
            # index bits 0..4, k_fused5_tcm with strided and with coalesced
            # lanes (QIBO_GB300_TC64_KERNEL picks the kernel and layout)
            sweep = []
            for bits in ([5, 10, 15, 20, 25], [0, 10, 15, 20, 25], [4, 10, 15, 20, 25], [3, 4, 12, 18, 24],
                         [0, 2, 12, 18, 24], [2, 3, 4, 15, 25], [0, 2, 4, 15, 25], [0, 1, 12, 18, 24],
                         [0, 1, 2, 15, 25], [1, 2, 3, 4, 20], [0, 1, 2, 3, 20], [0, 1, 2, 3, 4]):
                bits = [min(x, n - 5 + i) if x >= 5 else x for i, x in enumerate(bits)]
                qa = _lib.int_array([n - 1 - x for x in bits])
                row = {"index_bits": bits}
                for kname, pick in (("k_fused5_tcm", "tmem-strided"), ("k_fused5_tcm_coalesced", "tmem-shfl"),
                                    ("k_fused5_tc", "smem")):
                    os.environ["QIBO_GB300_TC64_KERNEL"] = pick
                    try:
                        for _ in range(args.warmup):
                            check(lib.qgb_apply_fused5_tc(st.ptr, n, st.code, qa, mp, rt.stream))
                        ev.start(rt.stream)
                        for _ in range(args.steps):
                            check(lib.qgb_apply_fused5_tc(st.ptr, n, st.code, qa, mp, rt.stream))
                        ms = ev.stop_ms(rt.stream) / args.steps
                    finally:
                        del os.environ["QIBO_GB300_TC64_KERNEL"]
                    row[kname] = {"ms": ms, "frac_of_hbm_peak": nbytes / (ms * 1e-3) / 1e9 / peak}
                sweep.append(row)
            res["placement_sweep"] = sweep
        if dtype == "complex128":
            # a chain of 10 unitary blocks through qgb_apply_circuit: the state
            # is converted once to the fixed-point format (norm pass + 2
            # conversion passes, amortised below) and the blocks run on it
            descs = [([1, n // 3, n // 2, n - 3, n - 1], [], u)] * 10
            b128 = GB300Backend("complex128")
            b128.engine_gb.apply_many(st, descs, blocked=True)
            ev.start(rt.stream)
            b128.engine_gb.apply_many(st, descs, blocked=True)
            ms = ev.stop_ms(rt.stream) / 10
            gbs = nbytes / (ms * 1e-3) / 1e9
            res["fixed_point_chain_of_10"] = {"kernel": "k_fused5_oz<fixed-point>", "ms_per_block": ms, "GB/s": gbs,
                                              "frac_of_hbm_peak": gbs / peak,
                                              "note": "includes the norm and the two conversion passes"}
        out[dtype] = res
        del st
    flag = C.c_int(0)
    check(lib.qgb_tc_status(C.byref(flag)))
    print(json.dumps({"workload": f"fused 5-qubit block kernels, n={n}, random 5-qubit unitary",
                      "hbm_peak_gbs": peak, "tc_wait_timeouts": flag.value, **out}))


def run_fusion(args):
    """The engine's fusion rule on both sides of its threshold: QFT (about
    13-15 fused ops per unfused pass) and QFT + depth-10 brickwork (about 9)
    at ``--nqubits`` in both precisions, each gate list run once as
    shared-memory passes and once as fused blocks
    (QIBO_GB300_FUSE_OPS_PER_PASS=0 / 100000), after one untimed run; CUDA
    events on the launch stream.  The engine keeps the fused list at most
    11 ops per pass."""
    from qibo_gb300 import QFT
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend, describe_gate
    from qibo_gb300.device import DeviceState

    n = args.nqubits
    rows = []
    for dtype in ("complex64", "complex128"):
        b = GB300Backend(dtype)
        rt, eng, lib = b.rt, b.engine_gb, b.rt.lib
        ev = Events(lib)
        for name in ("QFT", "QFT + depth-10 brickwork"):
            c = QFT(n)
            if name != "QFT":
                c.add(brickwork_gates(n, 10, n))
            descs = [describe_gate(g, b) for g in c.queue]
            npass = eng.count_passes(n, 1 if dtype == "complex128" else 0, descs)
            nfused, n5 = eng.fuse_stats(descs, n)
            st = DeviceState(n, dtype)
            row = {"circuit": name, "dtype": dtype, "gates": len(descs), "unfused_passes": npass,
                   "fused_ops": nfused, "fused_ops_per_pass": nfused / npass,
                   "engine_plan": "fused" if nfused <= 11 * npass else "passes"}
            for plan, v in (("passes_ms", "0"), ("fused_ms", "100000")):
                os.environ["QIBO_GB300_FUSE_OPS_PER_PASS"] = v
                try:
                    check(lib.qgb_state_zero(st.ptr, n, st.code, rt.stream))
                    eng.apply_many(st, descs, blocked=True, fuse=True)
                    ev.start(rt.stream)
                    eng.apply_many(st, descs, blocked=True, fuse=True)
                    row[plan] = ev.stop_ms(rt.stream)
                finally:
                    del os.environ["QIBO_GB300_FUSE_OPS_PER_PASS"]
            del st
            rows.append(row)
    print(json.dumps({"workload": f"engine fusion rule, n={n}", "rows": rows}))


def run_kernels(args):
    """Every hot-path call alone, on a dense random state of ``--nqubits``
    qubits (default 30: 17.2 GB complex128, 8.6 GB complex64; inputs >> L2),
    in both precisions: ``--warmup`` untimed calls, then ``--steps`` calls
    timed with CUDA events on the launch stream.  Algorithmic bytes per call
    (S = bytes per amplitude, N = 2^n): dense 1- and 2-qubit gates 2 N S; a
    gate touching a fraction f of the amplitudes (CZ 1/4, CNOT and SWAP 1/2,
    a doubly controlled gate 1/4) 2 f N S; a shared-memory pass 2 N S per
    pass; probabilities N S + 2^m 8; norm N S; Pauli expectation N S per
    distinct flip mask; collapse on k qubits 2 N S / 2^k + N S (the kept
    slice is read twice, every amplitude written once); sampling
    from probabilities N 8 + 8 per shot; sampling from the state N S + 8 per
    shot; parity counts 8 per shot."""
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check, int_array
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceArray, DeviceState
    from qibo_gb300.serving import compile_brickwork, u3_matrices

    n = args.nqubits
    N = 2**n
    peak = measured_peaks().get("hbm_gbs", 6800.0)
    rng = np.random.default_rng(7)

    def unitary(d):
        q, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        return np.ascontiguousarray(q.astype(np.complex128)).view(np.float64).ravel()

    u1, u2 = unitary(2), unitary(4)
    cz = np.ascontiguousarray(np.diag([1, 1, 1, -1]).astype(np.complex128)).view(np.float64).ravel()
    cx = np.ascontiguousarray(np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]],
                                       dtype=np.complex128)).view(np.float64).ravel()
    sw = np.ascontiguousarray(np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],
                                       dtype=np.complex128)).view(np.float64).ravel()
    layer_ops, layer_coefs = compile_brickwork(n, 1, rng.uniform(0, 2 * np.pi, (1, n, 3)))
    x_terms = n
    out = {"workload": f"every hot-path call alone, n={n}, dense random state", "hbm_peak_gbs": peak,
           "peak_source": ("MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in measured_peaks()
                           else "fallback 6.8 TB/s (of fallback)")}
    nshots = 1_000_000
    for dtype, S in (("complex128", 16), ("complex64", 8)):
        b = GB300Backend(dtype)
        rt, lib, eng = b.rt, b.rt.lib, b.engine_gb
        s = rt.stream
        st = DeviceState(n, dtype)
        code = st.code
        check(lib.qgb_state_zero(st.ptr, n, code, s))
        dense = [((q,), (), u3_matrices(rng.uniform(0, 2 * np.pi, 3))) for q in range(n)]
        eng.apply_many(st, dense, blocked=True)
        probs = DeviceArray((N,), np.float64, rt)
        p10 = DeviceArray((1024,), np.float64, rt)
        norm = DeviceArray((1,), np.float64, rt)
        samples = DeviceArray((nshots,), np.int64, rt)
        odd = DeviceArray((64,), np.int64, rt)
        outcome = DeviceArray((1,), np.int64, rt)
        rt.h2d(outcome.ptr, np.array([5], dtype=np.int64))
        allq = int_array(range(n))
        q10 = int_array(list(range(0, n, 2))[:10])  # 10 distinct qubits for every n >= 19
        scratch = rt.scratch(max(lib.qgb_probs_scratch_bytes(n, n), lib.qgb_sample_scratch_bytes(n),
                                 lib.qgb_sample_state_scratch_bytes(n), lib.qgb_norm_scratch_bytes(),
                                 lib.qgb_expect_scratch_bytes(n, 2 * n)))
        zz_x = [0] * n
        zz_z = [(1 << i) | (1 << ((i + 1) % n)) for i in range(n)]
        xs_x = [1 << i for i in range(n)]
        xs_z = [0] * n
        ones = _lib.double_array([1.0] * n)
        masks = (C.c_uint64 * 64)(*[int(m) for m in rng.integers(1, 2**n, 64)])
        npass = eng.count_passes(n, code, [((int(o["qubits"][0]),) if o["k"] == 1 else
                                            (int(o["qubits"][0]), int(o["qubits"][1])), (),
                                            layer_coefs[o["coef_offset"]:o["coef_offset"] + (8 if o["k"] == 1 else 32)]
                                            .view(np.complex128).reshape((2, 2) if o["k"] == 1 else (4, 4)))
                                           for o in layer_ops])

        def gate(qs, ctrl, m):
            return lambda: check(lib.qgb_apply_gate(st.ptr, n, code, int_array(qs), len(qs), int_array(ctrl),
                                                    len(ctrl), m.ctypes.data_as(_lib.dp), s))

        def circuit_gate(q):  # one dense 1q gate through qgb_apply_circuit, gate by gate
            ops, coefs = compile_brickwork(n, 1, rng.uniform(0, 2 * np.pi, (1, n, 3)))
            one = ops[q:q + 1].copy()
            one["coef_offset"] = 0
            c1 = np.ascontiguousarray(coefs[ops[q]["coef_offset"]:ops[q]["coef_offset"] + 8])
            return lambda: check(lib.qgb_apply_circuit(st.ptr, n, code, one.ctypes.data_as(C.POINTER(_lib.QgbOp)), 1,
                                                       c1.ctypes.data_as(_lib.dp), 0, s))

        def circuit_desc(desc):  # any gate (qubits, controls, matrix) through qgb_apply_circuit, gate by gate
            return lambda: eng.apply_many(st, [desc])

        def with_fp64_warps(w, fn):  # QIBO_GB300_DF_FP64_WARPS around one call
            def run():
                os.environ["QIBO_GB300_DF_FP64_WARPS"] = str(w)
                try:
                    fn()
                finally:
                    del os.environ["QIBO_GB300_DF_FP64_WARPS"]
            return run

        df = " (FP64 / double-float warps)" if dtype == "complex128" else ""
        calls = [
            (f"dense 1q gate by gate{df}, qubit 0", "k_1q_pairs_mix" if df else "k_1q_pairs", 2 * N * S,
             circuit_gate(0)),
            (f"dense 1q gate by gate{df}, qubit n-1", "k_1q_shfl_mix" if df else "k_1q_shfl", 2 * N * S,
             circuit_gate(n - 1)),
        ]
        u2m = u2.view(np.complex128).reshape(4, 4)
        u1m = u1.view(np.complex128).reshape(2, 2)
        calls += [
            (f"dense 2q gate by gate{df}, qubits 3, n-5", "k_dense_mix<2>" if df else "k_dense<2>", 2 * N * S,
             circuit_desc(((3, n - 5), (), u2m))),
            (f"U3 gate by gate{df} on qubit 5 controlled by qubits 1, 2", "k_dense_mix<1>" if df else "k_dense<1>",
             2 * N * S // 4, circuit_desc(((5,), (1, 2), u1m))),
        ]
        if dtype == "complex128":  # the share of FP64 warps among each scheduler's 8
            for w in (0, 1, 2, 3, 4, 8):
                calls.append((f"dense 1q gate by gate, qubit 0, {w}/8 warps in FP64", "k_1q_pairs_mix", 2 * N * S,
                              with_fp64_warps(w, circuit_gate(0))))
            for w in (0, 1, 3):
                calls.append((f"dense 1q gate by gate, qubit n-1, {w}/8 warps in FP64", "k_1q_shfl_mix", 2 * N * S,
                              with_fp64_warps(w, circuit_gate(n - 1))))
        calls += [
            ("dense 1q, qubit 0 (index bit n-1)", "k_1q_pairs", 2 * N * S, gate([0], [], u1)),
            ("dense 1q, qubit n/2", "k_1q_pairs", 2 * N * S, gate([n // 2], [], u1)),
            ("dense 1q, qubit n-1 (index bit 0, warp shuffles)", "k_1q_shfl", 2 * N * S, gate([n - 1], [], u1)),
            ("dense 2q, qubits 3, n-5", "k_dense<2>", 2 * N * S, gate([3, n - 5], [], u2)),
            ("CZ, qubits n/2, n/2+1 (diagonal on a quarter)", "k_phase", 2 * N * S // 4,
             gate([n // 2, n // 2 + 1], [], cz)),
            ("CNOT, qubits 2, n-2 (swap on a half)", "k_xlike", 2 * N * S // 2, gate([2, n - 2], [], cx)),
            ("SWAP, qubits 1, n-3", "k_swap", 2 * N * S // 2, gate([1, n - 3], [], sw)),
            ("U3 on qubit 5 controlled by qubits 1, 2", "k_1q_pairs (controlled)", 2 * N * S // 4, gate([5], [1, 2], u1)),
            (f"one brickwork layer in shared-memory passes ({npass} passes)", "k_pass", npass * 2 * N * S,
             lambda: check(lib.qgb_apply_circuit(st.ptr, n, code, layer_ops.ctypes.data_as(C.POINTER(_lib.QgbOp)),
                                                 len(layer_ops), layer_coefs.ctypes.data_as(_lib.dp),
                                                 _lib.QGB_PLAN_BLOCKED, s))),
            ("probabilities, all qubits", "k_probs_all", N * S + N * 8,
             lambda: check(lib.qgb_probabilities(st.ptr, n, code, allq, n, probs.ptr, scratch, s))),
            ("probabilities, 10 qubits", "k_probs_*", N * S + 1024 * 8,
             lambda: check(lib.qgb_probabilities(st.ptr, n, code, q10, 10, p10.ptr, scratch, s))),
            ("norm", "k_norm_part + k_final_sum", N * S,
             lambda: check(lib.qgb_norm2(st.ptr, n, code, norm.ptr, scratch, s))),
            (f"Z Z expectation, {n} terms (one flip mask)", "k_expect_diag", N * S,
             lambda: check(lib.qgb_expect_pauli(st.ptr, n, code, (C.c_uint64 * n)(*zz_x), (C.c_uint64 * n)(*zz_z),
                                                ones, n, norm.ptr, scratch, s))),
            (f"X expectation, {x_terms} terms ({x_terms} flip masks)", "k_expect_flip_tile", x_terms * N * S,
             lambda: check(lib.qgb_expect_pauli(st.ptr, n, code, (C.c_uint64 * n)(*xs_x), (C.c_uint64 * n)(*xs_z),
                                                ones, n, norm.ptr, scratch, s))),
            ("collapse on 3 qubits", "k_collapse_norm + k_collapse_apply", N * S // 8 + N * S // 8 + N * S,
             lambda: check(lib.qgb_collapse(st.ptr, n, code, int_array([0, n // 2, n - 1]), 3, outcome.ptr, 1,
                                            scratch, s))),
            (f"{nshots} shots from the 2^n probabilities", "k_chunk_sums + k_scan_* + k_draw", N * 8 + nshots * 8,
             lambda: check(lib.qgb_sample(probs.ptr, n, nshots, 11, samples.ptr, None, scratch, s))),
            (f"{nshots} shots straight from the state", "k_state_chunk_sums + k_scan_* + k_draw_state",
             N * S + nshots * 8,
             lambda: check(lib.qgb_sample_state(st.ptr, n, code, nshots, 12, samples.ptr, scratch, s))),
            (f"parity counts, {nshots} shots x 64 terms", "k_parity", nshots * 8,
             lambda: check(lib.qgb_parity_counts(samples.ptr, nshots, masks, 64, odd.ptr, s))),
        ]
        ev = Events(lib)
        check(lib.qgb_probabilities(st.ptr, n, code, allq, n, probs.ptr, scratch, s))
        rows = []
        for name, kern, nbytes, call in calls:
            if name.startswith("collapse"):
                eng.apply_many(st, dense, blocked=True)  # every collapse starts from a dense state
            for _ in range(args.warmup):
                call()
            ev.start(s)
            for _ in range(args.steps):
                call()
            ms = ev.stop_ms(s) / args.steps
            gbs = nbytes / (ms * 1e-3) / 1e9
            rows.append({"call": name, "kernels": kern, "ms": round(ms, 4), "bytes": int(nbytes),
                         "GB/s": round(gbs, 1), "frac_of_hbm_peak": round(gbs / peak, 3)})
        out[dtype] = rows
        del st, probs, samples
    print(json.dumps(out))


def run_memlimit(args):
    """33-qubit complex128 (137 GB) and 34-qubit complex64 (137 GB): QFT then
    a depth-10 U3+CZ brickwork with engine fusion into <= 5-qubit blocks
    (the engine keeps the fused list when it has at most 11 ops per pass of
    the unfused shared-memory plan), 1e7 shots drawn straight from the
    state, <sum_i Z_i Z_{i+1}> (open chain), and the complex64 infidelity
    against complex128 at 33 qubits."""
    from qibo_gb300 import QFT, Circuit
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend, describe_gate
    from qibo_gb300.device import DeviceArray, DeviceState

    res = {}
    keep = {}
    # 34-qubit complex64 first (freed after), then the two 33-qubit states
    # that are compared (137 + 69 GB resident together)
    for n, dtype in ((34, "complex64"), (33, "complex128"), (33, "complex64")):
        b = GB300Backend(dtype)
        rt, eng, lib = b.rt, b.engine_gb, b.rt.lib
        c = QFT(n)
        c.add(brickwork_gates(n, 10, n))
        descs = [describe_gate(g, b) for g in c.queue]
        code = 1 if dtype == "complex128" else 0
        npass = eng.count_passes(n, code, descs)
        nfused, n5 = eng.fuse_stats(descs, n)
        fused = nfused <= 11 * npass
        nops = nfused if fused else npass  # state passes of the plan the engine runs
        st = DeviceState(n, dtype)
        ev = Events(lib)
        check(lib.qgb_state_zero(st.ptr, n, st.code, rt.stream))
        ev.start(rt.stream)
        eng.apply_many(st, descs, blocked=True, fuse=True)
        gms = ev.stop_ms(rt.stream)
        # complex64 results get the FP64 renormalisation the backend applies
        # (3xTF32 blocks drift the norm by about 5e-7 each)
        norm_before = eng.renormalize(st) if dtype == "complex64" else None
        samples = DeviceArray((10_000_000,), np.int64, rt)
        ev.start(rt.stream)
        check(lib.qgb_sample_state(st.ptr, n, st.code, 10_000_000, 33, samples.ptr,
                                   rt.scratch(lib.qgb_sample_state_scratch_bytes(n)), rt.stream))
        sms = ev.stop_ms(rt.stream)
        t0 = time.perf_counter()
        zz = eng.expect_pauli(st, [0] * (n - 1), [(1 << i) | (1 << (i + 1)) for i in range(n - 1)], [1.0] * (n - 1))
        zz_ms = (time.perf_counter() - t0) * 1e3
        S = 16 if dtype == "complex128" else 8
        key = f"n{n}_{dtype}"
        res[key] = {"gates": len(descs), "plan": "fused blocks" if fused else "shared-memory passes",
                    "fused_ops": nfused, "fused_5q_blocks": n5, "unfused_passes": npass, "state_passes": nops,
                    "gate_ms": gms, "pass_gbs": nops * 2 * 2**n * S / (gms * 1e-3) / 1e9, "shots_1e7_ms": sms,
                    "zz_open_chain": zz, "zz_ms_host": zz_ms, "state_gb": 2**n * S / 1e9,
                    "norm_before_renormalisation": norm_before}
        del samples
        if n == 33:
            keep[dtype] = st
        else:
            del st
        rt.synchronize()
    rt = keep["complex128"].rt
    out = DeviceArray((2,), np.float64, rt)
    check(rt.lib.qgb_inner_mixed(keep["complex128"].ptr, 1, keep["complex64"].ptr, 0, 33, out.ptr,
                                 rt.scratch(rt.lib.qgb_inner_scratch_bytes()), rt.stream))
    re, im = out.to_numpy()
    res["infidelity_c64_vs_c128_n33"] = 1.0 - (re * re + im * im)
    print(json.dumps({"workload": "memory limit: QFT + depth-10 brickwork, 1e7 shots, <ZZ>", **res}))


def run_density(args):
    """A noisy circuit on a density matrix of ``--nqubits`` qubits (at most
    16; 14 by default, a 28-qubit vector of 4.3 GB in complex128): depth 10
    of U3 on every qubit, CZ on brickwork pairs, then a depolarizing channel
    (p = 0.01) and amplitude damping (gamma = 0.05) on every qubit.  Timed
    through the public API (``execute_circuit`` on a density-matrix circuit,
    the device synchronised), median of ``--steps`` runs after ``--warmup``.
    Reports the trace and the purity Tr(rho^2) (the squared norm of the
    entry vector) of the result."""
    from qibo_gb300 import Circuit, gates as G
    from qibo_gb300.backend import GB300Backend

    n = args.nqubits if args.nqubits <= 16 else 14
    backend = GB300Backend(args.dtype)
    rng = np.random.default_rng(14)
    c = Circuit(n, density_matrix=True)
    depth = 10
    for layer in range(depth):
        for q in range(n):
            c.add(G.U3(q, *rng.uniform(0, 2 * np.pi, 3)))
        for q in range(layer % 2, n - 1, 2):
            c.add(G.CZ(q, q + 1))
        for q in range(n):
            c.add(G.DepolarizingChannel((q,), 0.01))
            c.add(G.AmplitudeDampingChannel(q, 0.05))
    times = []
    res = None
    for i in range(args.warmup + args.steps):
        backend.rt.synchronize()
        t0 = time.perf_counter()
        res = backend.execute_circuit(c)
        backend.rt.synchronize()
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    rho = res.state()
    sec = statistics.median(times)
    print(json.dumps({"workload": f"noisy density matrix, n={n} ({2 * n}-qubit vector), depth {depth}",
                      "dtype": args.dtype, "gates": n * depth + sum(len(range(l % 2, n - 1, 2)) for l in range(depth)),
                      "channels": 2 * n * depth, "seconds": sec,
                      "vector_gb": 4**n * (16 if args.dtype == "complex128" else 8) / 1e9,
                      "trace": backend.engine_gb.density_trace(rho), "purity": backend.engine_gb.norm2(rho)}))


def run_chain(args):
    """The complex128 block kernel in a fixed-point chain at ``--nqubits``:
    a random 5-qubit unitary on three placements (qubits 0..4 = the top
    index bits, the middle five, and qubits n-5..n-1 = index bits 0..4), on
    a state first made dense; ms per block = (chain of 10 - chain of 2) / 8,
    CUDA events on the launch stream, so the chain's norm and conversion
    passes cancel.  2 * 2^n * 16 bytes per block."""
    from qibo_gb300._lib import check
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    n = args.nqubits
    b = GB300Backend("complex128")
    rt, eng, lib = b.rt, b.engine_gb, b.rt.lib
    st = DeviceState(n, "complex128")
    rng = np.random.default_rng(1)
    q, r = np.linalg.qr(rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32)))
    u = q * (np.diag(r) / np.abs(np.diag(r)))
    check(lib.qgb_state_zero(st.ptr, n, st.code, rt.stream))
    eng.apply_many(st, [(list(range(5 * k, 5 * k + 5)), [], u) for k in range(n // 5)], blocked=True)
    ev = Events(lib)
    peak = measured_peaks().get("hbm_gbs", 6800.0)

    def timed(descs):
        eng.apply_many(st, descs, blocked=True)
        ev.start(rt.stream)
        eng.apply_many(st, descs, blocked=True)
        return ev.stop_ms(rt.stream)

    rows = {}
    for name, qs in (("top index bits", [0, 1, 2, 3, 4]), ("middle", list(range(n // 2 - 2, n // 2 + 3))),
                     ("index bits 0..4", [n - 5, n - 4, n - 3, n - 2, n - 1])):
        ms = (timed([(qs, [], u)] * 10) - timed([(qs, [], u)] * 2)) / 8
        gbs = 2 * 2**n * 16 / (ms * 1e-3) / 1e9
        rows[name] = {"ms_per_block": round(ms, 3), "GB/s": round(gbs, 1), "frac_of_hbm_peak": round(gbs / peak, 3)}
    print(json.dumps({"workload": f"complex128 block kernel in a fixed-point chain, n={n}", "hbm_peak_gbs": peak,
                      **rows}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="brickwork",
                    choices=["brickwork", "qft20", "vqe24", "serving", "memlimit", "tc5", "kernels", "fusion",
                             "chain", "density"])
    ap.add_argument("--nqubits", type=int, default=N_QUBITS)
    ap.add_argument("--dtype", default="complex128")
    ap.add_argument("--mode", default="auto", choices=["auto", "gates", "blocked", "fused", "engine"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the complex64 leg")
    ap.add_argument("--serving-requests", type=int, default=400)
    ap.add_argument("--serving-rates", default="25,50,10000",
                    help="comma-separated Poisson arrival rates (requests/s) of the serving sample")
    args = ap.parse_args()
    args.serving_rates = [float(x) for x in args.serving_rates.split(",")]
    if args.impl == "reference":
        return run_reference(args)
    return {"brickwork": run_brickwork, "qft20": run_qft20, "vqe24": run_vqe24, "serving": run_serving,
            "memlimit": run_memlimit, "tc5": run_tc5, "kernels": run_kernels,
            "fusion": run_fusion, "chain": run_chain, "density": run_density}[args.workload](args)


if __name__ == "__main__":
    main()
