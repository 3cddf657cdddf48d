"""Serving path on the GPU: graph-replayed programs, batched small circuits
with fused outputs, and the continuous-batching server.

Tolerances: complex128 states/expectations 1e-12 max-abs against the FP64
oracle, complex64 1e-5; shots pass a chi-square test against |psi|^2; a
request's result is the same alone and inside a mixed stream (states and
expectations within the tolerances above, shots bit-identical for the same
seed)."""

import ctypes as C

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu

TOL = {"complex128": 1e-12, "complex64": 1e-5}


def oracle_state(n, depth, ang, dtype):
    ops = []
    a = ang.reshape(depth, n, 3)
    for l in range(depth):
        for q in range(n):
            ops.append(("U3", (q,), tuple(a[l, q])))
        for q in range(l % 2, n - 1, 2):
            ops.append(("CZ", (q, q + 1), ()))
    return ref.execute(ops, n, dtype=dtype)


def test_program_graph_replay_matches_oracle():
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceState, Runtime
    from qibo_gb300.serving import _op_ptr, compile_brickwork

    rt = Runtime.get()
    n, depth = 16, 8
    stream = C.c_void_p()
    check(rt.lib.qgb_stream_create(C.byref(stream)))  # graphs are captured on a real stream
    for dtype in ("complex128", "complex64"):
        code = 1 if dtype == "complex128" else 0
        prog = C.c_void_p()
        ang0 = np.random.default_rng(1).uniform(0, 2 * np.pi, (depth, n, 3))
        ops, coefs = compile_brickwork(n, depth, ang0)
        check(rt.lib.qgb_program_create(n, code, _op_ptr(ops), len(ops), coefs.ctypes.data_as(_lib.dp), 0,
                                        C.byref(prog)))
        try:
            for rep in range(3):  # first run captures the graph, later runs replay it
                ang = np.random.default_rng(10 + rep).uniform(0, 2 * np.pi, (depth, n, 3))
                ops, coefs = compile_brickwork(n, depth, ang)
                check(rt.lib.qgb_program_update(prog, _op_ptr(ops), len(ops), coefs.ctypes.data_as(_lib.dp),
                                                stream))
                st = DeviceState.zero(n, dtype)
                rt.synchronize()
                check(rt.lib.qgb_program_run(prog, st.ptr, stream))
                check(rt.lib.qgb_stream_sync(stream))
                got = np.asarray(st)
                want = oracle_state(n, depth, ang, dtype)
                assert np.max(np.abs(got - want)) < TOL[dtype] * (10 if dtype == "complex64" else 1), (dtype, rep)
            # a different gate shape is refused
            ops2, coefs2 = compile_brickwork(n, depth - 1, ang[:-1])
            with pytest.raises(ValueError):
                check(rt.lib.qgb_program_update(prog, _op_ptr(ops2), len(ops2), coefs2.ctypes.data_as(_lib.dp),
                                                stream))
            # the legacy default stream runs the same program without a graph
            st = DeviceState.zero(n, dtype)
            check(rt.lib.qgb_program_run(prog, st.ptr, None))
            rt.synchronize()
            assert np.max(np.abs(np.asarray(st) - want)) < TOL[dtype] * (10 if dtype == "complex64" else 1)
        finally:
            rt.lib.qgb_program_destroy(prog)
    rt.lib.qgb_stream_destroy(stream)


def _serve(reqs, **kw):
    from qibo_gb300.serving import Server

    srv = Server(**kw)
    try:
        stats = srv.run(reqs, realtime=False)
    finally:
        srv.close()
    return stats


def _clone(r):
    from qibo_gb300.serving import Request

    return Request(r.rid, r.nqubits, r.dtype, r.ops, r.coefs, r.shape, r.output, r.nshots, r.zmask, r.seed, 0.0)


def test_batched_small_circuits_outputs_vs_oracle():
    from qibo_gb300.serving import Request, compile_brickwork

    reqs = []
    k = 0
    for dtype in ("complex128", "complex64"):
        for n in (3, 7, 12):
            for out in ("state", "shots", "zexp"):
                ang = np.random.default_rng(100 + k).uniform(0, 2 * np.pi, (6, n, 3))
                ops, coefs = compile_brickwork(n, 6, ang)
                reqs.append(Request(k, n, dtype, ops, coefs, ("b", n, 6), out, 20000, (5 << 1) & (2**n - 1) or 1,
                                    7 + k))
                k += 1
    stats = _serve(reqs)
    assert stats["batches"] >= 1 and stats.get("large", 0) == 0
    from scipy.stats import chi2

    for r in reqs:
        ang = np.random.default_rng(100 + r.rid).uniform(0, 2 * np.pi, (6, r.nqubits, 3))
        want = oracle_state(r.nqubits, 6, ang, r.dtype)
        if r.output == "state":
            assert np.max(np.abs(r.result - want)) < TOL[r.dtype] * (10 if r.dtype == "complex64" else 1)
        elif r.output == "zexp":
            p = np.abs(want.astype(np.complex128)) ** 2
            sign = np.array([(-1) ** bin(i & int("".join(reversed(f"{r.zmask:0{r.nqubits}b}")), 2)).count("1")
                             for i in range(2**r.nqubits)])
            assert abs(r.result - float(p @ sign)) < (1e-5 if r.dtype == "complex64" else 1e-12)
        else:
            p = np.abs(want.astype(np.complex128)) ** 2
            counts = np.bincount(r.result, minlength=2**r.nqubits)
            exp = p * r.nshots
            m = exp > 5
            stat = np.sum((counts[m] - exp[m]) ** 2 / exp[m])
            assert chi2.sf(stat, m.sum() - 1) > 1e-4


def test_mixed_stream_results_equal_alone():
    """Continuous batching: each request's result inside a mixed stream
    (small batched + large per-stream, both dtypes, all output kinds,
    overlapping on the device) equals its result when served alone."""
    from qibo_gb300.serving import make_stream

    reqs = make_stream(60, rate=0.0, seed=3, nmin=6, nmax=18, dmin=3, dmax=10, nshots=4000)
    stats = _serve(reqs, nslots=8, batch_max=16)
    assert stats["large"] > 0 and stats["batches"] > 0
    assert stats.get("graph_replays", 0) > 0 or stats.get("programs_built", 0) > 0
    for r in reqs:
        alone = _clone(r)
        _serve([alone], nslots=1)
        if r.output == "shots":
            np.testing.assert_array_equal(r.result, alone.result)
        elif r.output == "zexp":
            assert abs(r.result - alone.result) < TOL[r.dtype]
        else:
            assert np.max(np.abs(r.result - alone.result)) < TOL[r.dtype]


def test_stream_results_vs_oracle_and_latency_stats():
    from qibo_gb300.serving import make_stream

    reqs = make_stream(40, rate=400.0, seed=5, nmin=10, nmax=16, dmin=4, dmax=8, nshots=1000)
    stats = _serve(reqs, nslots=8, batch_max=8)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for r in reqs:
        if r.output != "state":
            continue
        d = len(r.ops) and r.shape[2]
        ang = np.random.default_rng(10_000 + r.rid).uniform(0, 2 * np.pi, (d, r.nqubits, 3))
        want = oracle_state(r.nqubits, d, ang, r.dtype)
        assert np.max(np.abs(r.result - want)) < TOL[r.dtype] * (10 if r.dtype == "complex64" else 1)


def test_one_at_a_time_baseline_path():
    from qibo_gb300.serving import make_stream

    reqs = make_stream(6, rate=0.0, seed=9, nmin=10, nmax=14, dmin=3, dmax=5, nshots=500)
    stats = _serve(reqs, one_at_a_time=True)
    assert stats.get("batches", 0) == 0 and stats["large"] == 6


def test_fused_large_requests_concurrent_vs_oracle():
    """Requests of ``fuse_min_qubits`` qubits or more run through engine
    fusion on the tensor cores, twelve slots at once (each stream with its
    own complex128 fixed-point chain scratch); every state matches the FP64
    oracle."""
    from qibo_gb300.serving import Request, compile_brickwork

    reqs, angs = [], {}
    k = 0
    for dtype in ("complex128", "complex64"):
        for n in (16, 17, 18):
            for d in (8, 10):
                ang = np.random.default_rng(500 + k).uniform(0, 2 * np.pi, (d, n, 3))
                ops, coefs = compile_brickwork(n, d, ang)
                reqs.append(Request(k, n, dtype, ops, coefs, ("f", n, d), "state", 0, 0, 0))
                angs[k] = (d, ang)
                k += 1
    stats = _serve(reqs, nslots=12)
    assert stats.get("fused", 0) == len(reqs)
    for r in reqs:
        d, ang = angs[r.rid]
        want = oracle_state(r.nqubits, d, ang, "complex128")
        assert np.max(np.abs(r.result - want)) < TOL[r.dtype] * (10 if r.dtype == "complex64" else 1), (r.rid, r.dtype)


def _mixed_circuits(dtype):
    """Circuits of 6 (batched), 14 (graph-captured program) and 17 qubits
    (engine fusion), with and without measurements."""
    from qibo_gb300 import Circuit, gates

    out = []
    for k, n in enumerate((6, 14, 17, 14, 6)):
        ops = ref.brickwork_ops(n, 5, 900 + k)
        c = Circuit(n)
        for nm, q, p in ops:
            c.add(getattr(gates, nm)(*q, *p))
        if k % 2:
            c.add(gates.M(0, n - 1))
        out.append(c)
    return out


def test_execute_circuits_on_the_server_equal_alone():
    """Backend.execute_circuits (backends/abstract.py:2514-2530) through the
    server: each result equals execute_circuit of that circuit alone; an
    initial state per circuit is honoured; measured circuits give
    frequencies over nshots."""
    from qibo_gb300.backend import GB300Backend

    for dtype in ("complex128", "complex64"):
        b = GB300Backend(dtype)
        circs = _mixed_circuits(dtype)
        rng = np.random.default_rng(4)
        states = []
        for c in circs:
            s = rng.normal(size=2**c.nqubits) + 1j * rng.normal(size=2**c.nqubits)
            states.append(s / np.linalg.norm(s))
        for init in (None, states):
            res = b.execute_circuits(circs, init, nshots=500)
            st = b.server().stats
            assert st.get("batched_requests", 0) >= 2 and st.get("fused", 0) >= 1 and st.get("large", 0) >= 3
            for i, (c, r) in enumerate(zip(circs, res)):
                alone = b.execute_circuit(c.copy(deep=True), None if init is None else init[i].copy(), nshots=500)
                got, want = np.asarray(r.state()), np.asarray(alone.state())
                assert np.max(np.abs(got - want)) < TOL[dtype], (dtype, i, init is None)
                if c.measurements:
                    assert sum(r.frequencies().values()) == 500


def test_parametrized_sweep_replays_one_graph():
    """parallel_parametrized_execution (parallel.py:124-192): a 14-qubit
    RY/CZ circuit with 24 parameter sets runs as requests of one gate shape,
    which replay the captured graph of that shape; every state equals the
    circuit run alone with those parameters."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.parallel import parallel_parametrized_execution

    n = 14
    b = GB300Backend("complex128")
    c = Circuit(n)
    for layer in range(3):
        c.add([gates.RY(q, theta=0.0) for q in range(n)])
        c.add([gates.CZ(q, q + 1) for q in range(layer % 2, n - 1, 2)])
    c.add([gates.RY(q, theta=0.0) for q in range(n)])
    nparams = len(c.get_parameters())
    rng = np.random.default_rng(8)
    params = [rng.uniform(0, 2 * np.pi, nparams) for _ in range(24)]
    res = parallel_parametrized_execution(c, params, backend=b)
    st = b.server().stats
    assert st.get("graph_replays", 0) >= 24 - 8 and st.get("programs_built", 0) <= 8, dict(st)
    for p, r in zip(params, res):
        one = c.copy(deep=True)
        one.set_parameters(p)
        want = np.asarray(b.execute_circuit(one).state())
        assert np.max(np.abs(np.asarray(r.state()) - want)) < TOL["complex128"]
    # the template circuit's own parameters are left alone
    assert all(abs(v[0]) == 0.0 for v in c.get_parameters())
