"""Continuous-batching circuit server on one GB300.

Requests (a circuit, its qubit count and dtype, and the output wanted: the
final state, shots, or a Z-string expectation) arrive over time.  The
scheduler

* admits requests in arrival order as device memory (a budget over a
  size-class pool of state buffers, so the loop never calls cudaMalloc
  after warm-up) and execution slots (non-blocking CUDA streams) free up;
* runs small circuits (<= 13 qubits complex64, <= 12 complex128) many per
  launch through ``qgb_batch_run``, each CTA holding a whole state in shared
  memory and producing its output in the same kernel;
* runs mid-sized circuits as shared-memory passes on their own stream
  through a ``qgb_program`` per circuit shape (a small pool of them, one per
  request of that shape on the device at once), whose launches are captured
  once as a CUDA graph and replayed with new matrices for later requests of
  the same shape;
* runs circuits of ``fuse_min_qubits`` qubits or more, whose device time
  dwarfs their launch overhead, through ``qgb_apply_circuit`` with engine
  fusion: blocks of five qubits on the tensor cores (complex64 3xTF32,
  complex128 Ozaki scheme), each slot's stream with its own chain scratch;
* polls completion events without blocking, so work from requests that
  arrived at different times overlaps on the device.

This replaces the host thread pools of the reference's
``Backend.execute_circuits`` / ``parallel_circuits_execution``
(backends/abstract.py:2514-2530, parallel.py:60-121).  Latency is measured
from arrival to the moment the result is on the host.
"""

from __future__ import annotations

import collections
import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _lib
from ._lib import QgbBatchItem, QgbOp, check
from .device import Runtime

# numpy view of qgb_op (must match include/qgb300.h)
OP_DTYPE = np.dtype({"names": ["k", "ncontrols", "qubits", "controls", "coef_offset"],
                     "formats": [np.int32, np.int32, (np.int32, 5), (np.int32, 8), np.int64],
                     "offsets": [0, 4, 8, 28, 64], "itemsize": C.sizeof(QgbOp)})
OUT_KINDS = {"state": _lib.QGB_OUT_STATE, "shots": _lib.QGB_OUT_SAMPLES, "zexp": _lib.QGB_OUT_ZEXP}
DTYPES = {"complex64": (_lib.QGB_C64, 8), "complex128": (_lib.QGB_C128, 16)}


@dataclass
class Request:
    """One circuit to run.  ``ops``/``coefs`` are the compiled gate list
    (``OP_DTYPE`` records and their matrices); ``shape`` keys graph reuse."""

    rid: int
    nqubits: int
    dtype: str
    ops: np.ndarray
    coefs: np.ndarray
    shape: tuple
    output: str = "state"
    nshots: int = 10_000
    zmask: int = 0
    seed: int = 0
    arrival: float = 0.0
    initial: object = None  # host state to start from instead of |0...0>
    result: object = None
    t_arrived: float = math.nan  # when the scheduler saw it arrive
    t_done: float = math.nan

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrived

    def layout(self) -> dict:
        """Byte offsets inside the request's one device buffer: the state,
        then (shots) FP64 probabilities, the CDF scratch and the samples, or
        (zexp) the reduction scratch and the FP64 result."""
        def up(x):
            return (x + 255) // 256 * 256

        n = self.nqubits
        lay = {"state": 0}
        off = up((2**n) * DTYPES[self.dtype][1])
        if self.output == "shots":
            lay["probs"] = off
            off = up(off + (2**n) * 8)
            lay["cdf"] = off
            off = up(off + (2**n) // 64 * 8 + 8 * ((2**n) // 64 // 1024 + 64) + 256)
            lay["out"] = off
            off = up(off + self.nshots * 8)
        else:
            lay["scratch"] = off
            off = up(off + 2 * 2560 * 8 * 2)
            lay["out"] = off
            off = up(off + 64)
        lay["total"] = off
        return lay

    def footprint(self) -> int:
        return self.layout()["total"]


# --------------------------------------------------------------- compiling --
def u3_matrices(angles: np.ndarray) -> np.ndarray:
    """U3(theta, phi, lambda) matrices (backends/npmatrices.py:125-136) for an
    array of angle triples, vectorised: shape (..., 2, 2) complex128."""
    t, p, l = angles[..., 0], angles[..., 1], angles[..., 2]
    c, s = np.cos(t / 2), np.sin(t / 2)
    ep, em = np.exp(1j * (p + l) / 2), np.exp(1j * (p - l) / 2)
    m = np.empty(angles.shape[:-1] + (2, 2), dtype=np.complex128)
    m[..., 0, 0] = np.conj(ep) * c
    m[..., 0, 1] = -np.conj(em) * s
    m[..., 1, 0] = em * s
    m[..., 1, 1] = ep * c
    return m


_CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)


def compile_brickwork(n: int, depth: int, angles: np.ndarray):
    """Random U3 + CZ brickwork (per layer U3 on every qubit, then CZ on
    pairs (l%2, l%2+1), ...) compiled to ``OP_DTYPE`` records and matrices."""
    mats = u3_matrices(angles.reshape(depth, n, 3))
    records, coefs = [], []
    off = 0
    for l in range(depth):
        for q in range(n):
            records.append((1, 0, (q, 0, 0, 0, 0), (0,) * 8, off))
            coefs.append(mats[l, q].ravel())
            off += 8
        for q in range(l % 2, n - 1, 2):
            records.append((2, 0, (q, q + 1, 0, 0, 0), (0,) * 8, off))
            coefs.append(_CZ.ravel())
            off += 32
    ops = np.array(records, dtype=OP_DTYPE)
    c = np.ascontiguousarray(np.concatenate(coefs)).view(np.float64)
    return ops, c


def compile_descs(descs) -> tuple:
    """(qubits, controls, matrix) descriptors -> (OP_DTYPE records, coefs)."""
    records, coefs = [], []
    off = 0
    for q, ctrl, m in descs:
        m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).ravel()
        records.append((len(q), len(ctrl), tuple(q) + (0,) * (5 - len(q)), tuple(ctrl) + (0,) * (8 - len(ctrl)), off))
        coefs.append(m)
        off += 2 * m.size
    return np.array(records, dtype=OP_DTYPE), np.concatenate(coefs).view(np.float64)


def _op_ptr(ops: np.ndarray):
    return ops.ctypes.data_as(C.POINTER(QgbOp))


# ------------------------------------------------------------------ memory --
class DevicePool:
    """Size-class pool of device buffers under a byte budget."""

    def __init__(self, rt: Runtime, budget: int):
        self.rt = rt
        self.budget = budget
        self.used = 0
        self.free: Dict[int, List[int]] = collections.defaultdict(list)
        self.held = 0  # bytes held by the pool (in use or cached)

    @staticmethod
    def size_class(nbytes: int) -> int:
        return 1 << max(12, (int(nbytes) - 1).bit_length())

    def acquire(self, nbytes: int) -> Optional[int]:
        sc = self.size_class(nbytes)
        if self.used + sc > self.budget:
            return None
        if self.free[sc]:
            p = self.free[sc].pop()
        else:
            # make room by dropping cached buffers of other sizes
            while self.held + sc > self.budget and self._drop_one(sc):
                pass
            if self.held + sc > self.budget:
                return None
            p = self.rt.malloc(sc)
            self.held += sc
        self.used += sc
        return p

    def _drop_one(self, keep: int) -> bool:
        for sc, lst in self.free.items():
            if sc != keep and lst:
                self.rt.free(lst.pop())
                self.held -= sc
                return True
        return False

    def release(self, p: int, nbytes: int):
        sc = self.size_class(nbytes)
        self.used -= sc
        self.free[sc].append(p)

    def close(self):
        for sc, lst in self.free.items():
            for p in lst:
                self.rt.free(p)
        self.free.clear()


class PinnedPool:
    """Page-locked host buffers (size classes) for asynchronous result copies."""

    def __init__(self, rt: Runtime):
        self.rt = rt
        self.free: Dict[int, List[np.ndarray]] = collections.defaultdict(list)
        self.ptrs: List[int] = []

    def acquire(self, nbytes: int) -> np.ndarray:
        sc = 1 << max(12, (int(nbytes) - 1).bit_length())
        if self.free[sc]:
            return self.free[sc].pop()
        p = C.c_void_p()
        check(self.rt.lib.qgb_host_alloc(C.byref(p), sc))
        self.ptrs.append(p.value)
        return np.ctypeslib.as_array((C.c_uint8 * sc).from_address(p.value))

    def release(self, buf: np.ndarray):
        self.free[buf.nbytes].append(buf)

    def close(self):
        self.free.clear()
        for p in self.ptrs:
            self.rt.lib.qgb_host_free(p)
        self.ptrs = []


# ------------------------------------------------------------------ server --
@dataclass
class _Flight:
    requests: list
    event: int
    slot: int
    buffers: list = field(default_factory=list)   # (ptr, nbytes)
    hostbufs: list = field(default_factory=list)  # (request, pinned array, view)
    kind: str = "large"
    program: tuple = None  # (pool key, program) in use, returned on completion


class Server:
    def __init__(self, budget_bytes: Optional[int] = None, nslots: int = 16, batch_max: int = 256,
                 use_graphs: bool = True, one_at_a_time: bool = False, fuse_min_qubits: int = 16,
                 keep_states: bool = True):
        """``keep_states=False``: state outputs still reach the host (pinned
        buffers) but are dropped there instead of being kept in each
        request's ``result``, so that long streams of large states fit in
        host memory."""
        self.rt = Runtime.get()
        self.keep_states = keep_states
        self.lib = self.rt.lib
        free, total = self.rt.mem_info()
        self.pool = DevicePool(self.rt, budget_bytes or int(free * 0.85))
        self.pinned = PinnedPool(self.rt)
        self.one_at_a_time = one_at_a_time
        self.nslots = 1 if one_at_a_time else nslots
        self.batch_max = batch_max
        self.use_graphs = use_graphs and not one_at_a_time
        self.fuse_min_qubits = fuse_min_qubits
        self.streams, self.events, self.batch_ctx = [], [], []
        for _ in range(self.nslots):
            s, e, b = C.c_void_p(), C.c_void_p(), C.c_void_p()
            check(self.lib.qgb_stream_create(C.byref(s)))
            check(self.lib.qgb_event_create(C.byref(e)))
            check(self.lib.qgb_batch_create(64 << 20, C.byref(b)))
            self.streams.append(s)
            self.events.append(e)
            self.batch_ctx.append(b)
        self.free_slots = list(range(self.nslots))
        # idle programs per (circuit shape, dtype); one is taken out while its
        # request is on the device, so a shape may have several
        self.programs: Dict[tuple, List[int]] = collections.defaultdict(list)
        self.all_programs: List[int] = []
        self.stats = collections.Counter()

    def close(self):
        for s in self.streams:
            self.lib.qgb_stream_sync(s)
        for p in self.all_programs:
            self.lib.qgb_program_destroy(p)
        for s, e, b in zip(self.streams, self.events, self.batch_ctx):
            self.lib.qgb_stream_sync(s)
            self.lib.qgb_batch_destroy(b)
            self.lib.qgb_event_destroy(e)
            self.lib.qgb_stream_destroy(s)
        self.pool.close()
        self.pinned.close()

    # -- launch helpers --------------------------------------------------
    def _is_small(self, r: Request) -> bool:
        return not self.one_at_a_time and r.nqubits <= _lib.QGB_BATCH_MAX_QUBITS[DTYPES[r.dtype][0]]

    def _launch_batch(self, reqs: List[Request], slot: int) -> _Flight:
        code, S = DTYPES[reqs[0].dtype]
        stream = self.streams[slot]
        fl = _Flight(reqs, self.events[slot], slot, kind="batch")
        items = (QgbBatchItem * len(reqs))()
        for i, r in enumerate(reqs):
            st = self.pool.acquire(r.footprint())
            fl.buffers.append((st, r.footprint()))
            it = items[i]
            it.state = st
            it.nqubits = r.nqubits
            it.nops = len(r.ops)
            it.ops = _op_ptr(r.ops)
            it.coefs = r.coefs.ctypes.data_as(_lib.dp)
            if r.initial is None:
                it.init_zero = 1
            else:
                init = np.ascontiguousarray(r.initial, dtype=r.dtype)
                check(self.lib.qgb_memcpy_h2d(st, init.ctypes.data, init.nbytes, stream))
                it.init_zero = 0
            it.out_kind = OUT_KINDS[r.output]
            it.nshots = r.nshots
            it.seed = r.seed
            it.zmask = r.zmask
            it.out = st + r.layout()["out"]
        check(self.lib.qgb_batch_run(self.batch_ctx[slot], C.cast(items, C.c_void_p), len(reqs), code, stream))
        for i, r in enumerate(reqs):
            self._copy_out(fl, r, items[i].state, items[i].out, stream)
        check(self.lib.qgb_event_record(fl.event, stream))
        self.stats["batches"] += 1
        self.stats["batched_requests"] += len(reqs)
        return fl

    def _copy_out(self, fl: _Flight, r: Request, state: int, out: int, stream):
        code, S = DTYPES[r.dtype]
        if r.output == "state":
            nbytes = (2**r.nqubits) * S
        elif r.output == "shots":
            nbytes = r.nshots * 8
        else:
            nbytes = 8
        buf = self.pinned.acquire(nbytes)
        src = state if r.output == "state" else out
        check(self.lib.qgb_memcpy_d2h(buf.ctypes.data, src, nbytes, stream))
        fl.hostbufs.append((r, buf, nbytes))

    def _launch_large(self, r: Request, slot: int) -> _Flight:
        code, S = DTYPES[r.dtype]
        stream = self.streams[slot]
        fl = _Flight([r], self.events[slot], slot)
        fp = r.footprint()
        st = self.pool.acquire(fp)
        fl.buffers.append((st, fp))
        n = r.nqubits
        if r.initial is None:
            check(self.lib.qgb_state_zero(st, n, code, stream))
        else:
            init = np.ascontiguousarray(r.initial, dtype=r.dtype)
            check(self.lib.qgb_memcpy_h2d(st, init.ctypes.data, init.nbytes, stream))
        if self.one_at_a_time:  # the plain per-gate path: one kernel per gate, IEEE FP64 for complex128
            check(self.lib.qgb_apply_circuit(st, n, code, _op_ptr(r.ops), len(r.ops), r.coefs.ctypes.data_as(_lib.dp),
                                             _lib.QGB_PLAN_STRICT_FP64, stream))
        elif n >= self.fuse_min_qubits:
            check(self.lib.qgb_apply_circuit(st, n, code, _op_ptr(r.ops), len(r.ops), r.coefs.ctypes.data_as(_lib.dp),
                                             _lib.QGB_PLAN_BLOCKED | _lib.QGB_PLAN_FUSE, stream))
            self.stats["fused"] += 1
        else:
            key = (r.shape, r.dtype)
            if self.programs[key]:
                prog = self.programs[key].pop()
                check(self.lib.qgb_program_update(prog, _op_ptr(r.ops), len(r.ops), r.coefs.ctypes.data_as(_lib.dp),
                                                  stream))
                self.stats["graph_replays"] += 1
            else:
                p = C.c_void_p()
                flags = 0 if self.use_graphs else _lib.QGB_PROGRAM_NO_GRAPH
                check(self.lib.qgb_program_create(n, code, _op_ptr(r.ops), len(r.ops), r.coefs.ctypes.data_as(_lib.dp),
                                                  flags, C.byref(p)))
                prog = p.value
                self.all_programs.append(prog)
                self.stats["programs_built"] += 1
            check(self.lib.qgb_program_run(prog, st, stream))
            fl.program = (key, prog)
        lay = r.layout()
        if r.output == "shots":
            probs, cdf, samples = st + lay["probs"], st + lay["cdf"], st + lay["out"]
            allq = _lib.int_array(range(n))
            check(self.lib.qgb_probabilities(st, n, code, allq, n, probs, None, stream))
            check(self.lib.qgb_sample(probs, n, r.nshots, r.seed, samples, None, cdf, stream))
            self._copy_out(fl, r, st, samples, stream)
        elif r.output == "zexp":
            xm = (C.c_uint64 * 1)(0)
            zm = (C.c_uint64 * 1)(r.zmask)
            cf = _lib.double_array([1.0])
            check(self.lib.qgb_expect_pauli(st, n, code, xm, zm, cf, 1, st + lay["out"], st + lay["scratch"], stream))
            self._copy_out(fl, r, st, st + lay["out"], stream)
        else:
            self._copy_out(fl, r, st, 0, stream)
        check(self.lib.qgb_event_record(fl.event, stream))
        self.stats["large"] += 1
        return fl

    def _finish(self, fl: _Flight, now: float):
        for r, buf, nbytes in fl.hostbufs:
            view = buf[:nbytes]
            if r.output == "state":
                r.result = (view.view(np.complex128 if r.dtype == "complex128" else np.complex64).copy()
                            if self.keep_states else None)
            elif r.output == "shots":
                r.result = view.view(np.int64).copy()
            else:
                r.result = float(view.view(np.float64)[0])
            self.pinned.release(buf)
            r.t_done = now
        for p, nbytes in fl.buffers:
            self.pool.release(p, nbytes)
        if fl.program is not None:
            key, prog = fl.program
            self.programs[key].append(prog)
        self.free_slots.append(fl.slot)

    # -- the loop -----------------------------------------------------------
    def run(self, requests: List[Request], realtime: bool = True) -> dict:
        """Serve ``requests`` (``arrival`` in seconds from the start)."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting: collections.deque = collections.deque()
        inflight: List[_Flight] = []
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: math.inf)
        while pending or waiting or inflight:
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                r.t_arrived = min(r.arrival, time.perf_counter() - t0)
                waiting.append(r)
            progressed = False
            # completions
            for fl in list(inflight):
                if self.lib.qgb_event_query(fl.event) == _lib.QGB_OK:
                    t = time.perf_counter() - t0
                    self._finish(fl, t)
                    inflight.remove(fl)
                    progressed = True
            # admissions, in arrival order
            while waiting and self.free_slots:
                head = waiting[0]
                if self._is_small(head):
                    batch, budget = [], 0
                    for r in list(waiting):
                        if len(batch) >= self.batch_max:
                            break
                        if self._is_small(r) and r.dtype == head.dtype:
                            if self.pool.used + budget + DevicePool.size_class(r.footprint()) > self.pool.budget:
                                break
                            budget += DevicePool.size_class(r.footprint())
                            batch.append(r)
                    if not batch:
                        break
                    for r in batch:
                        waiting.remove(r)
                    slot = self.free_slots.pop()
                    inflight.append(self._launch_batch(batch, slot))
                else:
                    if self.pool.used + DevicePool.size_class(head.footprint()) > self.pool.budget:
                        if not inflight:
                            raise MemoryError(f"request {head.rid} ({head.nqubits} qubits) exceeds the device budget")
                        break
                    waiting.popleft()
                    slot = self.free_slots.pop()
                    inflight.append(self._launch_large(head, slot))
                progressed = True
            if not progressed:
                if realtime and not inflight and not waiting and pending:
                    time.sleep(max(0.0, min(0.001, pending[0].arrival - clock())))
                else:
                    time.sleep(20e-6)
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in requests])
        return {"requests": len(requests), "wall_s": wall, "circuits_per_s": len(requests) / wall,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), **dict(self.stats)}


def shard_requests(requests: List[Request], rank: int, world: int) -> List[Request]:
    """Replica sharding: one GPU per rank, requests dealt round-robin by id so
    every rank gets the same mix; no data moves between ranks."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return [r for r in requests if r.rid % world == rank]


def merge_stats(per_rank: List[dict]) -> dict:
    """Whole-job numbers from per-replica ``Server.run`` stats: requests add
    up, the wall time is the slowest replica's, latency percentiles are the
    worst replica's (an upper bound on the pooled percentile)."""
    n = sum(s["requests"] for s in per_rank)
    wall = max(s["wall_s"] for s in per_rank)
    return {"requests": n, "wall_s": wall, "circuits_per_s": n / wall if wall > 0 else float("inf"),
            "p50_ms": max(s["p50_ms"] for s in per_rank), "p99_ms": max(s["p99_ms"] for s in per_rank),
            "replicas": len(per_rank)}


def make_stream(nreq: int, rate: float, seed: int = 0, nmin: int = 10, nmax: int = 28, dmin: int = 5,
                dmax: int = 30, nshots: int = 10_000) -> List[Request]:
    """The serving workload: Poisson arrivals at ``rate`` per second; qubits
    uniform in [nmin, nmax]; depth uniform in [dmin, dmax]; complex64 or
    complex128 with probability 1/2; output state / shots / Z-string
    expectation with probability 1/3 each; angles from default_rng(10000+i)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq)) if rate > 0 else np.zeros(nreq)
    reqs = []
    for i in range(nreq):
        n = int(rng.integers(nmin, nmax + 1))
        d = int(rng.integers(dmin, dmax + 1))
        dt = "complex64" if rng.random() < 0.5 else "complex128"
        out = ("state", "shots", "zexp")[int(rng.integers(3))]
        ang = np.random.default_rng(10_000 + i).uniform(0, 2 * np.pi, (d, n, 3))
        ops, coefs = compile_brickwork(n, d, ang)
        zmask = int(rng.integers(1, 2**n))
        reqs.append(Request(i, n, dt, ops, coefs, ("brick", n, d), out, nshots, zmask, 1000 + i, float(t[i])))
    return reqs
