"""qibo's multi-circuit API on the continuous-batching server.

The reference runs several circuits with a host thread pool, one
``execute_circuit`` per thread (``Backend.execute_circuits``,
backends/abstract.py:2514-2530 -> ``parallel_circuits_execution``,
parallel.py:60-121; ``parallel_parametrized_execution``, parallel.py:124-192).
Here the circuits become requests of ``serving.Server``: small ones run many
per launch, mid-sized ones as graph-captured programs (one capture per gate
shape, replayed with each request's matrices, so a parameter sweep of one
circuit replays one graph), large ones with engine fusion on the tensor
cores, all overlapping on the device.  The functions keep the reference's
signatures and return the same result objects as ``execute_circuit``.
"""

from __future__ import annotations

from typing import List

import numpy as np


def _simple(circuit) -> bool:
    """Circuits the server runs: state vectors without collapsing
    measurements, noise or distribution (the rest go through
    ``execute_circuit`` one at a time)."""
    return not (getattr(circuit, "density_matrix", False) or getattr(circuit, "repeated_execution", False)
                or getattr(circuit, "accelerators", None))


def _state_list(states, n: int, tensor_types) -> list:
    if states is None:
        return [None] * n
    if isinstance(states, tensor_types) or (hasattr(states, "shape") and len(getattr(states, "shape")) == 1):
        return [states] * n  # one state for every circuit (parallel.py:99-103)
    states = list(states)
    if len(states) != n:
        raise ValueError("states must have the same length as circuits.")
    return states


def serve_circuits(backend, circuits, states=None, nshots: int = 1000) -> List:
    """Results of ``circuits`` (in order) from one server run; ``states``:
    None, one initial state for all, or one per circuit."""
    from .backend import describe_gate
    from .device import DeviceArray
    from .serving import Request, compile_descs

    circuits = list(circuits)
    states = _state_list(states, len(circuits), getattr(backend, "tensor_types", (np.ndarray,)))
    results: List = [None] * len(circuits)
    reqs = []
    for i, (c, s) in enumerate(zip(circuits, states)):
        descs = [d for d in (describe_gate(g, backend) for g in c.queue) if d is not None] if _simple(c) else []
        if not descs:
            results[i] = backend.execute_circuit(c, s, nshots)
            continue
        backend._validate_nqubits(c.nqubits)
        init = None
        if s is not None:
            init = s.to_numpy() if isinstance(s, DeviceArray) else np.asarray(s)
            if init.shape != (2**c.nqubits,):
                raise ValueError(f"Given initial state has shape {init.shape} instead of the expected "
                                 f"{(2 ** c.nqubits,)}.")
        ops, coefs = compile_descs(descs)
        shape = ("circuit", c.nqubits) + tuple((tuple(q), tuple(ctrl)) for q, ctrl, _ in descs)
        reqs.append(Request(i, c.nqubits, backend.dtype, ops, coefs, shape, "state", initial=init))
    if reqs:
        srv = backend.server()
        srv.stats.clear()
        srv.run(reqs, realtime=False)
        QuantumState, CircuitResult = backend._result_classes()
        for r in reqs:
            c = circuits[r.rid]
            if c.measurements:
                res = CircuitResult(r.result, c.measurements, backend=backend, nshots=nshots)
            else:
                res = QuantumState(r.result, backend=backend)
            c._final_state = res
            results[r.rid] = res
    return results


def _backend(backend):
    if backend is not None:
        return backend
    try:
        from qibo.backends import _check_backend

        return _check_backend(None)
    except ImportError:
        from . import get_backend

        return get_backend()


def parallel_circuits_execution(circuits, states=None, nshots=1000, processes=None, backend=None):
    """``qibo.parallel.parallel_circuits_execution`` (parallel.py:60-121) on
    the device: ``processes`` is accepted for compatibility; the circuits
    overlap on the GPU instead of host threads."""
    return _backend(backend).execute_circuits(circuits, states, nshots)


def parallel_parametrized_execution(circuit, parameters, initial_state=None, processes=None, backend=None):
    """``qibo.parallel.parallel_parametrized_execution`` (parallel.py:124-192)
    on the device: ``circuit`` with each parameter set in ``parameters`` (a
    list), from ``initial_state`` (or |0...0>).  Every copy has the same gate
    shape, so mid-sized circuits replay one captured graph."""
    if not isinstance(parameters, list):
        raise TypeError("parameters must be a list.")
    b = _backend(backend)
    circuits = []
    for params in parameters:
        c = circuit.copy(deep=True)
        c.set_parameters(params)
        circuits.append(c)
    states = None if initial_state is None else [initial_state] * len(circuits)
    return b.execute_circuits(circuits, states)
