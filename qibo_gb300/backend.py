"""The GB300 backend: qibo's ``Backend`` hot-path methods on the device.

``GB300Methods`` overrides the state-vector hot path of
``qibo.backends.abstract.Backend`` with calls into ``libqgb300.so``:

=================================  ==========================================
reference method (abstract.py)     here
=================================  ==========================================
``zero_state`` :2243               ``DeviceState.zero`` (device memset)
``cast`` / ``to_numpy``            host <-> device copies of states
``execute_circuit`` :2442          whole gate queue in one C call
``apply_gate`` :2322               ``qgb_apply_gate`` (in place)
``matrix_fused`` :2680             dense einsum product on the host (2^k <= 32)
``calculate_probabilities`` :2734  ``qgb_probabilities`` (FP64, on device)
``sample_shots`` :2774             ``qgb_sample`` (Philox + FP64 CDF)
``sample_frequencies`` :2760       ``qgb_sample`` into a device histogram
``exp_value_observable_symbolic``  ``qgb_expect_pauli`` (one pass per flip
  :2946                            mask, all terms)
``exp_value_observable_symbolic_``  basis rotations, device shots and
  ``from_samples`` :3056           ``qgb_parity_counts`` per term group
``collapse_state`` :2424           ``qgb_collapse`` (in place)
``execute_circuit_repeated``       per shot on the device: collapsing
  :2532                            measurements sampled and applied there
``set_seed`` :181                  seeds the Philox stream
=================================  ==========================================

The class is mixed either into qibo's ``NumpyBackend`` (``QiboGB300Backend``
in ``qibo_gb300.plugin``, when qibo is installed) or into the standalone base
below.  Everything not listed stays with the base class, on small host
arrays.
"""

from __future__ import annotations

import collections
import os
from typing import List

import numpy as np

from . import _lib
from . import gates as G
from ._lib import DeviceOutOfMemory, check, int_array
from .density import compile_queue, gate_pair, is_channel, wide_terms
from .device import DeviceArray, DeviceDensity, DeviceState, Runtime
from .engine import Engine, pauli_masks

SKIP_GATES = ("M", "I", "Align", "CallbackGate")


def describe_gate(gate, backend):
    """(qubits, controls, matrix) of a qibo or qibo_gb300 gate, or None for
    gates that leave the state unchanged (measurements without collapse,
    identities)."""
    name = type(gate).__name__
    if name in SKIP_GATES:
        if name == "M" and getattr(gate, "collapse", False):
            raise NotImplementedError("collapsing measurements are not supported by qibo_gb300")
        return None
    if is_channel(gate):
        raise NotImplementedError(f"{name} cannot be applied to statevector.")
    m = np.asarray(gate.matrix(backend), dtype=np.complex128)
    if getattr(gate, "is_controlled_by", False):
        return tuple(gate.target_qubits), tuple(gate.control_qubits), m
    return tuple(gate.qubits), (), m


# below this size the tensor-core block kernels do not run and dense 5-qubit
# blocks would only slow the shared-memory passes
FUSE_MIN_QUBITS = 12

class GB300Methods:
    """Hot-path overrides; expects ``self.dtype`` and the result classes."""

    name = "qibo_gb300"

    def _gb300_init(self, dtype="complex128"):
        self.rt = Runtime.get()
        self.engine_gb = Engine(self.rt)
        self.device = "/GPU:0"
        self.platform = "cuda"
        self.supports_multigpu = False
        self.oom_error = DeviceOutOfMemory
        self._seed = None
        self._seed_calls = 0
        # shared-memory multi-gate passes (QIBO_GB300_BLOCKED=0: one kernel per gate)
        self.blocked = os.environ.get("QIBO_GB300_BLOCKED", "1") != "0"
        # complex128 passes in IEEE FP64 instead of double-float (QIBO_GB300_STRICT_FP64=1)
        self.strict_fp64 = os.environ.get("QIBO_GB300_STRICT_FP64", "0") == "1"
        # complex64 results renormalised with an FP64 norm after the circuit
        # (QIBO_GB300_RENORMALIZE=0 turns it off)
        self.renormalize_c64 = os.environ.get("QIBO_GB300_RENORMALIZE", "1") != "0"
        # the engine fuses circuits of FUSE_MIN_QUBITS or more into blocks of
        # <= 5 qubits whose 5-qubit blocks run on the tensor cores
        # (QIBO_GB300_FUSE=0 turns it off)
        self.fuse = os.environ.get("QIBO_GB300_FUSE", "1") != "0"

    # -- states -----------------------------------------------------------
    def zero_state(self, nqubits, density_matrix=False, dtype=None):
        self._validate_nqubits(nqubits, density_matrix=density_matrix)
        if density_matrix:
            return DeviceDensity.zero(nqubits, dtype or self.dtype)
        return DeviceState.zero(nqubits, dtype or self.dtype)

    def cast(self, array, dtype=None, copy=False):
        if isinstance(array, DeviceState):
            dt = np.dtype(dtype or array.dtype)
            return array.astype(dt, copy=copy)
        return super().cast(array, dtype=dtype, copy=copy)

    def to_numpy(self, array):
        if isinstance(array, DeviceArray):
            return array.to_numpy()
        return super().to_numpy(array)

    def _as_device_state(self, state, nqubits=None, dtype=None):
        if isinstance(state, DeviceState):
            return state
        arr = np.asarray(state)
        dt = dtype or (arr.dtype if arr.dtype in (np.complex64, np.complex128) else self.dtype)
        if arr.ndim == 2:
            return DeviceDensity.from_numpy(arr, dt)
        return DeviceState.from_numpy(arr, dt)

    # -- gates ------------------------------------------------------------
    def apply_gate(self, gate, state, nqubits):
        """In place on the device state (qibojit's convention,
        doc/source/getting-started/backends.rst:57-61); returns the state."""
        state = self._as_device_state(state)
        if isinstance(state, DeviceDensity):
            self._run_density(state, compile_queue([gate], self, state.nsys, self._describe))
            return state
        desc = describe_gate(gate, self)
        if desc is not None:
            if self.dtype == "complex128" and not self.strict_fp64:
                # one gate through qgb_apply_circuit: dense 1-qubit gates with
                # the pairs shared between FP64 and double-float warps (0.67
                # of HBM against 0.35 in IEEE FP64 at 30 qubits)
                self.engine_gb.apply_many(state, [desc])
            else:
                self.engine_gb.apply(state, desc[0], desc[2], desc[1])
        return state

    def matrix_fused(self, fgate):
        return G.fused_matrix(fgate.target_qubits, fgate.gates, self)

    def _describe(self, gate):
        return describe_gate(gate, self)

    # -- density matrices and channels ----------------------------------------
    def apply_channel(self, channel, state, nqubits):
        """Backend.apply_channel (backends/abstract.py:2297-2318).  On a
        density matrix: the channel's superoperator on the device, in place.
        On a state vector: one of the channel's gates, or none, drawn with
        the channel's probabilities by the device sampler and applied."""
        state = self._as_device_state(state)
        if isinstance(state, DeviceDensity):
            self._run_density(state, compile_queue([channel], self, state.nsys, self._describe))
            return state
        probs = [float(np.real(c)) for c in channel.coefficients]
        probs.append(max(0.0, 1.0 - sum(probs)))
        index = int(self.sample_shots(np.asarray(probs), 1)[0])
        if index != len(channel.gates):
            state = self.apply_gate(channel.gates[index], state, nqubits)
        return state

    def depolarizing_error_density_matrix(self, gate, state, nqubits):
        """backends/abstract.py:2095-2132, in place on the device."""
        return self.apply_channel(gate, state, nqubits)

    def reset_error_density_matrix(self, gate, state, nqubits):
        """backends/abstract.py:2212-2232: the reset map of ``gate``'s p_0 and
        p_1 on its qubit, into a new density matrix (the caller may combine
        it with the input, as ThermalRelaxationChannel.apply does)."""
        from .density import _reset_superop

        rho = self._as_device_state(state).copy()
        q = gate.target_qubits[0]
        kw = gate.init_kwargs
        n = rho.nsys
        self._run_density(rho, [("gates", [((q, q + n), (), _reset_superop(float(kw["p_0"]), float(kw["p_1"])))])])
        return rho

    def thermal_error_density_matrix(self, gate, state, nqubits):
        """backends/abstract.py:2234-2241: ``gate`` acts on (q, q + n) of the
        2n-qubit vector of the density matrix, in place."""
        rho = self._as_device_state(state)
        m = np.asarray(gate.matrix(self), dtype=np.complex128)
        self._run_density(rho, [("gates", [(tuple(gate.qubits), (), m)])])
        return rho

    def _run_density(self, rho, items):
        """Run compiled density items (qibo_gb300.density.compile_queue) on ``rho``."""
        fuse = self.blocked and self.fuse and rho.nqubits >= FUSE_MIN_QUBITS
        for kind, payload in items:
            if kind == "gates":
                self.engine_gb.apply_many(rho, payload, blocked=self.blocked, strict_fp64=self.strict_fp64, fuse=fuse)
            elif kind == "wide":
                self._apply_wide_channel(rho, payload)
            else:
                raise RuntimeError("collapsing measurements on density matrices run through repeated execution")

    def _apply_wide_channel(self, rho, channel):
        """A channel whose superoperator exceeds a 5-qubit gate, as the
        reference's weighted sum (backends/abstract.py:2305-2310): each term
        on a copy of rho, accumulated on the device."""
        keep, terms = wide_terms(channel, self, rho.nsys)
        eng, lib, s = self.engine_gb, self.rt.lib, self.rt.stream
        acc = DeviceDensity(rho.nsys, rho.dtype, self.rt)
        work = DeviceDensity(rho.nsys, rho.dtype, self.rt)
        eng.axpby(acc, rho, keep, 0.0)
        fuse = self.blocked and self.fuse and rho.nqubits >= FUSE_MIN_QUBITS
        for c, pair in terms:
            check(lib.qgb_memcpy_d2d(work.ptr, rho.ptr, rho.nbytes, s))
            eng.apply_many(work, pair, blocked=self.blocked, strict_fp64=self.strict_fp64, fuse=fuse)
            eng.axpby(acc, work, c, 1.0)
        check(lib.qgb_memcpy_d2d(rho.ptr, acc.ptr, rho.nbytes, s))

    def _initial_density(self, initial_state, nqubits):
        if initial_state is None:
            return DeviceDensity.zero(nqubits, self.dtype)
        shape = tuple(initial_state.shape)
        if shape != (2**nqubits, 2**nqubits):
            raise ValueError(f"Given initial state has shape {shape} instead of the expected "
                             f"{(2 ** nqubits, 2 ** nqubits)}.")
        if isinstance(initial_state, DeviceDensity):
            return initial_state  # in place, like qibojit
        return self._as_device_state(initial_state)

    def _execute_density(self, circuit, initial_state, nshots):
        """execute_circuit for ``density_matrix=True`` circuits
        (backends/abstract.py:2442-2512 and _execute_circuit, :3306-3345):
        gates and channels as 2n-qubit operations on the device (see
        qibo_gb300.density), collapsing measurements through repeated
        execution."""
        nqubits = circuit.nqubits
        self._validate_nqubits(nqubits, density_matrix=True)
        if initial_state is not None and hasattr(initial_state, "queue") and hasattr(initial_state, "nqubits"):
            if not getattr(initial_state, "density_matrix", False):
                raise ValueError("Cannot set circuit with density_matrix False as initial state for circuit with "
                                 "density_matrix True.")
            return self.execute_circuit(initial_state + circuit, None, nshots)
        if getattr(circuit, "repeated_execution", False):
            return self.execute_circuit_repeated(circuit, nshots, initial_state)
        try:
            rho = self._initial_density(initial_state, nqubits)
            self._run_density(rho, compile_queue(circuit.queue, self, nqubits, self._describe))
        except DeviceOutOfMemory:
            raise RuntimeError(f"State does not fit in {self.device} memory."
                               "Please switch the execution device to a "
                               "different one using ``qibo.set_device``.")
        QuantumState, CircuitResult = self._result_classes()
        if circuit.measurements:
            result = CircuitResult(rho, circuit.measurements, backend=self, nshots=nshots)
        else:
            result = QuantumState(rho, backend=self)
        circuit._final_state = result
        return result

    def execute_circuit(self, circuit, initial_state=None, nshots=1000):
        nqubits = circuit.nqubits
        if getattr(circuit, "density_matrix", False):
            return self._execute_density(circuit, initial_state, nshots)
        self._validate_nqubits(nqubits)
        if getattr(circuit, "repeated_execution", False):
            if not circuit.measurements and not getattr(circuit, "has_collapse", False):
                raise RuntimeError("Attempting to perform noisy simulation with `density_matrix=False` and no "
                                   "Measurement gate in the Circuit.")
            return self.execute_circuit_repeated(circuit, nshots, initial_state)
        if getattr(circuit, "accelerators", None):
            raise NotImplementedError("distributed (multi-GPU) circuits are not supported by qibo_gb300")
        if initial_state is not None and hasattr(initial_state, "queue") and hasattr(initial_state, "nqubits"):
            return self.execute_circuit(initial_state + circuit, None, nshots)
        try:
            if initial_state is None:
                state = DeviceState.zero(nqubits, self.dtype)
            else:
                src = initial_state
                shape = tuple(src.shape)
                if shape != (2**nqubits,):
                    raise ValueError(f"Given initial state has shape {shape} instead of the expected "
                                     f"{(2 ** nqubits,)}.")
                if isinstance(src, DeviceState):
                    state = src  # in place, like qibojit
                else:
                    arr = np.asarray(src)
                    dt = arr.dtype if arr.dtype in (np.complex64, np.complex128) else self.dtype
                    state = DeviceState.from_numpy(arr, dt)
            descs = [d for d in (describe_gate(g, self) for g in circuit.queue) if d is not None]
            self.engine_gb.apply_many(state, descs, blocked=self.blocked, strict_fp64=self.strict_fp64,
                                      fuse=self.fuse and nqubits >= FUSE_MIN_QUBITS)
            if state.dtype == np.complex64 and self.renormalize_c64 and descs:
                self.engine_gb.renormalize(state)
        except DeviceOutOfMemory:
            raise RuntimeError(f"State does not fit in {self.device} memory."
                               "Please switch the execution device to a "
                               "different one using ``qibo.set_device``.")
        QuantumState, CircuitResult = self._result_classes()
        if circuit.measurements:
            result = CircuitResult(state, circuit.measurements, backend=self, nshots=nshots)
        else:
            result = QuantumState(state, backend=self)
        circuit._final_state = result
        return result

    def execute_circuits(self, circuits, initial_states=None, nshots=1000, processes=None):
        """Backend.execute_circuits (:2514-2530, a host thread pool in the
        reference) through the continuous-batching server
        (``qibo_gb300.parallel.serve_circuits``): the circuits overlap on the
        device, same-shape mid-sized circuits replay one captured graph.
        ``processes`` is accepted and unused."""
        from .parallel import serve_circuits

        return serve_circuits(self, circuits, initial_states, nshots)

    def server(self):
        """The backend's ``serving.Server`` (created on first use)."""
        srv = getattr(self, "_server", None)
        if srv is None:
            from .serving import Server

            srv = self._server = Server(nslots=8)
        return srv

    def execute_circuit_repeated(self, circuit, nshots, initial_state=None):
        """Backend.execute_circuit_repeated (backends/abstract.py:2532-2636)
        on the device, for circuits with collapsing measurements and for
        noisy state-vector circuits.  Every shot runs the circuit again from
        the initial state.  A collapsing measurement draws its outcome on the
        device from the FP64 probabilities of its sorted qubits (as
        gates/measurements.py:199-218), and the collapse reads it straight
        from device memory.  A unitary channel on a state vector applies one
        of its gates per shot, drawn for all shots at once by the device
        sampler (Backend.apply_channel, :2314-2318).  The final measurements
        draw one shot each into a device array.  Density-matrix circuits
        return the mean of the shots' final density matrices, accumulated on
        the device (:2603-2625)."""
        density = bool(getattr(circuit, "density_matrix", False))
        if getattr(circuit, "has_collapse", False) and not circuit.measurements and not density:
            raise RuntimeError("The circuit contains only collapsing measurements (`collapse=True`) but "
                               "`density_matrix=False`. Please set `density_matrix=True` to retrieve the final "
                               "state after execution.")
        nqubits, nshots = circuit.nqubits, int(nshots)
        nvec = 2 * nqubits if density else nqubits
        eng, rt, lib = self.engine_gb, self.rt, self.rt.lib
        flags = ((_lib.QGB_PLAN_BLOCKED if self.blocked else 0) | (_lib.QGB_PLAN_STRICT_FP64 if self.strict_fp64 else 0)
                 | (_lib.QGB_PLAN_FUSE if self.blocked and self.fuse and nvec >= FUSE_MIN_QUBITS else 0))
        for g in circuit.queue:
            if getattr(g, "symbolic_parameters", None):
                raise NotImplementedError("parameters that depend on measurement outcomes are not supported")
        # the circuit as items: runs of gates (packed once), collapsing
        # measurements, channels
        items, collapse_gates = [], []
        if density:
            for kind, payload in compile_queue(circuit.queue, self, nqubits, self._describe):
                if kind == "gates":
                    items.append(("gates", eng.pack_ops(payload), len(payload)))
                elif kind == "wide":
                    items.append(("wide", payload, 0))
                else:
                    qs = sorted(payload.target_qubits)
                    items.append(("collapse", int_array(qs), len(qs)))
                    collapse_gates.append((payload, len(qs)))
        else:
            run = []
            for g in circuit.queue:
                if type(g).__name__ == "M":
                    if getattr(g, "collapse", False):
                        if run:
                            items.append(("gates", eng.pack_ops(run), len(run)))
                            run = []
                        qs = sorted(g.target_qubits)
                        items.append(("collapse", int_array(qs), len(qs)))
                        collapse_gates.append((g, len(qs)))
                    continue
                if is_channel(g):
                    if not any(c.__name__ == "UnitaryChannel" for c in type(g).__mro__):
                        raise NotImplementedError(f"{type(g).__name__} cannot be applied to statevector.")
                    if run:
                        items.append(("gates", eng.pack_ops(run), len(run)))
                        run = []
                    opts = []
                    for x in g.gates:
                        d = describe_gate(x, self)
                        opts.append(None if d is None else eng.pack_ops([d]))
                    probs = [float(np.real(c)) for c in g.coefficients]
                    probs.append(max(0.0, 1.0 - sum(probs)))
                    draws = eng.sample(self._device_probs(np.asarray(probs)), nshots, self._next_key(), counts=False)
                    items.append(("channel", (opts, draws), 0))
                    continue
                d = describe_gate(g, self)
                if d is not None:
                    run.append(d)
            if run:
                items.append(("gates", eng.pack_ops(run), len(run)))
        meas_q = [q for m in circuit.measurements for q in m.target_qubits]
        nmeas, ncol = len(meas_q), len(collapse_gates)
        if density:
            probs_call, collapse_call, scratch_sizes = (lib.qgb_density_probabilities, lib.qgb_density_collapse,
                                                        [lib.qgb_density_scratch_bytes()])
        else:
            probs_call, collapse_call = lib.qgb_probabilities, lib.qgb_collapse
            scratch_sizes = [lib.qgb_norm_scratch_bytes(), lib.qgb_probs_scratch_bytes(nqubits, nmeas)]
            scratch_sizes += [lib.qgb_probs_scratch_bytes(nqubits, m) for _, m in collapse_gates]
        try:
            state = DeviceDensity(nqubits, self.dtype) if density else DeviceState(nqubits, self.dtype)
            mean = DeviceDensity(nqubits, self.dtype) if density else None
            init = None
            if initial_state is not None:
                init = self._as_device_state(initial_state)
                if tuple(init.shape) != tuple(state.shape):
                    raise ValueError(f"Given initial state has shape {tuple(init.shape)} instead of the expected "
                                     f"{tuple(state.shape)}.")
                if init.dtype != state.dtype:
                    init = init.astype(state.dtype)
            # device buffers for every shot, allocated once
            col_probs = [DeviceArray((2**m,), np.float64, rt) for _, m in collapse_gates]
            fin_probs = DeviceArray((2**nmeas,), np.float64, rt)
            outcomes = DeviceArray((max(1, nshots * ncol),), np.int64, rt)
            samples = DeviceArray((max(1, nshots),), np.int64, rt)
            sizes = scratch_sizes + [lib.qgb_sample_scratch_bytes(nmeas)]
            sizes += [lib.qgb_sample_scratch_bytes(m) for _, m in collapse_gates]
            scratch = rt.scratch(max(sizes))
            mq = int_array(meas_q)
            code, s = state.code, rt.stream
            n_probs = nqubits  # the probability and collapse calls take the system size
            for shot in range(nshots):
                if init is None:
                    check(lib.qgb_state_zero(state.ptr, nvec, code, s))
                else:
                    check(lib.qgb_memcpy_d2d(state.ptr, init.ptr, state.nbytes, s))
                j = 0
                for kind, payload, k in items:
                    if kind == "gates":
                        ops, allc = payload
                        check(lib.qgb_apply_circuit(state.ptr, nvec, code, ops, k, allc.ctypes.data_as(_lib.dp),
                                                    flags, s))
                    elif kind == "channel":
                        opts, draws = payload
                        idx = int(draws[shot])
                        if idx < len(opts) and opts[idx] is not None:
                            ops, allc = opts[idx]
                            check(lib.qgb_apply_circuit(state.ptr, nvec, code, ops, 1, allc.ctypes.data_as(_lib.dp),
                                                        flags, s))
                    elif kind == "wide":
                        self._apply_wide_channel(state, payload)
                    else:
                        out = outcomes.ptr + 8 * (shot * ncol + j)
                        check(probs_call(state.ptr, n_probs, code, payload, k, col_probs[j].ptr, scratch, s))
                        check(lib.qgb_sample(col_probs[j].ptr, k, 1, self._next_key(), out, None, scratch, s))
                        check(collapse_call(state.ptr, n_probs, code, payload, k, out, 1, scratch, s))
                        j += 1
                if nmeas:
                    check(probs_call(state.ptr, n_probs, code, mq, nmeas, fin_probs.ptr, scratch, s))
                    check(lib.qgb_sample(fin_probs.ptr, nmeas, 1, self._next_key(), samples.ptr + 8 * shot, None,
                                         scratch, s))
                if density:
                    eng.axpby(mean, state, 1.0 / nshots, 1.0 if shot else 0.0)
            dec = samples.to_numpy()[:nshots]
            col = outcomes.to_numpy()[: nshots * ncol].reshape(nshots, ncol) if ncol else None
        except DeviceOutOfMemory:
            raise RuntimeError(f"State does not fit in {self.device} memory.")
        # each collapsing measurement keeps its outcomes, as gate.result.add_shot does
        for j, (g, m) in enumerate(collapse_gates):
            res = getattr(g, "result", None)
            if res is not None and hasattr(res, "register_samples"):
                res.register_samples(self.samples_to_binary(col[:, j], m))
        binary = np.asarray(self.samples_to_binary(dec, nmeas)) if nmeas else None
        if density:
            QuantumState, CircuitResult = self._result_classes()
            if circuit.measurements:
                result = CircuitResult(mean, circuit.measurements, backend=self, samples=binary, nshots=nshots)
            else:
                result = QuantumState(mean, backend=self)
            circuit._final_state = result
            return result
        result = self._outcomes_class()(circuit.measurements, backend=self, samples=binary, nshots=nshots)
        if hasattr(result, "_repeated_execution_frequencies"):  # as backends/abstract.py:2631-2633
            result._repeated_execution_frequencies = collections.Counter(
                "".join(str(int(b)) for b in row) for row in binary)
        circuit._final_state = result
        return result

    def collapse_state(self, state, qubits, shot, nqubits, normalize=True, density_matrix=False):
        """Backend.collapse_state / _collapse_statevector
        (backends/abstract.py:2424-2440, :3279-3304): keep the slice of the
        state that agrees with outcome ``shot[0]`` of ``qubits`` (qubits[0]
        the most significant bit), divided by its norm, zeros elsewhere.  On
        the device and in place (qibojit's convention); returns the state."""
        st = self._as_device_state(state)
        outcome = int(np.asarray(shot).reshape(-1)[0])
        if density_matrix or isinstance(st, DeviceDensity):
            # _collapse_density_matrix (:3249-3277): rows and columns, over the kept trace
            self.engine_gb.density_collapse(st, list(qubits), outcome, normalize)
            return st
        self.engine_gb.collapse(st, list(qubits), outcome, normalize)
        return st

    def exp_value_observable_symbolic_from_samples(self, circuit, diagonal_terms_coefficients,
                                                   diagonal_terms_observables, diagonal_terms_qubits, nqubits,
                                                   constant, nshots):
        """Backend.exp_value_observable_symbolic_from_samples
        (backends/abstract.py:3056-3140) on the device.  The circuit runs
        once.  For each group of terms measured together, a copy of the state
        is rotated to the group's basis with the reference's basis rotations
        (X: H, Y: (Y + Z)/sqrt(2), gates/gates.py:191-241).  ``nshots``
        outcomes of the group's measured qubits are drawn on the device, and
        each term's sample mean of (-1)^parity comes from integer parity
        counts (qgb_parity_counts).  That is the reference's
        frequency-weighted sum (:2873-2926) without moving the samples to
        the host."""
        saved = getattr(circuit, "_final_state", None)
        try:
            result = self.execute_circuit(circuit, nshots=nshots)
            state = self._as_device_state(result.state())
        finally:
            circuit._final_state = saved
        h = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)
        ybasis = np.array([[1, -1j], [1j, -1]], dtype=np.complex128) / np.sqrt(2)
        expval = 0.0
        for coefs, observables, terms_qubits in zip(diagonal_terms_coefficients, diagonal_terms_observables,
                                                     diagonal_terms_qubits):
            measured = {}
            for qubits, observable in zip(terms_qubits, observables):
                for q, factor in zip(qubits, observable):
                    if factor != "I" and q not in measured:
                        measured[q] = factor
            qmap = list(measured)
            masks = []
            for qubits in terms_qubits:
                mk = 0
                for q in qubits:
                    mk ^= 1 << (len(qmap) - 1 - qmap.index(q))
                masks.append(mk)
            if not qmap:
                expval += sum(coefs)
                continue
            work = state.copy()
            rot = [((q,), (), h if f == "X" else ybasis) for q, f in measured.items() if f in ("X", "Y")]
            if rot:
                self.engine_gb.apply_many(work, rot, blocked=self.blocked, strict_fp64=self.strict_fp64)
            probs = self.engine_gb.probabilities(work, qmap)
            samples = self.engine_gb.sample_device(probs, nshots, self._next_key())
            means = self.engine_gb.parity_means(samples, nshots, masks)
            expval += sum(c * m for c, m in zip(coefs, means))
        return constant + expval

    # -- measurement --------------------------------------------------------
    def calculate_probabilities(self, state, qubits, nqubits, density_matrix=False):
        st = self._as_device_state(state)
        if density_matrix or isinstance(st, DeviceDensity):
            return self.engine_gb.density_probabilities(st, list(qubits))
        return self.engine_gb.probabilities(st, list(qubits))

    def _device_probs(self, probabilities):
        if isinstance(probabilities, DeviceArray):
            return probabilities
        p = np.asarray(probabilities, dtype=np.float64)
        m = max(1, (len(p) - 1).bit_length())
        padded = np.zeros(2**m, dtype=np.float64)
        padded[: len(p)] = p
        arr = DeviceArray((2**m,), np.float64, self.rt)
        self.rt.h2d(arr.ptr, padded)
        return arr

    def set_seed(self, seed):
        self._seed = seed
        self._seed_calls = 0
        np.random.seed(seed)

    def _next_key(self) -> int:
        """64-bit Philox key for the next sampling call: a function of the
        seed and of how many sampling calls followed ``set_seed``."""
        if self._seed is None:
            return int.from_bytes(os.urandom(8), "little")
        k = (int(self._seed) * 0x9E3779B97F4A7C15 + self._seed_calls * 0xD1B54A32D192ED03) & (2**64 - 1)
        self._seed_calls += 1
        return k

    def sample_shots(self, probabilities, nshots):
        n = len(probabilities)
        out = self.engine_gb.sample(self._device_probs(probabilities), int(nshots), self._next_key(), counts=False)
        if n and out.size and out.max() >= n:
            raise RuntimeError("sampled an index beyond the distribution")
        return out

    def sample_frequencies(self, probabilities, nshots):
        """Counter of outcome -> count.  The shots are the same draws either
        way: with fewer shots than outcomes they are copied back and counted
        on the host (nshots int64 instead of a 2^m histogram), otherwise the
        histogram is built on the device; the Counter is filled from whole
        arrays."""
        n = len(probabilities)
        probs = self._device_probs(probabilities)
        if int(nshots) < n:
            shots = self.engine_gb.sample(probs, int(nshots), self._next_key(), counts=False)
            vals, cnts = np.unique(shots, return_counts=True)
            return collections.Counter(dict(zip(vals.tolist(), cnts.tolist())))
        counts = self.engine_gb.sample(probs, int(nshots), self._next_key(), counts=True)
        nz = np.flatnonzero(counts[:n])
        return collections.Counter(dict(zip(nz.tolist(), counts[nz].tolist())))

    # -- observables ----------------------------------------------------------
    def expectation_value(self, hamiltonian, state, normalize):
        from .observables import dense_expectation

        st = self._as_device_state(state)
        return dense_expectation(self.engine_gb, hamiltonian, st, normalize)

    def exp_value_observable_symbolic(self, circuit, terms, term_qubits, term_coefficients, nqubits):
        result = circuit._final_state if circuit._final_state is not None else self.execute_circuit(circuit)
        st = self._as_device_state(result.state())
        xs, zs, cs = [], [], []
        const = 0.0
        for term, qubits, coef in zip(terms, term_qubits, term_coefficients):
            x, z = pauli_masks(term, qubits)
            if x == 0 and z == 0:
                const += float(np.real(coef))
                continue
            xs.append(x)
            zs.append(z)
            cs.append(float(np.real(coef)))
        if isinstance(st, DeviceDensity):  # Re Tr(P rho) per term (:2985-3030)
            val = self.engine_gb.density_expect_pauli(st, xs, zs, cs) if cs else 0.0
            if const:
                val += const * self.engine_gb.density_trace(st)
            return val
        val = self.engine_gb.expect_pauli(st, xs, zs, cs) if cs else 0.0
        if const:
            val += const * self.engine_gb.norm2(st)
        return val


class StandaloneBase:
    """Minimal stand-in for ``qibo.backends.abstract.Backend`` when qibo is
    not installed: validation, dtype handling, host casts."""

    def __init__(self):
        self.dtype = "complex128"
        self.nthreads = 1
        self.matrices = None
        self.versions = {}
        self.numeric_types = (int, float, complex)
        self.tensor_types = (np.ndarray,)

    def set_dtype(self, dtype):
        if str(dtype) not in ("complex64", "complex128"):
            raise ValueError(f"qibo_gb300 supports complex64 and complex128, not {dtype}")
        self.dtype = str(dtype)

    def set_threads(self, nthreads):
        self.nthreads = int(nthreads)

    def set_device(self, device):
        if not device.startswith("/GPU"):
            raise ValueError(f"Device {device} is not available for {self}.")

    def _validate_nqubits(self, nqubits, density_matrix=False):
        if not isinstance(nqubits, int) or nqubits < 1:
            raise ValueError(f"nqubits must be a positive integer, but got {nqubits}.")
        maxq = int(os.environ.get("QIBO_MAX_QUBITS", "-1"))
        if maxq != -1 and nqubits > maxq:
            raise ValueError(f"Requested {nqubits} qubits for state vector allocation; the maximum allowed is "
                             f"{maxq} qubits (QIBO_MAX_QUBITS).")

    def cast(self, array, dtype=None, copy=False):
        return np.array(array, dtype=dtype or self.dtype, copy=copy) if copy else np.asarray(array, dtype=dtype or self.dtype)

    def to_numpy(self, array):
        return np.asarray(array)

    def samples_to_binary(self, samples, nqubits):
        """Backend.samples_to_binary (backends/abstract.py:2783-2786)."""
        qrange = np.arange(nqubits - 1, -1, -1, dtype=np.int32)
        return np.right_shift(np.asarray(samples)[:, None], qrange) % 2

    def __repr__(self):
        return f"{self.name} ({self.platform})"


class GB300Backend(GB300Methods, StandaloneBase):
    """Standalone backend (no qibo installed)."""

    def __init__(self, dtype="complex128"):
        StandaloneBase.__init__(self)
        self.set_dtype(dtype)
        self._gb300_init(dtype)

    def _result_classes(self):
        from .result import CircuitResult, QuantumState

        return QuantumState, CircuitResult

    def _outcomes_class(self):
        from .result import MeasurementOutcomes

        return MeasurementOutcomes
