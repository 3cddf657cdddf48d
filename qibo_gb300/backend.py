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

from . import gates as G
from ._lib import DeviceOutOfMemory
from .device import DeviceArray, DeviceState, Runtime
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
    if name.endswith("Channel") or name in ("KrausChannel", "UnitaryChannel", "PauliNoiseChannel"):
        raise NotImplementedError("noise channels need the density-matrix path, not supported")
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
        if density_matrix:
            raise NotImplementedError("qibo_gb300 simulates state vectors only")
        self._validate_nqubits(nqubits)
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
        if arr.ndim != 1:
            raise NotImplementedError("qibo_gb300 simulates state vectors only")
        dt = dtype or (arr.dtype if arr.dtype in (np.complex64, np.complex128) else self.dtype)
        return DeviceState.from_numpy(arr, dt)

    # -- gates ------------------------------------------------------------
    def apply_gate(self, gate, state, nqubits):
        """In place on the device state (qibojit's convention,
        doc/source/getting-started/backends.rst:57-61); returns the state."""
        state = self._as_device_state(state)
        desc = describe_gate(gate, self)
        if desc is not None:
            self.engine_gb.apply(state, desc[0], desc[2], desc[1])
        return state

    def matrix_fused(self, fgate):
        return G.fused_matrix(fgate.target_qubits, fgate.gates, self)

    def execute_circuit(self, circuit, initial_state=None, nshots=1000):
        nqubits = circuit.nqubits
        if getattr(circuit, "density_matrix", False):
            raise NotImplementedError("qibo_gb300 simulates state vectors only")
        self._validate_nqubits(nqubits)
        if getattr(circuit, "repeated_execution", False):
            raise NotImplementedError("collapse / noisy repeated execution is not supported by qibo_gb300")
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
        """Backend.execute_circuits (:2514): here sequential on the device."""
        if initial_states is None:
            initial_states = [None] * len(circuits)
        return [self.execute_circuit(c, s, nshots) for c, s in zip(circuits, initial_states)]

    # -- measurement --------------------------------------------------------
    def calculate_probabilities(self, state, qubits, nqubits, density_matrix=False):
        if density_matrix:
            raise NotImplementedError("qibo_gb300 simulates state vectors only")
        st = self._as_device_state(state)
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
        n = len(probabilities)
        counts = self.engine_gb.sample(self._device_probs(probabilities), int(nshots), self._next_key(), counts=True)
        nz = np.nonzero(counts[:n])[0]
        return collections.Counter({int(i): int(counts[i]) for i in nz})

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
