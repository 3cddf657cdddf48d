"""``Circuit`` with the interface of the reference's ``qibo.models.Circuit``
(models/circuit.py:122-1521) for hosts without qibo, plus ``QFT``
(models/qft.py:9-58).  With qibo installed, qibo's own Circuit runs on the
same backend through the plugin."""

from __future__ import annotations

import math
from typing import Iterable

import numpy as np

from . import gates as G
from .fusion import fuse_gates


class Circuit:
    def __init__(self, nqubits: int, density_matrix: bool = False, accelerators=None, **kwargs):
        if not isinstance(nqubits, int) or nqubits < 1:
            raise ValueError(f"nqubits must be a positive integer, got {nqubits}")
        if accelerators:
            raise NotImplementedError("multi-device (distributed) circuits are not supported")
        self.nqubits = nqubits
        self.density_matrix = bool(density_matrix)
        self.accelerators = None
        self.queue = []
        self.measurements = []
        self.has_collapse = False
        self.has_unitary_channel = False
        self._final_state = None

    # -- construction (models/circuit.py:608-760) -------------------------
    def add(self, gate):
        if isinstance(gate, Iterable) and not isinstance(gate, G.Gate):
            for g in gate:
                self.add(g)
            return
        for q in gate.qubits:
            if q >= self.nqubits or q < 0:
                raise ValueError(f"gate {gate} acts on qubit {q} of a {self.nqubits}-qubit circuit")
        if isinstance(gate, G.M):
            # basis rotations first, once (models/circuit.py:658-666)
            for base in gate.basis:
                if base not in self.queue:
                    self.add(base)
            self.queue.append(gate)
            if gate.collapse:
                self.has_collapse = True
            else:
                self.measurements.append(gate)
            return gate.result
        self.queue.append(gate)
        # a gate after a measurement on the same qubits makes that measurement
        # collapse the state (models/circuit.py:684-689)
        for measurement in list(self.measurements):
            if set(measurement.qubits) & set(gate.qubits):
                measurement.collapse = True
                self.has_collapse = True
                self.measurements.remove(measurement)
        if isinstance(gate, G.UnitaryChannel):  # models/circuit.py:697-698
            self.has_unitary_channel = True
        return None

    @property
    def repeated_execution(self) -> bool:
        """models/circuit.py:321-324."""
        return self.has_collapse or (self.has_unitary_channel and not self.density_matrix)

    @property
    def ngates(self):
        return len(self.queue)

    def __add__(self, other: "Circuit") -> "Circuit":
        if self.density_matrix != other.density_matrix:
            raise ValueError("Cannot add circuits with different density_matrix settings.")
        c = Circuit(max(self.nqubits, other.nqubits), density_matrix=self.density_matrix)
        c.add(self.queue)
        c.add(other.queue)
        return c

    def copy(self, deep: bool = False) -> "Circuit":
        """A circuit with the same gates (models/circuit.py ``copy``); with
        ``deep`` the gates are copies, so changing their parameters leaves
        this circuit's alone."""
        import copy as _copy

        c = Circuit(self.nqubits, density_matrix=self.density_matrix)
        c.add([_copy.deepcopy(g) for g in self.queue] if deep else list(self.queue))
        return c

    def invert(self) -> "Circuit":
        c = Circuit(self.nqubits)
        c.add([g.dagger() for g in reversed(self.queue) if not isinstance(g, G.M)])
        return c

    # -- parameters (models/circuit.py:788-907) ---------------------------
    @property
    def trainable_gates(self):
        return [g for g in self.queue if g.trainable and g.nparams > 0 and not isinstance(g, G.Unitary)]

    def associate_gates_with_parameters(self):
        out = []
        for g in self.trainable_gates:
            out.extend([g] * len(g.parameters))
        return out

    def get_parameters(self, format: str = "list"):
        if format == "flatlist":
            return [p for g in self.trainable_gates for p in g.parameters]
        return [tuple(g.parameters) for g in self.trainable_gates]

    def set_parameters(self, parameters):
        gates = self.trainable_gates
        flat = np.asarray(parameters, dtype=object)
        if flat.ndim == 1 and len(flat) == sum(g.nparams for g in gates):
            k = 0
            for g in gates:
                g.parameters = tuple(float(v) for v in flat[k:k + g.nparams])
                k += g.nparams
            return
        if len(parameters) != len(gates):
            raise ValueError(f"expected {len(gates)} parameter entries, got {len(parameters)}")
        for g, p in zip(gates, parameters):
            g.parameters = p

    # -- fusion (models/circuit.py:954-1003) ------------------------------
    def fuse(self, max_qubits: int = 2) -> "Circuit":
        if not 1 <= max_qubits <= 5:
            raise ValueError("max_qubits must be between 1 and 5")
        c = Circuit(self.nqubits, density_matrix=self.density_matrix)
        c.queue = fuse_gates(self.queue, max_qubits, G.FusedGate, lambda g: isinstance(g, (G.M, G.Channel)))
        c.measurements = list(self.measurements)
        return c

    # -- execution (models/circuit.py:1071-1110) ---------------------------
    def execute(self, initial_state=None, nshots: int = 1000, backend=None):
        from . import get_backend

        backend = backend or get_backend()
        return backend.execute_circuit(self, initial_state=initial_state, nshots=nshots)

    def __call__(self, initial_state=None, nshots: int = 1000):
        return self.execute(initial_state=initial_state, nshots=nshots)

    def __repr__(self):
        return f"Circuit(nqubits={self.nqubits}, ngates={self.ngates})"


def QFT(nqubits: int, with_swaps: bool = True, **kwargs) -> Circuit:
    """Quantum Fourier transform: H on each qubit followed by controlled
    phases CU1(i2, i1, pi / 2^(i2-i1)), then SWAPs (models/qft.py:47-58)."""
    c = Circuit(nqubits, **kwargs)
    for i1 in range(nqubits):
        c.add(G.H(i1))
        for i2 in range(i1 + 1, nqubits):
            c.add(G.CU1(i2, i1, math.pi / 2 ** (i2 - i1)))
    if with_swaps:
        for q in range(nqubits // 2):
            c.add(G.SWAP(q, nqubits - q - 1))
    return c
