"""Gate objects with qibo's constructor signatures and attributes.

These mirror the reference's ``qibo.gates`` (gates/gates.py, gates/abstract.py,
gates/special.py, gates/measurements.py) closely enough that code written
against qibo runs unchanged on hosts where qibo itself is not installed:
``gate.qubits`` is controls then targets (gates/abstract.py:440),
``gate.matrix(backend)`` is the closed form of backends/npmatrices.py,
``gate.controlled_by(*q)`` marks extra controls (gates/abstract.py:155).
When qibo is installed, the backend accepts qibo's own gate objects too.
"""

from __future__ import annotations

import cmath
import math
from typing import Sequence, Tuple

import numpy as np

SQ2 = 1.0 / math.sqrt(2.0)


def _u3(t, p, l):
    c, s = math.cos(t / 2), math.sin(t / 2)
    ep, em = cmath.exp(1j * (p + l) / 2), cmath.exp(1j * (p - l) / 2)
    return np.array([[ep.conjugate() * c, -em.conjugate() * s], [em * s, ep * c]])


def _ctrl(u):
    m = np.eye(4, dtype=np.complex128)
    m[2:, 2:] = u
    return m


def _matrix(name: str, p: Sequence[float]) -> np.ndarray:
    """Closed-form complex128 matrix (backends/npmatrices.py:27-473)."""
    if name == "H":
        return np.array([[1, 1], [1, -1]], dtype=np.complex128) * SQ2
    if name == "X":
        return np.array([[0, 1], [1, 0]], dtype=np.complex128)
    if name == "Y":
        return np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    if name == "Z":
        return np.array([[1, 0], [0, -1]], dtype=np.complex128)
    if name == "SX":
        return np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]) / 2
    if name == "SXDG":
        return np.array([[1 - 1j, 1 + 1j], [1 + 1j, 1 - 1j]]) / 2
    if name == "S":
        return np.array([[1, 0], [0, 1j]], dtype=np.complex128)
    if name == "SDG":
        return np.array([[1, 0], [0, -1j]], dtype=np.complex128)
    if name == "T":
        return np.array([[1, 0], [0, cmath.exp(1j * math.pi / 4)]])
    if name == "TDG":
        return np.array([[1, 0], [0, cmath.exp(-1j * math.pi / 4)]])
    if name == "I":
        return np.eye(2, dtype=np.complex128)
    if name == "RX":
        c, s = math.cos(p[0] / 2), -1j * math.sin(p[0] / 2)
        return np.array([[c, s], [s, c]], dtype=np.complex128)
    if name == "RY":
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)
    if name == "RZ":
        e = cmath.exp(0.5j * p[0])
        return np.array([[e.conjugate(), 0], [0, e]])
    if name == "U1":
        return np.array([[1, 0], [0, cmath.exp(1j * p[0])]])
    if name == "U2":
        ep, em = cmath.exp(1j * (p[0] + p[1]) / 2), cmath.exp(1j * (p[0] - p[1]) / 2)
        return np.array([[ep.conjugate(), -em.conjugate()], [em, ep]]) * SQ2
    if name == "U3":
        return _u3(*p)
    base = {"CNOT": "X", "CY": "Y", "CZ": "Z", "CSX": "SX", "CSXDG": "SXDG", "CRX": "RX", "CRY": "RY",
            "CRZ": "RZ", "CU1": "U1", "CU2": "U2", "CU3": "U3"}
    if name in base:
        return _ctrl(_matrix(base[name], p))
    if name == "SWAP":
        return np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)
    if name == "iSWAP":
        return np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]])
    if name == "FSWAP":
        return np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, -1]], dtype=np.complex128)
    if name == "fSim":
        c, s, e = math.cos(p[0]), -1j * math.sin(p[0]), cmath.exp(-1j * p[1])
        return np.array([[1, 0, 0, 0], [0, c, s, 0], [0, s, c, 0], [0, 0, 0, e]])
    if name in ("RXX", "RYY"):
        c, s = math.cos(p[0] / 2), -1j * math.sin(p[0] / 2)
        sg = 1 if name == "RXX" else -1
        return np.array([[c, 0, 0, sg * s], [0, c, s, 0], [0, s, c, 0], [sg * s, 0, 0, c]])
    if name == "RZZ":
        e = cmath.exp(0.5j * p[0])
        return np.diag([e.conjugate(), e, e, e.conjugate()])
    if name == "TOFFOLI":
        m = np.eye(8, dtype=np.complex128)
        m[6:, 6:] = [[0, 1], [1, 0]]
        return m
    if name == "CCZ":
        m = np.eye(8, dtype=np.complex128)
        m[7, 7] = -1
        return m
    raise NotImplementedError(f"no matrix for gate {name}")


class Gate:
    """Base gate: ``target_qubits``, ``control_qubits``, ``parameters``."""

    nparams = 0
    ncontrols = 0

    def __init__(self, *args, trainable: bool = True, **kwargs):
        # parameters by keyword (theta, phi, lam: qibo's names) come after
        # the positional ones
        kw = tuple(kwargs.pop(key) for key in ("theta", "phi", "lam") if key in kwargs)
        nq = len(args) - max(0, self.nparams - len(kw))
        qubits = tuple(int(q) for q in args[:nq])
        params = tuple(args[nq:]) + kw
        if kwargs.get("q") is not None:
            qubits = (int(kwargs.pop("q")),)
        self.name = type(self).__name__
        # control qubits are kept sorted (gates/abstract.py:144-146)
        self.control_qubits: Tuple[int, ...] = tuple(sorted(qubits[: self.ncontrols]))
        self.target_qubits: Tuple[int, ...] = qubits[self.ncontrols:]
        self.is_controlled_by = False
        self.trainable = trainable
        self._parameters = tuple(float(x) for x in params)
        self.init_args = list(args)
        self.init_kwargs = {}

    @property
    def qubits(self) -> Tuple[int, ...]:
        return self.control_qubits + self.target_qubits

    @property
    def parameters(self):
        return self._parameters

    @parameters.setter
    def parameters(self, values):
        if np.isscalar(values):
            values = (values,)
        self._parameters = tuple(float(v) for v in values)

    def matrix(self, backend=None) -> np.ndarray:
        return _matrix(self.name, self._parameters)

    def controlled_by(self, *qubits):
        """Control the gate on extra qubits (gates/abstract.py:155)."""
        if self.is_controlled_by or self.control_qubits:
            raise NotImplementedError("controlled_by on a gate that already has controls")
        self.is_controlled_by = True
        self.control_qubits = tuple(sorted(int(q) for q in qubits))
        return self

    def dagger(self) -> "Gate":
        return Unitary(np.conj(self.matrix()).T, *self.qubits) if not self.is_controlled_by else \
            Unitary(np.conj(self.matrix()).T, *self.target_qubits).controlled_by(*self.control_qubits)

    def apply(self, backend, state, nqubits):
        return backend.apply_gate(self, state, nqubits)

    def __repr__(self):
        return f"{self.name}{self.qubits}"


def _make(name, nparams=0, ncontrols=0):
    return type(name, (Gate,), {"nparams": nparams, "ncontrols": ncontrols})


H, X, Y, Z, S, SDG, T, TDG, SX, SXDG = (_make(n) for n in ("H", "X", "Y", "Z", "S", "SDG", "T", "TDG", "SX", "SXDG"))
RX, RY, RZ, U1 = (_make(n, 1) for n in ("RX", "RY", "RZ", "U1"))
U2 = _make("U2", 2)
U3 = _make("U3", 3)
CNOT, CY, CZ, CSX, CSXDG = (_make(n, 0, 1) for n in ("CNOT", "CY", "CZ", "CSX", "CSXDG"))
CRX, CRY, CRZ, CU1 = (_make(n, 1, 1) for n in ("CRX", "CRY", "CRZ", "CU1"))
CU2 = _make("CU2", 2, 1)
CU3 = _make("CU3", 3, 1)
SWAP, iSWAP, FSWAP = (_make(n) for n in ("SWAP", "iSWAP", "FSWAP"))
fSim = _make("fSim", 2)
RXX, RYY, RZZ = (_make(n, 1) for n in ("RXX", "RYY", "RZZ"))
TOFFOLI = _make("TOFFOLI", 0, 2)
CCZ = _make("CCZ", 0, 2)


class I(Gate):  # noqa: E742 (qibo's gate name)
    def matrix(self, backend=None):
        return np.eye(2 ** len(self.target_qubits), dtype=np.complex128)


class Unitary(Gate):
    """Arbitrary unitary on ``qubits`` (gates/gates.py:2774)."""

    def __init__(self, unitary, *qubits, trainable: bool = True, **kwargs):
        super().__init__(*qubits, trainable=trainable)
        self._matrix = np.asarray(unitary, dtype=np.complex128)
        d = 2 ** len(self.target_qubits)
        if self._matrix.shape != (d, d):
            raise ValueError(f"Unitary of shape {self._matrix.shape} on {len(self.target_qubits)} qubits")
        self._parameters = (self._matrix,)

    @property
    def parameters(self):
        return (self._matrix,)

    @parameters.setter
    def parameters(self, values):
        m = values[0] if isinstance(values, (tuple, list)) else values
        self._matrix = np.asarray(m, dtype=np.complex128)

    def matrix(self, backend=None):
        return self._matrix


class MeasurementResult:
    """Outcomes of one measurement gate (measurements.py:61-163): the samples
    registered after execution, one binary row per shot."""

    def __init__(self, gate):
        self.gate = gate
        self._samples = None

    def register_samples(self, samples):
        self._samples = np.asarray(samples)

    def has_samples(self):
        return self._samples is not None

    def samples(self, binary: bool = True):
        if self._samples is None:
            raise RuntimeError("the measurement has no samples: execute the circuit first")
        if binary:
            return self._samples
        n = self._samples.shape[-1]
        return (self._samples @ (2 ** np.arange(n - 1, -1, -1))).astype(np.int64)

    def reset(self):
        self._samples = None


def _basis_rotation(basis, q):
    """The gate that rotates ``basis`` onto Z on qubit q (X: H, Y: (Y + Z)/sqrt(2),
    Z: none; gates/gates.py:191-292)."""
    name = basis if isinstance(basis, str) else getattr(basis, "__name__", str(basis))
    if name == "Z":
        return None
    if name == "X":
        return H(q)
    if name == "Y":
        return Unitary(np.array([[1, -1j], [1j, -1]], dtype=np.complex128) / np.sqrt(2), q)
    raise NotImplementedError(f"measurement basis {name}: only X, Y and Z are supported")


class M(Gate):
    """Measurement of ``qubits`` (gates/measurements.py:11-218).  A no-op on
    the state, except that ``collapse=True`` measures during the circuit:
    the state is projected onto the drawn outcome and the circuit runs once
    per shot (the backend's ``execute_circuit_repeated``).  ``basis`` (X, Y
    or Z, one for all qubits or one per qubit) adds the reference's basis
    rotations before the measurement (gates/measurements.py:96-105)."""

    def __init__(self, *q, register_name=None, collapse: bool = False, basis=None, p0=None, p1=None):
        super().__init__(*q)
        if p0 is not None or p1 is not None:
            raise NotImplementedError("bit-flip measurement noise is not supported by qibo_gb300")
        self.register_name = register_name
        self.collapse = bool(collapse)
        bases = basis if isinstance(basis, (list, tuple)) else [basis or "Z"] * len(self.target_qubits)
        if len(bases) != len(self.target_qubits):
            raise ValueError(f"Given basis list has length {len(bases)} while the measurement acts on "
                             f"{len(self.target_qubits)} qubits.")
        self.basis = [g for g in (_basis_rotation(b, q) for b, q in zip(bases, self.target_qubits)) if g is not None]
        self.result = MeasurementResult(self)

    def matrix(self, backend=None):
        raise NotImplementedError("measurement gates have no matrix")

    def apply(self, backend, state, nqubits):
        if not self.collapse:
            return state
        qubits = sorted(self.target_qubits)
        probs = backend.calculate_probabilities(state, qubits, nqubits)
        shot = backend.sample_shots(probs, 1)
        self.result.register_samples(backend.samples_to_binary(np.asarray(shot), len(qubits)))
        return backend.collapse_state(state, qubits, shot, nqubits)


class FusedGate(Gate):
    """Block of gates applied as one dense matrix (gates/special.py:28).

    ``target_qubits`` is the sorted union of the member gates' qubits
    (gates/special.py:38, :59-60)."""

    def __init__(self, *q):
        super().__init__(*sorted(set(q)))
        self.gates = []

    def append(self, gate):
        self.gates.append(gate)

    def matrix(self, backend=None):
        return fused_matrix(self.target_qubits, self.gates, backend)

    def __repr__(self):
        return f"FusedGate{self.target_qubits}[{len(self.gates)}]"


def gate_full_matrix(gate, backend=None) -> Tuple[Tuple[int, ...], np.ndarray]:
    """(qubits, matrix) of a gate with ``controlled_by`` controls folded in
    (identity on every control pattern except all-ones)."""
    m = np.asarray(gate.matrix(backend), dtype=np.complex128)
    if getattr(gate, "is_controlled_by", False) and gate.control_qubits:
        d = 2 ** (len(gate.control_qubits) + len(gate.target_qubits))
        full = np.eye(d, dtype=np.complex128)
        full[d - m.shape[0]:, d - m.shape[0]:] = m
        return tuple(gate.control_qubits) + tuple(gate.target_qubits), full
    return tuple(gate.qubits), m


def fused_matrix(target_qubits: Sequence[int], gates, backend=None) -> np.ndarray:
    """Product of member gate matrices embedded on ``target_qubits`` (sorted),
    the same unitary as Backend.matrix_fused (backends/abstract.py:2680-2717),
    built with an einsum per gate instead of kron + sparse products."""
    tq = list(target_qubits)
    k = len(tq)
    total = np.eye(2**k, dtype=np.complex128).reshape((2,) * (2 * k))
    letters = "abcdefghijklmnopqrstuvwxyz"
    for g in gates:
        qs, m = gate_full_matrix(g, backend)
        kg = len(qs)
        mt = m.reshape((2,) * (2 * kg))
        # rows of total: axes 0..k-1 (output), cols: k..2k-1
        out_ax = [letters[i] for i in range(k)]
        in_ax = [letters[k + i] for i in range(k)]
        new = list(out_ax)
        g_out = []
        g_in = []
        for j, q in enumerate(qs):
            pos = tq.index(q)
            g_in.append(out_ax[pos])
            g_out.append(letters[2 * k + j])
            new[pos] = letters[2 * k + j]
        spec = "".join(g_out + g_in) + "," + "".join(out_ax + in_ax) + "->" + "".join(new + in_ax)
        total = np.einsum(spec, mt, total)
    return total.reshape(2**k, 2**k)


# noise channels (gates/channels.py), in the gates namespace as in qibo
from .channels import (AmplitudeDampingChannel, Channel, DepolarizingChannel, KrausChannel,  # noqa: E402
                       PauliNoiseChannel, PhaseDampingChannel, ReadoutErrorChannel, ResetChannel,
                       ThermalRelaxationChannel, UnitaryChannel)
