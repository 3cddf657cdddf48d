"""Noise channels with qibo's constructor signatures and attributes.

They mirror the reference's ``qibo.gates.channels`` (gates/channels.py)
for hosts where qibo is not installed: every channel exposes ``gates``
(its Kraus operators or unitaries as gate objects), ``coefficients`` and
``coefficient_sum`` (Backend.apply_channel, backends/abstract.py:2297-2312,
computes (1 - sum c_k) rho + sum_k c_k K_k rho K_k^dagger from them), and
the ``init_kwargs`` the reference's special-cased channels read
(``lam`` of DepolarizingChannel, ``p_0``/``p_1`` of ResetChannel and
ThermalRelaxationChannel, ``e_t2`` or ``p_z`` of the latter).  With qibo
installed, the backend takes qibo's own channel objects the same way.
"""

from __future__ import annotations

import itertools
import math
from typing import Sequence

import numpy as np

from . import gates as G

PRECISION_TOL = 1e-8


def _qubit_lists(qubits, count):
    if isinstance(qubits, int):
        return [(qubits,)] * count
    if isinstance(qubits, tuple):
        return [qubits] * count
    if not isinstance(qubits, list):
        raise TypeError(f"``qubits`` must be of type int or tuple or int. Got {type(qubits)} instead")
    if not all(isinstance(q, tuple) for q in qubits):
        raise TypeError("All elements of ``qubits`` list must be tuples.")
    return qubits


class Channel(G.Gate):
    """Base channel (gates/channels.py:16-41)."""

    def __init__(self):
        super().__init__()
        self.coefficients = tuple()
        self.gates = tuple()
        self.coefficient_sum = 0.0

    @property
    def qubits(self):
        return tuple(self.target_qubits)

    def controlled_by(self, *q):
        raise ValueError(f"Noise channel cannot be controlled on qubits {q}.")

    def matrix(self, backend=None):
        raise NotImplementedError("noise channels have no matrix")

    def apply(self, backend, state, nqubits):
        if len(state.shape) == 1:
            raise NotImplementedError(f"{self.__class__.__name__} cannot be applied to statevector.")
        return backend.apply_channel(self, state, nqubits)

    def __repr__(self):
        return f"{self.name}{tuple(self.target_qubits)}"


class KrausChannel(Channel):
    """sum_k K_k rho K_k^dagger (gates/channels.py:203-326).  ``qubits``: an
    int or tuple for every operator, or a list of tuples (one per operator);
    ``operators``: matrices (2^k x 2^k) or gate objects."""

    def __init__(self, qubits, operators):
        super().__init__()
        self.name = "KrausChannel"
        qubits = _qubit_lists(qubits, len(operators))
        if isinstance(operators[0], G.Gate):
            if qubits:
                operators = [G.Unitary(op.matrix(), *qs) for op, qs in zip(operators, qubits)]
            gates = list(operators)
        else:
            if len(qubits) != len(operators):
                raise ValueError(f"``qubits`` list has length {len(qubits)} while {len(operators)} operators were given.")
            gates = []
            for qs, m in zip(qubits, operators):
                m = np.asarray(m)
                if m.shape != (2 ** len(qs), 2 ** len(qs)):
                    raise ValueError(f"Invalid Kraus operator shape {m.shape} for acting on {len(qs)} qubits.")
                gates.append(G.Unitary(m, *qs))
        self.gates = tuple(gates)
        self.target_qubits = tuple(sorted({q for g in self.gates for q in g.target_qubits}))
        self.coefficients = (1,) * len(self.gates)
        self.coefficient_sum = 1
        self.init_args = [self.gates]
        self.init_kwargs = {}


class UnitaryChannel(KrausChannel):
    """(1 - sum p_k) rho + sum_k p_k U_k rho U_k^dagger; on state vectors one
    U_k (or none) drawn per application (gates/channels.py:329-388)."""

    def __init__(self, qubits, operators):
        if not all(isinstance(pair, tuple) for pair in operators):
            raise TypeError("``operators`` must be a list of tuples ``(pk, Uk)``.")
        probabilities = [pair[0] for pair in operators]
        if any(p < 0 or p > 1 for p in probabilities):
            raise ValueError("Probabilities should be between 0 and 1.")
        super().__init__(qubits, [pair[1] for pair in operators])
        self.name = "UnitaryChannel"
        self.coefficients = tuple(probabilities)
        self.coefficient_sum = sum(probabilities)
        if self.coefficient_sum > 1 + PRECISION_TOL or self.coefficient_sum < 0:
            raise ValueError(f"UnitaryChannel probability sum should be between 0 and 1 but is {self.coefficient_sum}.")
        self.init_args = [probabilities, self.gates]

    def apply(self, backend, state, nqubits):
        return backend.apply_channel(self, state, nqubits)


_PAULI = {"I": G.I, "X": G.X, "Y": G.Y, "Z": G.Z}


class PauliNoiseChannel(UnitaryChannel):
    """Pauli strings with probabilities, e.g. ``[("X", 0.1), ("Z", 0.2)]``
    (gates/channels.py:391-468)."""

    def __init__(self, qubits, operators: Sequence):
        if isinstance(qubits, int):
            qubits = (qubits,)
        qubits = tuple(qubits)
        gates, probs = [], []
        for pauli, p in operators:
            f = G.FusedGate(*qubits)
            for q, s in zip(qubits, pauli):
                f.append(_PAULI[s](q))
            gates.append(f)
            probs.append(p)
        super().__init__([], list(zip(probs, gates)))
        self.name = "PauliNoiseChannel"
        self.init_args = qubits
        self.init_kwargs = dict(operators)


class DepolarizingChannel(PauliNoiseChannel):
    """(1 - lam) rho + lam Tr_q(rho) (x) I / 2^k on density matrices; on state
    vectors the equivalent Pauli noise with every non-identity string at
    probability lam / 4^k (gates/channels.py:471-528)."""

    def __init__(self, qubits, lam: float):
        if isinstance(qubits, int):
            qubits = (qubits,)
        qubits = tuple(qubits)
        nterms = 4 ** len(qubits)
        if lam < 0 or lam > nterms / (nterms - 1):
            raise ValueError(f"Depolarizing parameter must be in between 0 and {nterms / (nterms - 1)}.")
        paulis = ["".join(p) for p in itertools.product("IXYZ", repeat=len(qubits))][1:]
        super().__init__(qubits, [(p, lam / nterms) for p in paulis])
        self.name = "DepolarizingChannel"
        self.target_qubits = qubits
        self.init_args = [qubits]
        self.init_kwargs = {"lam": lam}


class ThermalRelaxationChannel(KrausChannel):
    """Thermal relaxation of one qubit (gates/channels.py:531-707), with
    p_0 = (1 - e^(-t/T1)) (1 - eta), p_1 = (1 - e^(-t/T1)) eta and, for
    T1 >= T2, p_z = (e^(-t/T1) - e^(-t/T2)) / 2 (eta the excited
    population, t the gate time)."""

    def __init__(self, qubit: int, parameters: list):
        if len(parameters) not in (3, 4):
            raise ValueError(f"``parameters`` list must have 3 or 4 elements while {len(parameters)} were given.")
        t_1, t_2, time = parameters[:3]
        eta = parameters[3] if len(parameters) == 4 else 0.0
        if eta < 0 or eta > 1:
            raise ValueError(f"Invalid excited state population {eta}.")
        if time < 0.0:
            raise ValueError(f"Invalid gate time: {time} < 0.")
        if t_1 <= 0.0:
            raise ValueError(f"Invalid t_1 relaxation time parameter: {t_1} <= 0.0.")
        if t_2 <= 0.0:
            raise ValueError(f"Invalid t_2 relaxation time parameter: {t_2} <= 0.0.")
        if t_2 > 2 * t_1:
            raise ValueError("Invalid t_2 relaxation time parameter: t_2 > 2 * t_1.")
        p_reset = 1 - math.exp(-time / t_1)
        p_0, p_1 = p_reset * (1 - eta), p_reset * eta
        kw = {}
        if t_1 < t_2:
            e_t2 = math.exp(-time / t_2)
            # Kraus form of the T1 < T2 map (amplitude damping towards the
            # equilibrium populations plus the remaining dephasing)
            k = math.sqrt(4 * e_t2**2 + (p_0 - p_1) ** 2)
            c = math.sqrt(max(0.0, 1 - (p_0 + p_1 + k) / 2))
            c2 = math.sqrt(max(0.0, 1 - (p_0 + p_1 - k) / 2))
            ops = [math.sqrt(p_0) * np.array([[0, 1], [0, 0]]), math.sqrt(p_1) * np.array([[0, 0], [1, 0]]),
                   c * np.array([[(p_0 - p_1 - k) / (2 * e_t2), 0], [0, 1]]),
                   c2 * np.array([[(p_0 - p_1 + k) / (2 * e_t2), 0], [0, 1]])]
            kw["e_t2"] = e_t2
        else:
            p_z = (math.exp(-time / t_1) - math.exp(-time / t_2)) / 2
            ops = [math.sqrt(p_0) * np.array([[1, 0], [0, 0]]), math.sqrt(p_0) * np.array([[0, 1], [0, 0]]),
                   math.sqrt(p_1) * np.array([[0, 0], [1, 0]]), math.sqrt(p_1) * np.array([[0, 0], [0, 1]]),
                   math.sqrt(p_z) * np.array([[1, 0], [0, -1]]),
                   math.sqrt(max(0.0, 1 - p_0 - p_1 - p_z)) * np.eye(2)]
            kw["p_z"] = p_z
        super().__init__([(qubit,)] * len(ops), ops)
        self.name = "ThermalRelaxationChannel"
        self.t_1, self.t_2 = t_1, t_2
        self.init_args = [qubit, t_1, t_2, time]
        self.init_kwargs = dict(kw, excited_population=eta, p_0=p_0, p_1=p_1)


class AmplitudeDampingChannel(KrausChannel):
    """K_0 = [[1, 0], [0, sqrt(1 - g)]], K_1 = [[0, sqrt(g)], [0, 0]]
    (gates/channels.py:710-747)."""

    def __init__(self, qubit, gamma: float):
        if not isinstance(gamma, float):
            raise TypeError(f"gamma must be type float, but it is type {type(gamma)}.")
        if gamma < 0.0 or gamma > 1.0:
            raise ValueError("gamma must be a float between 0 and 1.")
        ops = [np.array([[1, 0], [0, math.sqrt(1 - gamma)]], dtype=complex),
               np.array([[0, math.sqrt(gamma)], [0, 0]], dtype=complex)]
        super().__init__([(qubit,)] * 2, ops)
        self.name = "AmplitudeDampingChannel"
        self.init_kwargs = {"gamma": gamma}


class PhaseDampingChannel(KrausChannel):
    """K_0 = [[1, 0], [0, sqrt(1 - g)]], K_1 = [[0, 0], [0, sqrt(g)]]
    (gates/channels.py:750-787)."""

    def __init__(self, qubit, gamma: float):
        if not isinstance(gamma, float):
            raise TypeError(f"gamma must be type float, but it is type {type(gamma)}.")
        if gamma < 0.0 or gamma > 1.0:
            raise ValueError("gamma must be a float between 0 and 1.")
        ops = [np.array([[1, 0], [0, math.sqrt(1 - gamma)]], dtype=complex),
               np.array([[0, 0], [0, math.sqrt(gamma)]], dtype=complex)]
        super().__init__([(qubit,)] * 2, ops)
        self.name = "PhaseDampingChannel"
        self.init_kwargs = {"gamma": gamma}


class ReadoutErrorChannel(KrausChannel):
    """Quantum-to-classical readout error with transition matrix P
    (P[i, j] = p(j | i), rows summing to 1): Kraus operators
    sqrt(P[k, j]) |j><k| (gates/channels.py:790-835)."""

    def __init__(self, qubits, probabilities):
        P = np.asarray(probabilities, dtype=float)
        if np.any(P.sum(axis=1) < 1 - PRECISION_TOL) or np.any(P.sum(axis=1) > 1 + PRECISION_TOL):
            raise ValueError("all rows of probabilities must sum to 1.")
        if isinstance(qubits, int):
            qubits = (qubits,)
        qubits = tuple(qubits)
        d = len(P)
        ops = []
        for j in range(d):
            for k in range(d):
                op = np.zeros((d, d))
                op[j, k] = math.sqrt(P[k, j])
                ops.append(op)
        super().__init__([qubits] * len(ops), ops)
        self.name = "ReadoutErrorChannel"
        self.probabilities = P


class ResetChannel(KrausChannel):
    """(1 - p_0 - p_1) rho + Tr_q(rho) (x) (p_0 |0><0| + p_1 |1><1|)
    (gates/channels.py:838-887)."""

    def __init__(self, qubit, probabilities):
        if len(probabilities) != 2:
            raise ValueError(f"ResetChannel needs 2 probabilities, got {len(probabilities)} instead.")
        p_0, p_1 = probabilities
        if p_0 < 0:
            raise ValueError(f"Invalid p_0 ({p_0} < 0).")
        if p_1 < 0:
            raise ValueError(f"Invalid p_1 ({p_1} < 0).")
        if p_0 + p_1 > 1 + PRECISION_TOL:
            raise ValueError(f"Invalid probabilities (p_0 + p_1 = {p_0 + p_1} > 1).")
        ops = [math.sqrt(p_0) * np.array([[1, 0], [0, 0]]), math.sqrt(p_0) * np.array([[0, 1], [0, 0]]),
               math.sqrt(p_1) * np.array([[0, 0], [1, 0]]), math.sqrt(p_1) * np.array([[0, 0], [0, 1]])]
        if p_0 + p_1 < 1:
            ops.append(math.sqrt(abs(1 - p_0 - p_1)) * np.eye(2))
        super().__init__([(qubit,)] * len(ops), ops)
        self.name = "ResetChannel"
        self.init_kwargs = {"p_0": p_0, "p_1": p_1}
