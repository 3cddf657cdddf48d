"""Density matrices on the device: gates and channels as 2n-qubit operations.

A density matrix rho of n qubits is a ``DeviceDensity``, the 2n-qubit vector
v[i 2^n + j] = rho[i, j] (row qubit q = vector qubit q, column qubit q =
vector qubit n + q; the reference's ``rho.ravel()``,
backends/abstract.py:2234-2241).  On that vector:

* a gate U on qubits T (controls C) is U on T (controls C) followed by
  conj(U) on T + n (controls C + n): rho -> U rho U^dagger, the two einsums
  of Backend.apply_gate with a density matrix (backends/abstract.py:
  2322-2361) and of _apply_gate_controlled_by_density_matrix (:3199-3247);
* a channel on qubits T is the superoperator S on (T, T + n), one dense
  gate of 2|T| qubits:
  - Kraus / unitary / Pauli channels (Backend.apply_channel,
    backends/abstract.py:2297-2312, rho -> (1 - sum c_k) rho +
    sum_k c_k K_k rho K_k^dagger): S = (1 - sum c_k) I + sum_k c_k K_k (x) conj(K_k);
  - DepolarizingChannel (depolarizing_error_density_matrix, :2095-2132,
    rho -> (1 - lam) rho + lam Tr_T(rho) (x) I / d): S = (1 - lam) I +
    (lam / d) |Phi><Phi| with Phi = sum_r |r>|r>;
  - ResetChannel (reset_error_density_matrix, :2212-2232, rho ->
    (1 - p0 - p1) rho + Tr_q(rho) (x) (p0 |0><0| + p1 |1><1|));
  - ThermalRelaxationChannel (gates/channels.py:678-707): for T1 < T2 the
    channel's 4 x 4 matrix on (q, q + n) itself (thermal_error_density_
    matrix, :2234-2241); otherwise the reset map minus p_z rho plus
    p_z Z rho Z, where the reference applies that Z to qubit 0 whatever the
    channel's qubit (gates/channels.py:702-706) -- kept, so that results
    agree with it.
  A superoperator of more than 5 vector qubits (a Kraus channel on 3 or
  more qubits) runs as the reference's weighted sum instead: each term on a
  copy, accumulated with ``qgb_state_axpby``.

The gate lists then run through ``qgb_apply_circuit`` like any state-vector
circuit of 2n qubits: shared-memory passes, and engine fusion with tensor
cores once 2n >= 12.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from . import gates as G

SKIP_GATES = ("M", "I", "Align", "CallbackGate")
MAX_SUPEROP_QUBITS = 5  # the widest dense gate of qgb_apply_circuit


def is_channel(gate) -> bool:
    return hasattr(gate, "coefficients") and hasattr(gate, "gates") and type(gate).__name__.endswith("Channel")


def embed(m: np.ndarray, qubits: Sequence[int], target: Sequence[int]) -> np.ndarray:
    """Matrix ``m`` on ``qubits`` (its index-bit order) as a matrix on all of
    ``target`` (in that order), identity on the others."""
    qubits, target = list(qubits), list(target)
    k = len(target)
    rest = [q for q in target if q not in qubits]
    full = np.kron(np.asarray(m, dtype=np.complex128), np.eye(2 ** len(rest), dtype=np.complex128))
    order = qubits + rest
    perm = [order.index(q) for q in target]
    return full.reshape((2,) * (2 * k)).transpose(perm + [k + p for p in perm]).reshape(2**k, 2**k)


def gate_pair(desc, n: int) -> List[tuple]:
    """(qubits, controls, U) on the rows and (qubits + n, controls + n,
    conj(U)) on the columns."""
    qs, ctrl, m = desc
    return [(tuple(qs), tuple(ctrl), m),
            (tuple(q + n for q in qs), tuple(c + n for c in ctrl), np.conj(m))]


def _reset_superop(p0: float, p1: float) -> np.ndarray:
    """4 x 4 on (q, q + n), index 2 row_bit + column_bit."""
    s = (1.0 - p0 - p1) * np.eye(4, dtype=np.complex128)
    s[0, 0] += p0
    s[0, 3] += p0
    s[3, 0] += p1
    s[3, 3] += p1
    return s


def _zz() -> np.ndarray:
    z = np.diag([1.0, -1.0]).astype(np.complex128)
    return np.kron(z, z)


def superoperator(channel, backend, n: int):
    """(vector qubits, S) of ``channel`` on an n-qubit density matrix, or
    None when S would exceed a 5-qubit gate."""
    name = type(channel).__name__
    kw = getattr(channel, "init_kwargs", {}) or {}
    if name == "DepolarizingChannel":
        T = sorted(set(channel.target_qubits))
        if 2 * len(T) > MAX_SUPEROP_QUBITS:
            return None
        d = 2 ** len(T)
        lam = float(kw["lam"])
        s = (1.0 - lam) * np.eye(d * d, dtype=np.complex128)
        diag = [r * d + r for r in range(d)]
        s[np.ix_(diag, diag)] += lam / d
        return tuple(T) + tuple(q + n for q in T), s
    if name == "ResetChannel":
        q = channel.target_qubits[0]
        return (q, q + n), _reset_superop(float(kw["p_0"]), float(kw["p_1"]))
    if name == "ThermalRelaxationChannel":
        q = channel.target_qubits[0]
        p0, p1 = float(kw["p_0"]), float(kw["p_1"])
        if channel.t_1 < channel.t_2:
            e = float(kw["e_t2"])
            s = np.array([[1 - p1, 0, 0, p0], [0, e, 0, 0], [0, 0, e, 0], [p1, 0, 0, 1 - p0]], dtype=np.complex128)
            return (q, q + n), s
        pz = float(kw["p_z"])
        T = sorted({q, 0})
        V = tuple(T) + tuple(t + n for t in T)
        s = embed(_reset_superop(p0, p1), (q, q + n), V) - pz * np.eye(4 ** len(T)) + pz * embed(_zz(), (0, n), V)
        return V, s
    # Kraus, unitary and Pauli channels: the weighted sum of their gates
    parts = [G.gate_full_matrix(g, backend) for g in channel.gates]
    T = sorted({q for qs, _ in parts for q in qs})
    if 2 * len(T) > MAX_SUPEROP_QUBITS:
        return None
    s = (1.0 - float(np.real(channel.coefficient_sum))) * np.eye(4 ** len(T), dtype=np.complex128)
    for c, (qs, m) in zip(channel.coefficients, parts):
        k = embed(m, qs, T)
        s += complex(c) * np.kron(k, np.conj(k))
    return tuple(T) + tuple(q + n for q in T), s


def compile_queue(queue, backend, n: int, describe) -> List[tuple]:
    """The circuit as items on the 2n-qubit vector: ("gates", descs),
    ("wide", channel) for a channel run as a weighted sum, ("collapse",
    measurement gate).  ``describe(gate)`` gives (qubits, controls, matrix)."""
    items: List[tuple] = []
    run: List[tuple] = []

    def flush():
        if run:
            items.append(("gates", list(run)))
            run.clear()

    for g in queue:
        name = type(g).__name__
        if name in SKIP_GATES:
            if name == "M" and getattr(g, "collapse", False):
                flush()
                items.append(("collapse", g))
            continue
        if is_channel(g):
            sup = superoperator(g, backend, n)
            if sup is None:
                flush()
                items.append(("wide", g))
            else:
                run.append((sup[0], (), sup[1]))
            continue
        run.extend(gate_pair(describe(g), n))
    flush()
    return items


def wide_terms(channel, backend, n: int) -> Tuple[float, List[Tuple[float, List[tuple]]]]:
    """(1 - sum c_k, [(c_k, gate pair of K_k)]) for a channel run as a sum."""
    terms = []
    for c, g in zip(channel.coefficients, channel.gates):
        qs, m = G.gate_full_matrix(g, backend)
        terms.append((float(np.real(c)), gate_pair((qs, (), m), n)))
    return 1.0 - float(np.real(channel.coefficient_sum)), terms
