"""Density-matrix circuits of the golden fixtures.

``make_golden.py`` builds them with the reference's ``qibo.gates`` and
``qibo.Circuit``; the tests build the same constructor calls with
``qibo_gb300.gates`` / ``qibo_gb300.Circuit`` (or replay them through the
oracle), so a fixture and its check describe one circuit.  Every random
matrix comes from a seeded generator in this file.
"""

from __future__ import annotations

import numpy as np


def unitary(d: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def random_rho(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    m = rng.normal(size=(2**n, 2**n)) + 1j * rng.normal(size=(2**n, 2**n))
    rho = m @ m.conj().T
    return rho / np.trace(rho)


def noisy(gates, Circuit, n: int):
    """Gates with controls and controlled_by, and every channel kind: one-
    and two-qubit superoperators, 3-qubit Kraus / unitary / depolarizing
    channels (weighted sums), both thermal-relaxation branches (T1 >= T2 on
    a qubit other than 0), readout error, reset."""
    g = gates
    c = Circuit(n, density_matrix=True)
    c.add(g.H(0))
    c.add(g.CNOT(0, 1))
    c.add(g.RY(2, 0.7))
    c.add(g.U3(3, 0.3, 1.1, -0.4).controlled_by(0, 2))
    c.add(g.DepolarizingChannel((1,), 0.1))
    c.add(g.PauliNoiseChannel(2, [("X", 0.1), ("Y", 0.05), ("Z", 0.2)]))
    c.add(g.AmplitudeDampingChannel(3, 0.3))
    c.add(g.PhaseDampingChannel(0, 0.25))
    c.add(g.ResetChannel(1, [0.15, 0.05]))
    c.add(g.CZ(1, 2))
    c.add(g.ThermalRelaxationChannel(2, [1.0, 1.5, 0.4, 0.2]))
    c.add(g.ThermalRelaxationChannel(3, [2.0, 1.0, 0.3]))
    c.add(g.DepolarizingChannel((0, 3), 0.2))
    c.add(g.KrausChannel([(0,), (1, 3)], [np.sqrt(0.6) * unitary(2, 1), np.sqrt(0.4) * unitary(4, 2)]))
    c.add(g.UnitaryChannel([(1, 2), (0,)], [(0.3, unitary(4, 3)), (0.2, unitary(2, 4))]))
    c.add(g.ReadoutErrorChannel(2, np.array([[0.9, 0.1], [0.25, 0.75]])))
    c.add(g.TOFFOLI(3, 1, 0))
    c.add(g.fSim(2, 0, 0.6, 0.25))
    c.add(g.DepolarizingChannel((0, 1, 2), 0.15))
    for q in range(4, n):
        c.add(g.CNOT(q - 1, q))
        c.add(g.AmplitudeDampingChannel(q, 0.1 + 0.05 * q))
        c.add(g.RX(q, 0.3 * q))
    return c


def layers(gates, Circuit, n: int, depth: int, seed: int):
    """U3 + CZ brickwork with single-qubit depolarizing and amplitude damping
    after every layer and a two-qubit Pauli channel on alternating pairs."""
    g = gates
    ang = np.random.default_rng(seed).uniform(0, 2 * np.pi, (depth, n, 3))
    c = Circuit(n, density_matrix=True)
    for layer in range(depth):
        for q in range(n):
            c.add(g.U3(q, *ang[layer, q]))
        for q in range(layer % 2, n - 1, 2):
            c.add(g.CZ(q, q + 1))
        for q in range(n):
            c.add(g.DepolarizingChannel((q,), 0.01 * (1 + q % 3)))
        for q in range(layer % 2, n, 3):
            c.add(g.AmplitudeDampingChannel(q, 0.05))
        for q in range((layer + 1) % 2, n - 1, 2):
            c.add(g.PauliNoiseChannel((q, q + 1), [("XZ", 0.02), ("YY", 0.01), ("ZI", 0.03)]))
    return c


# name -> (nqubits, builder(gates, Circuit), initial-state seed or None for |0><0|)
CASES = {
    "dm_noisy4": (4, lambda g, C: noisy(g, C, 4), 5),
    "dm_noisy6": (6, lambda g, C: noisy(g, C, 6), 6),
    "dm_layers8": (8, lambda g, C: layers(g, C, 8, 3, 88), None),
}

# probability subsets checked per case (caller order)
PROB_SETS = {"dm_noisy4": [[0, 1, 2, 3], [2, 0], [3]], "dm_noisy6": [[5, 1, 0], [4]],
             "dm_layers8": [[0, 7], [3, 6, 1, 4]]}

# entries of the n = 8 final density matrix kept in the fixture (1 MB whole)
SAMPLED = {"dm_layers8": 4096}


def sample_indices(n: int, count: int, seed: int = 8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, 4**n, size=count, dtype=np.int64)
    diag = np.arange(2**n, dtype=np.int64) * (2**n + 1)
    return np.unique(np.concatenate([idx, diag[:64]]))
