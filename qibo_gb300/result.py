"""Result objects with the interface of the reference's ``qibo.result``
(result.py:31-872), used when qibo itself is not installed.  With qibo
installed the backend returns qibo's own ``QuantumState``/``CircuitResult``.
"""

from __future__ import annotations

import collections

import numpy as np


def frequencies_to_binary(frequencies, nqubits):
    """measurements.py:15-16."""
    return collections.Counter({f"{k:b}".zfill(nqubits): v for k, v in frequencies.items()})


class QuantumState:
    """Final state of a circuit (result.py:31-163)."""

    def __init__(self, state, backend=None):
        from . import get_backend

        self.backend = backend or get_backend()
        self.density_matrix = len(state.shape) == 2
        self.nqubits = int(np.log2(state.shape[0]))
        self._state = state

    def state(self, numpy: bool = False):
        if numpy:
            return np.asarray(self._state)
        return self._state

    def probabilities(self, qubits=None):
        if qubits is None:
            qubits = tuple(range(self.nqubits))
        return self.backend.calculate_probabilities(self._state, qubits, self.nqubits,
                                                    density_matrix=self.density_matrix)

    def to_dict(self):
        return {"state": self.state(numpy=True), "dtype": type(self).__name__}

    def dump(self, filename: str):
        """result.py:125-134: ``np.save`` of ``to_dict``."""
        np.save(filename, self.to_dict())

    @classmethod
    def load(cls, filename: str):
        payload = np.load(filename, allow_pickle=True).item()
        return cls(payload["state"])

    def __str__(self):
        return f"QuantumState(nqubits={self.nqubits})"


class CircuitResult(QuantumState):
    """State plus measurement outcomes (result.py:805-872, MeasurementOutcomes
    :166-548).  Probabilities of the measured qubits are computed eagerly
    (result.py:828), frequencies and samples lazily."""

    def __init__(self, final_state, measurements, backend=None, samples=None, nshots=1000):
        super().__init__(final_state, backend)
        self.measurements = measurements
        self.nshots = nshots
        self.measured_qubits = tuple(q for m in measurements for q in m.target_qubits)
        if not self.measured_qubits:
            raise ValueError("Circuit does not contain measurements. Use a `QuantumState` instead.")
        self._probs = QuantumState.probabilities(self, self.measured_qubits) if samples is None else None
        self._samples = samples
        self._frequencies = None

    def probabilities(self, qubits=None):
        return QuantumState.probabilities(self, qubits)

    def has_samples(self):
        return self._samples is not None

    def frequencies(self, binary: bool = True, registers: bool = False):
        if self._frequencies is None:
            if self._samples is None:
                self._frequencies = self.backend.sample_frequencies(self._probs, self.nshots)
            else:
                dec = self.samples(binary=False)
                vals, cnts = np.unique(np.asarray(dec), return_counts=True)
                self._frequencies = collections.Counter(dict(zip(vals.tolist(), cnts.tolist())))
        if registers:
            out = {}
            for gate in self.measurements:
                idx = [self.measured_qubits.index(q) for q in gate.target_qubits]
                c = collections.Counter()
                n = len(self.measured_qubits)
                for k, v in self._frequencies.items():
                    bits = f"{k:b}".zfill(n)
                    sub = "".join(bits[i] for i in idx)
                    c[sub if binary else int(sub, 2)] += v
                out[gate.register_name or f"register{len(out)}"] = c
            return out
        if binary:
            return frequencies_to_binary(self._frequencies, len(self.measured_qubits))
        return self._frequencies

    def samples(self, binary: bool = True, registers: bool = False):
        if self._samples is None:
            dec = self.backend.sample_shots(self._probs, self.nshots)
            self._samples = self.backend.samples_to_binary(np.asarray(dec), len(self.measured_qubits))
        if binary:
            return self._samples
        n = len(self.measured_qubits)
        return (np.asarray(self._samples) @ (2 ** np.arange(n - 1, -1, -1))).astype(np.int64)


class MeasurementOutcomes(CircuitResult):
    """Measurement outcomes without a final state (result.py:166-548): what
    repeated execution returns, with one sample per shot.  Probabilities are
    the observed frequencies over the shots (result.py:211-230)."""

    def __init__(self, measurements, backend=None, samples=None, nshots=1000):
        from . import get_backend

        self.backend = backend or get_backend()
        self.measurements = measurements
        self.nshots = nshots
        self.measured_qubits = tuple(q for m in measurements for q in m.target_qubits)
        self.density_matrix = False
        self.nqubits = None
        self._state = None
        self._probs = None
        self._samples = None if samples is None else np.asarray(samples)
        self._frequencies = None
        if self._samples is not None:
            for m in measurements:
                idx = [self.measured_qubits.index(q) for q in m.target_qubits]
                if hasattr(m, "result"):
                    m.result.register_samples(self._samples[:, idx])

    def state(self, numpy: bool = False):
        raise RuntimeError("repeated execution keeps no final state: use samples or frequencies")

    def probabilities(self, qubits=None):
        n = len(self.measured_qubits)
        qubits = self.measured_qubits if qubits is None else tuple(qubits)
        idx = [self.measured_qubits.index(q) for q in qubits]
        p = np.zeros(2 ** len(idx))
        for k, v in self.frequencies(binary=False).items():
            bits = [(k >> (n - 1 - i)) & 1 for i in idx]
            p[int("".join(map(str, bits)) or "0", 2)] += v
        return p / self.nshots

    def __str__(self):
        return f"MeasurementOutcomes(nshots={self.nshots}, qubits={self.measured_qubits})"
