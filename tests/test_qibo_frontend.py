"""qibo's own front end through the plugin backend, on the CPU.

``qibo.set_backend("qibo_gb300")`` resolves to ``QiboGB300Backend``
(qibo_gb300/plugin.py), and qibo's ``Circuit``, ``CircuitResult`` /
``MeasurementOutcomes`` (result.py:207-282, :819-837), measurement gates
(gates/measurements.py:189-204) and ``SymbolicHamiltonian.expectation``
(hamiltonians/hamiltonians.py:586-627) drive it exactly as they drive the
reference NumpyBackend.  The only thing replaced is the C-ABI library: the
host stand-in in tests/host_device.py runs each ``qgb_*`` call on host memory
with the oracle's algorithms, so the package's Python layer (runtime, device
arrays, engine, backend) is the one that ships.  Results are compared with
the oracle, and each backend method the drop-in must serve is checked to be
reached through qibo's call path.
"""

from __future__ import annotations

import collections

import numpy as np
import pytest

from conftest import import_reference
from oracle import numpy_ref as ref

HOT_PATH = ("execute_circuit", "calculate_probabilities", "sample_frequencies", "sample_shots",
            "exp_value_observable_symbolic", "execute_circuit_repeated", "collapse_state",
            "exp_value_observable_symbolic_from_samples", "apply_gate", "matrix_fused")


@pytest.fixture
def qibo_gb300_backend(monkeypatch):
    qibo = import_reference()
    if qibo is None:
        pytest.skip("reference qibo not importable here")
    from host_device import HostLib

    from qibo_gb300 import _lib
    from qibo_gb300.device import Runtime
    from qibo_gb300.plugin import qibo_backend_class

    host = HostLib()
    monkeypatch.setattr(_lib, "_lib", host)
    monkeypatch.setattr(Runtime, "_instance", None)
    cls = qibo_backend_class()
    seen = collections.Counter()
    for name in HOT_PATH:
        meth = getattr(cls, name)

        def spy(self, *a, _m=meth, _n=name, **k):
            seen[_n] += 1
            return _m(self, *a, **k)

        monkeypatch.setattr(cls, name, spy)
    qibo.set_backend("qibo_gb300")
    backend = qibo.get_backend()
    try:
        yield qibo, backend, host, seen
    finally:
        qibo.set_backend("numpy")


def test_backend_is_the_plugin(qibo_gb300_backend):
    qibo, backend, host, _ = qibo_gb300_backend
    from qibo.backends.numpy import NumpyBackend

    assert type(backend).__name__ == "QiboGB300Backend" and isinstance(backend, NumpyBackend)
    assert backend.name == "qibo_gb300" and backend.dtype == "complex128"
    assert host.calls == {}  # nothing computed yet


def test_qft_circuit_result_frequencies_and_samples(qibo_gb300_backend):
    """models/qft.py QFT(5) plus a measurement of every qubit, called as
    ``circuit(nshots=...)``: qibo's CircuitResult takes the device state and
    the FP64 device probabilities; frequencies and samples have the
    reference's types and keys."""
    qibo, backend, host, seen = qibo_gb300_backend
    from qibo.result import CircuitResult

    n, nshots = 5, 300
    rng = np.random.default_rng(3)
    psi = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    psi /= np.linalg.norm(psi)
    c = qibo.models.QFT(n)
    c.add(qibo.gates.M(*range(n)))
    backend.set_seed(1234)
    res = c(initial_state=psi.copy(), nshots=nshots)
    assert isinstance(res, CircuitResult) and res.nshots == nshots
    want = ref.execute(ref.qft_ops(n), n, psi)
    np.testing.assert_allclose(np.asarray(res.state()), want, atol=1e-12)
    np.testing.assert_allclose(np.asarray(res.probabilities()), np.abs(want) ** 2, atol=1e-14)
    freqs = res.frequencies()
    assert isinstance(freqs, collections.Counter) and sum(freqs.values()) == nshots
    assert all(isinstance(k, str) and len(k) == n and set(k) <= {"0", "1"} for k in freqs)
    ifreqs = res.frequencies(binary=False)
    assert all(isinstance(k, int) and 0 <= k < 2**n for k in ifreqs) and sum(ifreqs.values()) == nshots
    # a fresh result draws samples (sample_shots) instead of frequencies
    res2 = c(initial_state=psi.copy(), nshots=nshots)
    samples = np.asarray(res2.samples())
    assert samples.shape == (nshots, n) and set(np.unique(samples)) <= {0, 1}
    dec = np.asarray(res2.samples(binary=False))
    assert dec.shape == (nshots,) and dec.min() >= 0 and dec.max() < 2**n
    for name in ("execute_circuit", "calculate_probabilities", "sample_frequencies", "sample_shots"):
        assert seen[name] > 0, name
    assert host.calls["qgb_apply_circuit"] > 0 and host.calls["qgb_sample"] > 0


def test_collapse_and_repeated_execution(qibo_gb300_backend):
    """A circuit with M(collapse=True) runs shot by shot
    (execute_circuit_repeated); qibo's MeasurementOutcomes takes the device
    outcomes.  qibo's own M.apply reaches calculate_probabilities,
    sample_shots and collapse_state."""
    qibo, backend, host, seen = qibo_gb300_backend
    from qibo.result import MeasurementOutcomes

    c = qibo.Circuit(3)
    c.add(qibo.gates.H(0))
    c.add(qibo.gates.M(0, collapse=True))
    c.add(qibo.gates.CNOT(0, 1))
    c.add(qibo.gates.H(2))
    c.add(qibo.gates.M(0, 1, 2))
    res = c(nshots=40)
    assert isinstance(res, MeasurementOutcomes)
    freqs = res.frequencies()
    assert sum(freqs.values()) == 40
    # qubits 0 and 1 always agree after the collapse and the CNOT
    assert all(k[0] == k[1] for k in freqs)
    assert seen["execute_circuit_repeated"] > 0 and host.calls["qgb_collapse"] > 0

    # qibo's measurement gate applied to a backend state (gates/measurements.py:189-204)
    state = backend.zero_state(2)
    state = backend.apply_gate(qibo.gates.H(0), state, 2)
    state = backend.apply_gate(qibo.gates.CNOT(0, 1), state, 2)
    m = qibo.gates.M(1, collapse=True)
    out = m.apply(backend, state, 2)
    v = np.asarray(backend.to_numpy(out))
    assert np.isclose(np.vdot(v, v).real, 1.0)
    assert np.isclose(abs(v[0]) + abs(v[3]), 1.0) and abs(v[1]) < 1e-15 and abs(v[2]) < 1e-15
    assert seen["collapse_state"] > 0 and seen["apply_gate"] > 0


def test_symbolic_hamiltonian_expectation(qibo_gb300_backend):
    """SymbolicHamiltonian.expectation(circuit) dispatches to
    exp_value_observable_symbolic; with nshots, to the from-samples form."""
    qibo, backend, host, seen = qibo_gb300_backend
    from qibo.hamiltonians import TFIM, SymbolicHamiltonian
    from qibo.symbols import X, Y, Z

    n = 4
    ops = ref.brickwork_ops(n, 3, 7)
    c = qibo.Circuit(n)
    for nm, q, p in ops:
        c.add(getattr(qibo.gates, nm)(*q, *p))
    psi = ref.execute(ops, n)
    ham = TFIM(n, h=0.7, dense=False)
    e = ham.expectation(c)
    terms, tq, cf = ref.tfim_terms(n, 0.7)
    assert abs(e - ref.exp_value_observable_symbolic(psi, terms, tq, cf, n)) < 1e-12
    h2 = SymbolicHamiltonian(0.5 * X(0) * Y(2) - 1.25 * Z(1) * Z(3) + 0.3, nqubits=n)
    e2 = h2.expectation(c.copy(deep=True))
    want2 = 0.3 + ref.exp_value_observable_symbolic(psi, ["XY", "ZZ"], [(0, 2), (1, 3)], [0.5, -1.25], n)
    assert abs(e2 - want2) < 1e-12
    assert seen["exp_value_observable_symbolic"] >= 2 and host.calls["qgb_expect_pauli"] >= 2
    # shot-based expectation: within a few standard errors of the exact value
    hz = SymbolicHamiltonian(Z(0) * Z(1) + 0.5 * Z(2), nqubits=n)
    exact = ref.exp_value_observable_symbolic(psi, ["ZZ", "Z"], [(0, 1), (2,)], [1.0, 0.5], n)
    est = hz.expectation(c.copy(deep=True), nshots=20000)
    assert abs(est - exact) < 0.05
    assert seen["exp_value_observable_symbolic_from_samples"] > 0 and host.calls["qgb_parity_counts"] > 0


def test_fused_circuit_runs(qibo_gb300_backend):
    """circuit.fuse() output (FusedGate, gates/special.py) is accepted: its
    matrix comes from the backend's matrix_fused."""
    qibo, backend, host, seen = qibo_gb300_backend
    n = 5
    ops = ref.brickwork_ops(n, 4, 11)
    c = qibo.Circuit(n)
    for nm, q, p in ops:
        c.add(getattr(qibo.gates, nm)(*q, *p))
    fused = c.fuse(max_qubits=3)
    assert any(type(g).__name__ == "FusedGate" for g in fused.queue)
    res = fused()
    np.testing.assert_allclose(np.asarray(res.state()), ref.execute(ops, n), atol=1e-12)
    assert seen["matrix_fused"] > 0


def test_every_hot_path_method_reached(qibo_gb300_backend):
    """All the scenarios above in one backend: every method of the drop-in
    hot path is reached through qibo's own call path."""
    qibo, backend, host, seen = qibo_gb300_backend
    from qibo.hamiltonians import SymbolicHamiltonian
    from qibo.symbols import Z

    c = qibo.models.QFT(3)
    c.add(qibo.gates.M(0, 1, 2))
    r = c(nshots=50)
    r.frequencies()
    c(nshots=50).samples()
    rc = qibo.Circuit(2)
    rc.add(qibo.gates.H(0))
    rc.add(qibo.gates.M(0, collapse=True))
    rc.add(qibo.gates.M(0, 1))
    rc(nshots=5).frequencies()
    st = backend.apply_gate(qibo.gates.H(0), backend.zero_state(1), 1)
    qibo.gates.M(0, collapse=True).apply(backend, st, 1)
    h = SymbolicHamiltonian(Z(0) * Z(1), nqubits=2)
    hc = qibo.Circuit(2)
    hc.add(qibo.gates.RX(0, 0.3))
    h.expectation(hc)
    h.expectation(hc.copy(deep=True), nshots=100)
    fc = qibo.Circuit(3)
    fc.add(qibo.gates.H(0))
    fc.add(qibo.gates.CNOT(0, 1))
    fc.add(qibo.gates.RY(2, 0.4))
    fc.fuse(max_qubits=2)()
    for name in HOT_PATH:
        assert seen[name] > 0, f"{name} not reached through qibo's call path"
