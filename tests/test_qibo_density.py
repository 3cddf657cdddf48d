"""Density matrices through qibo's own front end, on the CPU, against the
reference NumpyBackend run on the same circuits.

``qibo.set_backend("qibo_gb300")`` resolves to the plugin backend; the C-ABI
library is replaced by the host stand-in (tests/host_device.py), so the
package's density path -- gates as row/column pairs on the 2n-qubit vector,
channels as superoperators or weighted sums, diagonal probabilities, trace
collapses, Pauli traces -- is the code that ships, and its results are
compared with qibo's NumpyBackend (backends/abstract.py:2095-2361,
:2734-2748, :3199-3277) on the same circuits and inputs.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import import_reference
from oracle import numpy_ref as ref

TOL = 1e-12


@pytest.fixture
def qibo_pair(monkeypatch):
    qibo = import_reference()
    if qibo is None:
        pytest.skip("reference qibo not importable here")
    from host_device import HostLib
    from qibo.backends.numpy import NumpyBackend

    from qibo_gb300 import _lib
    from qibo_gb300.device import Runtime

    host = HostLib()
    monkeypatch.setattr(_lib, "_lib", host)
    monkeypatch.setattr(Runtime, "_instance", None)
    qibo.set_backend("qibo_gb300")
    backend = qibo.get_backend()
    try:
        yield qibo, backend, NumpyBackend(), host
    finally:
        qibo.set_backend("numpy")


def _random_rho(n, seed):
    rng = np.random.default_rng(seed)
    m = rng.normal(size=(2**n, 2**n)) + 1j * rng.normal(size=(2**n, 2**n))
    rho = m @ m.conj().T
    return rho / np.trace(rho)


def _unitary(d, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _noisy_circuit(qibo, n=4):
    """Gates (with controls and controlled_by) and every channel kind: one-
    and two-qubit superoperators, a 3-qubit Kraus and a 3-qubit unitary
    channel (weighted sums), both thermal-relaxation branches (T1 >= T2 on a
    qubit other than 0), readout error, reset."""
    g = qibo.gates
    c = qibo.Circuit(n, density_matrix=True)
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
    a = np.sqrt(0.6) * _unitary(2, 1)
    b = np.sqrt(0.4) * _unitary(4, 2)
    c.add(g.KrausChannel([(0,), (1, 3)], [a, b]))
    c.add(g.UnitaryChannel([(1, 2), (0,)], [(0.3, _unitary(4, 3)), (0.2, _unitary(2, 4))]))
    c.add(g.ReadoutErrorChannel(2, np.array([[0.9, 0.1], [0.25, 0.75]])))
    c.add(g.TOFFOLI(3, 1, 0))
    c.add(g.fSim(2, 0, 0.6, 0.25))
    c.add(g.DepolarizingChannel((0, 1, 2), 0.15))
    return c


def test_noisy_circuit_matches_reference(qibo_pair):
    qibo, backend, numpy_backend, host = qibo_pair
    n = 4
    rho0 = _random_rho(n, 5)
    mine = _noisy_circuit(qibo, n)(initial_state=rho0.copy())
    want = numpy_backend.execute_circuit(_noisy_circuit(qibo, n), initial_state=rho0.copy())
    got = np.asarray(mine.state())
    assert got.shape == (2**n, 2**n) and mine.density_matrix
    np.testing.assert_allclose(got, want.state(), atol=TOL)
    for qs in ([0, 1, 2, 3], [2, 0], [3], [1, 3, 0]):
        np.testing.assert_allclose(np.asarray(mine.probabilities(qs)), want.probabilities(qs), atol=TOL)
    assert host.calls["qgb_state_axpby"] > 0  # the 3-qubit channels ran as weighted sums
    assert host.calls["qgb_density_probabilities"] > 0


def test_zero_state_and_measured_frequencies(qibo_pair):
    qibo, backend, numpy_backend, host = qibo_pair
    g = qibo.gates
    c = qibo.Circuit(3, density_matrix=True)
    c.add(g.H(0))
    c.add(g.CNOT(0, 2))
    c.add(g.DepolarizingChannel((2,), 0.3))
    c.add(g.M(0, 2))
    res = c(nshots=2000)
    want = numpy_backend.execute_circuit(c, nshots=10)
    np.testing.assert_allclose(np.asarray(res.state()), want.state(), atol=TOL)
    np.testing.assert_allclose(np.asarray(res.probabilities()), want.probabilities(), atol=TOL)
    freqs = res.frequencies()
    assert sum(freqs.values()) == 2000 and set(freqs) <= {"00", "01", "10", "11"}
    p = want.probabilities([0, 2])
    for k, v in freqs.items():
        pk = p[int(k, 2)]
        assert abs(v / 2000 - pk) < 5 * np.sqrt(pk * (1 - pk) / 2000) + 1e-9


def test_direct_gate_and_channel_application(qibo_pair):
    """gate.apply / channel.apply on a backend density matrix, as qibo code
    calls them (gates/channels.py:518-528, :678-707, :886-887)."""
    qibo, backend, numpy_backend, host = qibo_pair
    g = qibo.gates
    n = 3
    rho0 = _random_rho(n, 11)
    ops = [g.RX(1, 0.4), g.CNOT(2, 0), g.DepolarizingChannel((0, 2), 0.25), g.ResetChannel(1, [0.2, 0.3]),
           g.ThermalRelaxationChannel(2, [2.0, 1.0, 0.5, 0.1]), g.ThermalRelaxationChannel(0, [1.0, 1.8, 0.3]),
           g.AmplitudeDampingChannel(0, 0.2), g.Y(1).controlled_by(0)]
    want = rho0.copy()
    st = backend.cast(rho0.copy())
    for op in ops:
        want = op.apply(numpy_backend, want, n)
        st = op.apply(backend, st, n)
        np.testing.assert_allclose(np.asarray(backend.to_numpy(st)), want, atol=TOL, err_msg=str(op))


def test_symbolic_and_dense_expectations(qibo_pair):
    qibo, backend, numpy_backend, host = qibo_pair
    from qibo.hamiltonians import TFIM, SymbolicHamiltonian
    from qibo.symbols import X, Y, Z

    n = 4
    rho0 = _random_rho(n, 21)
    c = _noisy_circuit(qibo, n)
    ham = TFIM(n, h=0.7, dense=False)
    want_state = numpy_backend.execute_circuit(_noisy_circuit(qibo, n), initial_state=rho0.copy()).state()
    c(initial_state=rho0.copy())
    terms, tq, cf = ref.tfim_terms(n, 0.7)
    e = ham.expectation(c)
    assert abs(e - ref.exp_value_observable_symbolic_density(want_state, terms, tq, cf, n)) < TOL
    h2 = SymbolicHamiltonian(0.5 * X(0) * Y(2) - 1.25 * Z(1) * Z(3) + 0.3 * Y(1) + 0.2, nqubits=n)
    c2 = _noisy_circuit(qibo, n)
    c2(initial_state=rho0.copy())
    e2 = h2.expectation(c2)
    dense = h2.matrix
    assert abs(e2 - float(np.real(np.trace(np.asarray(dense) @ want_state)))) < TOL
    assert host.calls["qgb_density_expect_pauli"] >= 2
    # dense Hamiltonian on a density matrix: Re Tr(H rho)
    hd = TFIM(n, h=0.7, dense=True)
    st = backend.cast(want_state.copy())
    assert abs(hd.expectation(st) - ref.expectation_value_density(np.asarray(hd.matrix), want_state, False)) < TOL


def test_collapse_and_probabilities_match_reference(qibo_pair):
    qibo, backend, numpy_backend, host = qibo_pair
    n = 4
    rho = _random_rho(n, 31)
    for qs, k in (([2], 1), ([0, 3], 2), ([1, 2, 3], 5)):
        for normalize in (True, False):
            got = backend.collapse_state(backend.cast(rho.copy()), qs, np.array([k]), n, normalize=normalize,
                                         density_matrix=True)
            want = numpy_backend.collapse_state(rho.copy(), qs, np.array([k]), n, normalize=normalize,
                                                density_matrix=True)
            np.testing.assert_allclose(np.asarray(backend.to_numpy(got)), want, atol=TOL)
        p = backend.calculate_probabilities(backend.cast(rho.copy()), qs, n, density_matrix=True)
        np.testing.assert_allclose(np.asarray(backend.to_numpy(p)),
                                   numpy_backend.calculate_probabilities(rho, qs, n, density_matrix=True), atol=TOL)


def test_collapsing_measurement_in_density_circuit(qibo_pair):
    """A collapsing measurement makes the circuit run shot by shot; the
    result is the mean of the shots' density matrices (:2603-2625).  After
    H and a collapse of qubit 0 that mean is diagonal (coherence gone) with
    weights near 1/2; the qubit 1 CNOT copy agrees with qubit 0."""
    qibo, backend, numpy_backend, host = qibo_pair
    g = qibo.gates
    c = qibo.Circuit(2, density_matrix=True)
    c.add(g.H(0))
    c.add(g.M(0, collapse=True))
    c.add(g.CNOT(0, 1))
    c.add(g.M(0, 1))
    nshots = 400
    res = c(nshots=nshots)
    rho = np.asarray(res.state())
    assert abs(np.trace(rho) - 1) < 1e-12
    off = rho - np.diag(np.diag(rho))
    assert np.max(np.abs(off)) < 1e-15
    assert abs(rho[0, 0] - 0.5) < 5 * 0.5 / np.sqrt(nshots) and abs(rho[0, 0] + rho[3, 3] - 1) < 1e-12
    freqs = res.frequencies()
    assert sum(freqs.values()) == nshots and set(freqs) <= {"00", "11"}
    assert host.calls["qgb_density_collapse"] >= nshots


def test_noisy_state_vector_repeated_execution(qibo_pair):
    """A unitary channel in a state-vector circuit: one of its gates per
    shot (Backend.apply_channel, :2314-2318); outcome frequencies follow the
    density-matrix probabilities."""
    qibo, backend, numpy_backend, host = qibo_pair
    g = qibo.gates
    c = qibo.Circuit(2)
    c.add(g.H(1))
    c.add(g.PauliNoiseChannel(0, [("X", 0.3)]))
    c.add(g.M(0, 1))
    nshots = 3000
    res = c(nshots=nshots)
    freqs = res.frequencies()
    assert sum(freqs.values()) == nshots
    p1 = sum(v for k, v in freqs.items() if k[0] == "1") / nshots
    assert abs(p1 - 0.3) < 5 * np.sqrt(0.3 * 0.7 / nshots)
    # a Kraus channel cannot act on a state vector (gates/channels.py:33-41)
    c2 = qibo.Circuit(1)
    c2.add(g.AmplitudeDampingChannel(0, 0.3))
    with pytest.raises(NotImplementedError):
        c2()


def test_device_density_arithmetic(qibo_pair):
    qibo, backend, numpy_backend, host = qibo_pair
    a, b = _random_rho(2, 41), _random_rho(2, 42)
    da, db = backend.cast(a.copy()), backend.cast(b.copy())
    np.testing.assert_allclose(np.asarray(0.25 * da - db * 0.5 + da), 0.25 * a - 0.5 * b + a, atol=TOL)
    np.testing.assert_allclose(np.asarray(-da), -a, atol=TOL)
    np.testing.assert_allclose(np.asarray(da), a, atol=0)  # operands unchanged
