"""Density matrices on the GB300 against the reference's own outputs.

The circuits of tests/golden/density_cases.py (gates with controls,
every channel kind, 3-qubit channels run as weighted sums, both thermal-
relaxation branches) are built with qibo_gb300's gates and run on the
device; final density matrices, diagonal probabilities, Pauli-sum energies,
collapses and purities are compared with the fixtures that
tests/golden/make_golden.py wrote by running the reference NumpyBackend.
Tolerances: 1e-12 max-abs in complex128, 1e-5 in complex64.  At 15 and 16
qubits (30- and 32-qubit vectors, 17 and 34 GB) the check is a closed form:
single-qubit gates and channels on a product state give the product of the
single-qubit density matrices, and a CZ/U3 brickwork followed by its
inverse returns it.
"""

from __future__ import annotations

import gc
import json
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = {"complex128": 1e-12, "complex64": 1e-5}


@pytest.fixture(scope="module")
def gold():
    data = np.load(os.path.join(GOLD, "reference_vectors.npz"))
    with open(os.path.join(GOLD, "reference_vectors.json")) as f:
        meta = json.load(f)
    sys.path.insert(0, GOLD)
    import density_cases

    return data, meta, density_cases


def _backend(dtype="complex128", fuse=True, blocked=True):
    from qibo_gb300.backend import GB300Backend

    b = GB300Backend(dtype)
    b.fuse, b.blocked = fuse, blocked
    return b


def _run_case(gold, name, dtype="complex128", fuse=True, blocked=True):
    from qibo_gb300 import Circuit, gates

    data, meta, dc = gold
    n, build, seed = dc.CASES[name]
    b = _backend(dtype, fuse, blocked)
    c = build(gates, Circuit)
    init = None if seed is None else data[f"{name}_init"].copy()
    res = b.execute_circuit(c, initial_state=init)
    return b, c, res, n


@pytest.mark.parametrize("name", ["dm_noisy4", "dm_noisy6", "dm_layers8"])
@pytest.mark.parametrize("fuse,blocked", [(True, True), (False, True), (False, False)])
def test_density_circuit_matches_reference(gold, name, fuse, blocked):
    from oracle import numpy_ref as ref

    data, meta, dc = gold
    b, c, res, n = _run_case(gold, name, fuse=fuse, blocked=blocked)
    assert res.density_matrix
    rho = res.state()
    if name in dc.SAMPLED:
        got = rho.take(data[f"{name}_idx"])
        np.testing.assert_allclose(got, data[f"{name}_vals"], atol=TOL["complex128"])
    else:
        np.testing.assert_allclose(np.asarray(rho), data[f"{name}_final"], atol=TOL["complex128"])
    for i, qs in enumerate(dc.PROB_SETS[name]):
        np.testing.assert_allclose(np.asarray(res.probabilities(qs)), data[f"{name}_probs_{i}"], atol=1e-13)
    terms, tq, cf = ref.tfim_terms(n, 0.5)
    e = b.exp_value_observable_symbolic(c, terms, tq, cf, n)
    assert abs(e - float(data[f"{name}_tfim"])) < TOL["complex128"]
    # trace and purity from device reads
    assert abs(b.engine_gb.density_trace(rho) - 1.0) < 1e-12
    if name not in dc.SAMPLED:
        full = np.asarray(rho)
        assert abs(np.real(np.trace(full @ full)) - float(data[f"{name}_purity"])) < 1e-12
        got = b.collapse_state(rho, [1], np.array([1]), n, density_matrix=True)
        np.testing.assert_allclose(np.asarray(got), data[f"{name}_collapse"], atol=TOL["complex128"])


def test_density_complex64(gold):
    """complex64 of the 8-qubit noisy brickwork (tensor-core blocks on the
    16-qubit vector) against the complex128 reference output."""
    data, meta, dc = gold
    b, c, res, n = _run_case(gold, "dm_layers8", dtype="complex64")
    got = res.state().take(data["dm_layers8_idx"])
    np.testing.assert_allclose(got, data["dm_layers8_vals"], atol=TOL["complex64"])
    for i, qs in enumerate(dc.PROB_SETS["dm_layers8"]):
        np.testing.assert_allclose(np.asarray(res.probabilities(qs)), data[f"dm_layers8_probs_{i}"], atol=1e-5)


def test_dense_expectation_on_density(gold):
    from oracle import numpy_ref as ref

    data, meta, dc = gold
    b, c, res, n = _run_case(gold, "dm_noisy4")
    rng = np.random.default_rng(4)
    h = rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))
    h = h + h.conj().T
    want = ref.expectation_value_density(h, data["dm_noisy4_final"], True)
    assert abs(b.expectation_value(h, res.state(), True) - want) < 1e-12


def test_collapsing_measurement_mean_state():
    """A collapsing measurement on a density circuit: the mean of the shots'
    states is diagonal after H + collapse (coherence removed exactly) with
    weights within 5 sigma of 1/2, and the CNOT copy agrees."""
    from qibo_gb300 import Circuit, gates

    b = _backend()
    c = Circuit(2, density_matrix=True)
    c.add(gates.H(0))
    c.add(gates.M(0, collapse=True))
    c.add(gates.CNOT(0, 1))
    c.add(gates.M(0, 1))
    b.set_seed(77)
    nshots = 400
    res = b.execute_circuit(c, nshots=nshots)
    rho = np.asarray(res.state())
    assert abs(np.trace(rho) - 1) < 1e-12
    assert np.max(np.abs(rho - np.diag(np.diag(rho)))) < 1e-15
    assert abs(rho[0, 0].real - 0.5) < 5 * 0.5 / np.sqrt(nshots)
    freqs = res.frequencies()
    assert sum(freqs.values()) == nshots and set(freqs) <= {"00", "11"}


def test_noisy_state_vector_frequencies():
    """A Pauli channel in a state-vector circuit runs shot by shot with one
    drawn gate per shot: the flip frequency follows the channel's probability."""
    from qibo_gb300 import Circuit, gates

    b = _backend()
    c = Circuit(3)
    c.add(gates.H(1))
    c.add(gates.PauliNoiseChannel(0, [("X", 0.3)]))
    c.add(gates.DepolarizingChannel((2,), 0.4))
    c.add(gates.M(0, 1, 2))
    b.set_seed(5)
    nshots = 4000
    freqs = b.execute_circuit(c, nshots=nshots).frequencies()
    assert sum(freqs.values()) == nshots
    p0 = sum(v for k, v in freqs.items() if k[0] == "1") / nshots
    p2 = sum(v for k, v in freqs.items() if k[2] == "1") / nshots
    assert abs(p0 - 0.3) < 5 * np.sqrt(0.21 / nshots)
    assert abs(p2 - 0.2) < 5 * np.sqrt(0.16 / nshots)  # X or Y of the depolarizing flips: 2 x 0.4 / 4


def _single_qubit_rhos(n, seed):
    """rho_q of qubit q after U3 and single-qubit channels, on the host."""
    from oracle import numpy_ref as ref

    ang = np.random.default_rng(seed).uniform(0, 2 * np.pi, (n, 3))
    out = []
    for q in range(n):
        r = np.zeros((2, 2), dtype=np.complex128)
        r[0, 0] = 1
        r = ref.apply_gate_density(r, ref.gate_matrix("U3", ang[q]), [0], 1)
        r = ref.depolarizing_density(r, [0], 0.05 + 0.01 * (q % 4), 1)
        g = 0.1 + 0.02 * (q % 5)
        ks = [((0,), np.array([[1, 0], [0, np.sqrt(1 - g)]])), ((0,), np.array([[0, np.sqrt(g)], [0, 0]]))]
        r = ref.apply_channel_density(r, [1, 1], ks, 1, 1)
        out.append(r)
    return ang, out


def _product_entries(rhos, n, idx):
    i, j = idx // 2**n, idx % 2**n
    val = np.ones(idx.shape, dtype=np.complex128)
    for q in range(n):
        bi, bj = (i >> (n - 1 - q)) & 1, (j >> (n - 1 - q)) & 1
        val *= rhos[q][bi, bj]
    return val


@pytest.mark.parametrize("n,dtype", [(15, "complex128"), (16, "complex64")])
def test_large_product_density_and_brickwork_inverse(n, dtype):
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.device import Runtime

    free, _ = Runtime.get().mem_info()
    need = 4**n * (16 if dtype == "complex128" else 8)
    if free < need + (8 << 30):
        pytest.skip(f"needs {need / 1e9:.0f} GB of device memory")
    ang, rhos = _single_qubit_rhos(n, n)
    c = Circuit(n, density_matrix=True)
    for q in range(n):
        c.add(gates.U3(q, *ang[q]))
        c.add(gates.DepolarizingChannel((q,), 0.05 + 0.01 * (q % 4)))
        c.add(gates.AmplitudeDampingChannel(q, 0.1 + 0.02 * (q % 5)))
    rng = np.random.default_rng(3)
    bw = []
    for layer in range(2):
        bw += [gates.U3(q, *rng.uniform(0, 2 * np.pi, 3)) for q in range(n)]
        bw += [gates.CZ(q, q + 1) for q in range(layer % 2, n - 1, 2)]
    inv = []
    for g in reversed(bw):
        if type(g).__name__ == "U3":
            th, ph, la = g.parameters
            inv.append(gates.U3(g.target_qubits[0], -th, -la, -ph))
        else:
            inv.append(g)
    c.add(bw + inv)
    b = _backend(dtype)
    rho = b.execute_circuit(c).state()
    rng = np.random.default_rng(11)
    idx = np.unique(np.concatenate([rng.integers(0, 4**n, 4096), np.arange(0, 4**n, 2**n + 1)[:256]]))
    err = np.max(np.abs(rho.take(idx) - _product_entries(rhos, n, idx)))
    assert err < TOL[dtype], f"n={n} {dtype}: {err}"
    assert abs(b.engine_gb.density_trace(rho) - 1.0) < (1e-12 if dtype == "complex128" else 1e-5)
    del rho, b
    gc.collect()
