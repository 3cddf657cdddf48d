"""Pin the CPU oracle against golden vectors produced by the reference itself
and against the reference tests' own known-answer values.  CPU only."""

import json
import math
import os

import numpy as np
import pytest

from oracle import numpy_ref as ref

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gold():
    data = np.load(os.path.join(GOLD, "reference_vectors.npz"))
    with open(os.path.join(GOLD, "reference_vectors.json")) as f:
        meta = json.load(f)
    return data, meta


def test_oracle_gate_catalogue(gold):
    data, meta = gold
    psi0 = data["gates_init"]
    for i, g in enumerate(meta["gates"]):
        m = ref.gate_matrix(g["name"], g["params"])
        np.testing.assert_allclose(m, data[f"gate_{i}_matrix"], atol=1e-15, err_msg=g["name"])
        out = ref.apply_gate(psi0, m, g["gate_qubits"], 4)
        np.testing.assert_allclose(out, data[f"gate_{i}"], atol=1e-14, err_msg=str(g))


def test_oracle_controlled_by(gold):
    data, meta = gold
    psi0 = data["gates_init"]
    for i, g in enumerate(meta["controlled_by"]):
        out = ref.execute([(g["name"], g["targets"], g["params"], g["controls"])], 4, psi0)
        np.testing.assert_allclose(out, data[f"ctrl_{i}"], atol=1e-14, err_msg=str(g))


@pytest.mark.parametrize("n", [4, 5, 6, 10])
def test_oracle_qft(gold, n):
    data, _ = gold
    out = ref.execute(ref.qft_ops(n), n, data[f"qft{n}_init"])
    np.testing.assert_allclose(out, data[f"qft{n}_final"], atol=1e-13)


def test_oracle_qft_is_dft():
    """QFT equals the exact DFT matrix (reference tests/test_models_qft.py:11-77)."""
    n = 5
    rng = np.random.default_rng(5)
    s = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    s /= np.linalg.norm(s)
    k = np.arange(2**n)
    dft = np.exp(2j * np.pi * np.outer(k, k) / 2**n) / np.sqrt(2**n)
    np.testing.assert_allclose(ref.execute(ref.qft_ops(n), n, s), dft @ s, atol=1e-12)


def test_oracle_brickwork(gold):
    data, _ = gold
    ang = data["brick8_angles"]
    ops = []
    for l in range(ang.shape[0]):
        for q in range(8):
            ops.append(("U3", (q,), tuple(ang[l, q])))
        for q in range(l % 2, 7, 2):
            ops.append(("CZ", (q, q + 1), ()))
    np.testing.assert_allclose(ref.execute(ops, 8), data["brick8_c128"], atol=1e-13)
    np.testing.assert_allclose(ref.execute(ops, 8, dtype="complex64"), data["brick8_c64"], atol=2e-6)
    # brickwork_ops with the same seed reproduces the golden angles
    np.testing.assert_allclose(ref.execute(ref.brickwork_ops(8, 6, 30), 8), data["brick8_c128"], atol=1e-13)


def test_oracle_matrix_fused():
    rng = np.random.default_rng(3)
    ops = ref.brickwork_ops(3, 2, 7)
    mats = [((q), ref.gate_matrix(nm, p)) for nm, q, p in ops]
    fused = ref.matrix_fused([0, 1, 2], mats)
    s = rng.normal(size=8) + 1j * rng.normal(size=8)
    np.testing.assert_allclose(fused @ s, ref.execute(ops, 3, s), atol=1e-13)


def test_oracle_probabilities(gold):
    data, meta = gold
    st = data["brick8_c128"]
    for i, qs in enumerate(meta["prob_sets"]):
        np.testing.assert_allclose(ref.calculate_probabilities(st, qs, 8), data[f"probs_{i}"], atol=1e-15)


def test_oracle_frequencies_seeded(gold):
    """The reference's seeded counts (legacy MT19937 after set_seed(1234))."""
    data, _ = gold
    np.random.seed(1234)
    f = ref.sample_frequencies(data["freq3_probs"], 100000)
    counts = np.array([f.get(i, 0) for i in range(8)])
    np.testing.assert_array_equal(counts, data["freq3_counts"])


def test_oracle_reference_test_frequencies():
    """Golden counts of tests/test_measurements_probabilistic.py:29-31 (numpy platform):
    4 equal outcomes, 1000 shots, seed 1234 -> {0:249, 1:231, 2:253, 3:267}."""
    np.random.seed(1234)
    f = ref.sample_frequencies(np.full(4, 0.25), 1000)
    assert dict(f) == {0: 249, 1: 231, 2: 253, 3: 267}


@pytest.mark.parametrize("n", [6, 8])
def test_oracle_tfim(gold, n):
    data, _ = gold
    t, q, c = ref.tfim_terms(n)
    e = ref.exp_value_observable_symbolic(data[f"tfim{n}_state"], t, q, c, n)
    np.testing.assert_allclose(e, data[f"tfim{n}_energy"], atol=1e-12)


def test_oracle_vqe_energy_and_psr(gold):
    data, _ = gold
    p = data["vqe4_params"]
    t, q, c = ref.tfim_terms(4)
    e = ref.exp_value_observable_symbolic(ref.execute(ref.vqe_ops(4, 2, p), 4), t, q, c, 4)
    np.testing.assert_allclose(e, data["vqe4_energy"], atol=1e-12)
    g = ref.parameter_shift_grad(lambda x: ref.vqe_ops(4, 2, x), 4, p, t, q, c)
    np.testing.assert_allclose(g, data["vqe4_psr_grads"], atol=1e-12)


@pytest.mark.parametrize("scale, kat", [(1.0, [-8.51104358e-02, -5.20075970e-01, 0.0]),
                                         (0.5, [-0.02405061, -0.13560379, 0.0])])
def test_oracle_reference_derivative_kat(scale, kat):
    """KAT of tests/test_derivative.py:28-31: RX(0), RY(0), RZ(0) with
    params linspace(0.1, 1, 3) * scale, observable Z0, exact parameter shift."""
    p = np.linspace(0.1, 1, 3) * scale

    def build(x):
        return [("RX", (0,), (x[0],)), ("RY", (0,), (x[1],)), ("RZ", (0,), (x[2],))]

    g = ref.parameter_shift_grad(build, 1, p, ["Z"], [(0,)], [1.0], scale_factor=scale)
    np.testing.assert_allclose(g, kat, atol=1e-8)


def test_oracle_collapse(gold):
    """Backend.collapse_state (backends/abstract.py:3279-3304) against the
    reference's own outputs, with and without normalisation."""
    data, meta = gold
    st = data["brick8_c128"]
    for i, (qs, k) in enumerate(meta["collapse_cases"]):
        np.testing.assert_allclose(ref.collapse_statevector(st, qs, k, 8), data[f"collapse_{i}"], atol=1e-15)
        np.testing.assert_allclose(ref.collapse_statevector(st, qs, k, 8, normalize=False),
                                   data[f"collapse_{i}_unnorm"], atol=1e-15)


def test_oracle_expectation_from_frequencies(gold):
    """exp_value_diagonal_observable_symbolic_from_samples (:2873-2926) on the
    reference's frequency table."""
    data, meta = gold
    fs = meta["fromsamples"]
    got = ref.exp_value_from_frequencies(fs["freq"], fs["terms_qubits"], fs["coefs"], fs["qubit_map"], fs["constant"])
    assert abs(got - float(data["fromsamples_value"])) < 1e-15


class _Recorded:
    """A gate or channel constructor call, recorded for the oracle."""

    def __init__(self, name, args):
        self.name, self.args, self.controls = name, args, ()

    def controlled_by(self, *q):
        self.controls = tuple(q)
        return self


class _RecordingGates:
    def __getattr__(self, name):
        return lambda *args: _Recorded(name, args)


class _RecordingCircuit:
    def __init__(self, nqubits, density_matrix=False):
        self.nqubits, self.queue = nqubits, []

    def add(self, op):
        self.queue.append(op)

    def ops(self):
        return [(op.name, op.args, op.controls) for op in self.queue]


def _density_cases():
    import sys

    sys.path.insert(0, GOLD)
    import density_cases

    return density_cases


@pytest.mark.parametrize("name", ["dm_noisy4", "dm_noisy6", "dm_layers8"])
def test_oracle_density_circuits(gold, name):
    """The oracle's density-matrix restatement (gates, every channel kind,
    diagonal probabilities, Pauli-sum energy, collapse) against the
    reference's own outputs for the circuits of tests/golden/density_cases.py."""
    data, meta = gold
    dc = _density_cases()
    n, build, seed = dc.CASES[name]
    c = build(_RecordingGates(), _RecordingCircuit)
    rho0 = data[f"{name}_init"] if seed is not None else None
    rho = ref.execute_density(c.ops(), n, rho0)
    if name in dc.SAMPLED:
        np.testing.assert_allclose(rho.ravel()[data[f"{name}_idx"]], data[f"{name}_vals"], atol=1e-13)
    else:
        np.testing.assert_allclose(rho, data[f"{name}_final"], atol=1e-13)
        np.testing.assert_allclose(ref.collapse_density(rho, [1], 1, n), data[f"{name}_collapse"], atol=1e-13)
    for i, qs in enumerate(dc.PROB_SETS[name]):
        np.testing.assert_allclose(ref.calculate_probabilities_density(rho, qs, n), data[f"{name}_probs_{i}"],
                                   atol=1e-13)
    terms, tq, cf = ref.tfim_terms(n, 0.5)
    assert abs(ref.exp_value_observable_symbolic_density(rho, terms, tq, cf, n) - float(data[f"{name}_tfim"])) < 1e-12
    assert abs(np.real(np.trace(rho @ rho)) - float(data[f"{name}_purity"])) < 1e-12
