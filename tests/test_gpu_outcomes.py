"""Measurement outcomes on the GPU: state collapse, expectation values from
shots, and repeated execution of circuits with collapsing measurements.

Tolerances: collapsed states 1e-12 max-abs (complex128) / 1e-6 (complex64)
against the reference's own outputs (tests/golden); parity counts exact;
expectations from shots within 5 sum|c| / sqrt(nshots) of the exact value,
and to 1e-12 of the reference's frequency formula applied to the same
shots; outcome histograms of repeated execution pass a chi-square test
(p > 1e-4) against the exact distribution from the oracle."""

import json
import os

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gold():
    data = np.load(os.path.join(GOLD, "reference_vectors.npz"))
    with open(os.path.join(GOLD, "reference_vectors.json")) as f:
        meta = json.load(f)
    return data, meta


def _chi2_ok(counts, probs, nshots):
    from scipy.stats import chi2

    exp = np.asarray(probs) * nshots
    m = exp > 5
    stat = np.sum((np.asarray(counts)[m] - exp[m]) ** 2 / exp[m])
    return chi2.sf(stat, max(1, m.sum() - 1)) > 1e-4


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-6)])
def test_collapse_matches_reference(gold, dtype, tol):
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    data, meta = gold
    b = GB300Backend(dtype)
    st = data["brick8_c128"]
    for i, (qs, k) in enumerate(meta["collapse_cases"]):
        for normalize, key in ((True, f"collapse_{i}"), (False, f"collapse_{i}_unnorm")):
            dev = DeviceState.from_numpy(st.astype(dtype), dtype)
            out = b.collapse_state(dev, qs, np.array([k]), 8, normalize=normalize)
            assert np.max(np.abs(np.asarray(out) - data[key])) < tol, (i, normalize)


def test_collapse_rejects_bad_arguments():
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    b = GB300Backend("complex128")
    st = DeviceState.zero(4, "complex128")
    with pytest.raises(ValueError):
        b.collapse_state(st, [1, 2], np.array([4]), 4)  # outcome beyond 2 qubits
    with pytest.raises(ValueError):
        b.collapse_state(st, [1, 1], np.array([0]), 4)  # repeated qubit


def test_parity_counts_exact():
    from qibo_gb300.device import DeviceArray, Runtime
    from qibo_gb300.engine import Engine

    rt = Runtime.get()
    eng = Engine(rt)
    rng = np.random.default_rng(5)
    all_masks = [0, 1, 3, 0x80001, 0xFFFFF] + [int(m) for m in rng.integers(1, 2**20, 300)]
    for nshots, masks in ((1, all_masks), (31, all_masks), (1000, all_masks), (300_001, all_masks[:12])):
        s = rng.integers(0, 2**20, nshots, dtype=np.int64)
        dev = DeviceArray((nshots,), np.int64, rt)
        rt.h2d(dev.ptr, s)
        got = eng.parity_means(dev, nshots, masks)  # 305 masks: two launches of at most 256
        odd = np.zeros(len(masks), dtype=np.int64)
        for j, m in enumerate(masks):
            v = s & m
            pc = np.zeros(nshots, dtype=np.int64)
            for bit in range(20):
                pc += (v >> bit) & 1
            odd[j] = int((pc & 1).sum())
        np.testing.assert_array_equal(got, (nshots - 2 * odd) / nshots)


def _random_circuit(n, depth, seed):
    from qibo_gb300 import Circuit, gates

    ops = ref.brickwork_ops(n, depth, seed)
    c = Circuit(n)
    for name, qs, params in ops:
        c.add(getattr(gates, name)(*qs, *params))
    return c, ops


def _tfim_groups(n, h=0.7):
    """TFIM terms in the two groups measured together: the Z Z couplings
    and the X fields (hamiltonians/models.py:587-662)."""
    zz = ([-1.0] * n, ["ZZ"] * n, [(i, (i + 1) % n) for i in range(n)])
    xx = ([-h] * n, ["X"] * n, [(i,) for i in range(n)])
    return [zz, xx]


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_expectation_from_samples_statistics(dtype):
    from qibo_gb300.backend import GB300Backend

    n, nshots = 8, 400_000
    b = GB300Backend(dtype)
    b.set_seed(11)
    c, ops = _random_circuit(n, 4, 3)
    groups = _tfim_groups(n)
    got = b.exp_value_observable_symbolic_from_samples(c, [g[0] for g in groups], [g[1] for g in groups],
                                                       [g[2] for g in groups], n, 0.25, nshots)
    st = ref.execute(ops, n)
    exact = 0.25
    for coefs, obs, qubits in groups:
        exact += ref.exp_value_observable_symbolic(st, obs, qubits, coefs, n)
    bound = 5 * sum(abs(x) for g in groups for x in g[0]) / np.sqrt(nshots)
    assert abs(got - exact) < bound, (got, exact, bound)
    assert c._final_state is None  # the caller's circuit is left unexecuted, as in the reference


def test_expectation_from_samples_equals_reference_formula():
    """The device parity counts give exactly the reference's frequency-weighted
    sum (backends/abstract.py:2873-2926) on the same shots."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    n, nshots = 6, 50_000
    b = GB300Backend("complex128")
    c, ops = _random_circuit(n, 3, 8)
    st = DeviceState.from_numpy(ref.execute(ops, n), "complex128")
    qmap = [4, 0, 2, 5]
    terms = [(4,), (0, 2), (5, 4, 0), (2, 5)]
    coefs = [0.5, -1.5, 0.25, 2.0]
    probs = b.engine_gb.probabilities(st, qmap)
    samples = b.engine_gb.sample_device(probs, nshots, 99)
    masks = [sum(1 << (len(qmap) - 1 - qmap.index(q)) for q in t) for t in terms]
    got = float(np.dot(coefs, b.engine_gb.parity_means(samples, nshots, masks)))
    s = samples.to_numpy()
    keys, cnt = np.unique(s, return_counts=True)
    freq = {f"{int(k):0{len(qmap)}b}": int(v) for k, v in zip(keys, cnt)}
    assert abs(got - ref.exp_value_from_frequencies(freq, terms, coefs, qmap)) < 1e-12


def test_repeated_execution_bell_collapse():
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend

    for dtype in ("complex128", "complex64"):
        b = GB300Backend(dtype)
        b.set_seed(3)
        c = Circuit(2)
        c.add(gates.H(0)); c.add(gates.CNOT(0, 1))
        c.add(gates.M(0, collapse=True))
        c.add(gates.M(0, 1))
        res = b.execute_circuit(c, nshots=1000)
        s = res.samples()
        assert s.shape == (1000, 2) and np.all(s[:, 0] == s[:, 1])
        col = c.queue[2].result.samples()
        np.testing.assert_array_equal(col[:, 0], s[:, 0])  # the collapse decided the later measurement
        f = res.frequencies(binary=True)
        assert set(f) <= {"00", "11"} and _chi2_ok([f.get("00", 0), f.get("11", 0)], [0.5, 0.5], 1000)
        with pytest.raises(RuntimeError):
            res.state()


def test_repeated_execution_distribution_vs_oracle():
    """A 4-qubit circuit measured mid-way on qubits 1 and 3: the histogram of
    the final measurement matches the exact mixture over the mid-circuit
    outcomes (oracle: collapse each branch, continue, weight by its
    probability); the run is reproducible for a fixed seed."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend

    n, nshots = 4, 4000
    pre = ref.brickwork_ops(n, 2, 21)
    post = ref.brickwork_ops(n, 2, 22)
    mq, fq = [1, 3], [0, 1, 2, 3]
    psi = ref.execute(pre, n)
    pk = ref.calculate_probabilities(psi, mq, n)
    dist = np.zeros(2**n)
    for k, p in enumerate(pk):
        if p < 1e-15:
            continue
        branch = ref.execute(post, n, initial_state=ref.collapse_statevector(psi, mq, k, n))
        dist += p * ref.calculate_probabilities(branch, fq, n)

    def build():
        c = Circuit(n)
        for name, qs, params in pre:
            c.add(getattr(gates, name)(*qs, *params))
        c.add(gates.M(*mq, collapse=True))
        for name, qs, params in post:
            c.add(getattr(gates, name)(*qs, *params))
        c.add(gates.M(*fq))
        return c

    b = GB300Backend("complex128")
    b.set_seed(17)
    r1 = b.execute_circuit(build(), nshots=nshots)
    counts = np.bincount(r1.samples(binary=False), minlength=2**n)
    assert _chi2_ok(counts, dist, nshots)
    b.set_seed(17)
    r2 = b.execute_circuit(build(), nshots=nshots)
    np.testing.assert_array_equal(r1.samples(), r2.samples())


def test_measurement_then_gate_collapses():
    """models/circuit.py:684-689: M(0) followed by a gate on qubit 0 becomes a
    collapsing measurement; H then M(0, collapse) then H gives 0 or 1 with
    probability 1/2 each, and the final measurement is again 1/2."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend

    b = GB300Backend("complex128")
    b.set_seed(5)
    c = Circuit(1)
    c.add(gates.H(0))
    m = gates.M(0)
    c.add(m)
    c.add(gates.H(0))
    c.add(gates.M(0))
    assert m.collapse and c.repeated_execution
    res = b.execute_circuit(c, nshots=2000)
    s = res.samples(binary=False)
    assert _chi2_ok(np.bincount(s, minlength=2), [0.5, 0.5], 2000)
    mid = m.result.samples(binary=False)
    assert _chi2_ok(np.bincount(mid, minlength=2), [0.5, 0.5], 2000)
