"""GPU parity: every kernel, through the C-ABI, against the reference's golden
vectors and the CPU oracle.

Tolerances: complex128 results match the reference to 1e-12 max-abs (the
drop-in bar for complex128; observed errors are ~1e-15); complex64 results to 1e-5
max-abs against the complex64 reference run; FP64 probabilities to 1e-14;
sampled histograms pass a chi-square test at p > 1e-4.
"""

import json
import math
import os

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
TOL128 = 1e-12
TOL64 = 1e-5


@pytest.fixture(scope="module")
def gold():
    data = np.load(os.path.join(GOLD, "reference_vectors.npz"))
    meta = json.load(open(os.path.join(GOLD, "reference_vectors.json")))
    return data, meta


@pytest.fixture(scope="module")
def backend():
    from qibo_gb300.backend import GB300Backend

    return GB300Backend("complex128")


def make_circuit(n, ops):
    from qibo_gb300 import Circuit, gates

    c = Circuit(n)
    for op in ops:
        g = getattr(gates, op[0])(*op[1], *op[2])
        if len(op) > 3 and op[3]:
            g = g.controlled_by(*op[3])
        c.add(g)
    return c


def run(backend, n, ops, psi=None, dtype="complex128", blocked=None, strict=False, fuse=True):
    backend.set_dtype(dtype)
    if blocked is not None:
        backend.blocked = blocked
    backend.strict_fp64 = strict
    backend.fuse = fuse
    try:
        res = backend.execute_circuit(make_circuit(n, ops), None if psi is None else psi.copy())
        return np.asarray(res.state())
    finally:
        backend.set_dtype("complex128")
        backend.blocked = True
        backend.strict_fp64 = False
        backend.fuse = True


def rand_state(n, seed, dtype=np.complex128):
    r = np.random.default_rng(seed)
    s = r.normal(size=2**n) + 1j * r.normal(size=2**n)
    return (s / np.linalg.norm(s)).astype(dtype)


# ---------------------------------------------------------------- gates --
def test_gate_catalogue_c128(backend, gold):
    data, meta = gold
    psi0 = data["gates_init"]
    for i, g in enumerate(meta["gates"]):
        out = run(backend, 4, [(g["name"], g["qubits"], g["params"])], psi0)
        assert np.max(np.abs(out - data[f"gate_{i}"])) < TOL128, g


def test_gate_catalogue_c64(backend, gold):
    data, meta = gold
    psi0 = data["gates_init"].astype(np.complex64)
    for i, g in enumerate(meta["gates"]):
        out = run(backend, 4, [(g["name"], g["qubits"], g["params"])], psi0, dtype="complex64")
        assert out.dtype == np.complex64
        assert np.max(np.abs(out - data[f"gate_{i}"])) < TOL64, g


def test_controlled_by_c128(backend, gold):
    data, meta = gold
    psi0 = data["gates_init"]
    for i, g in enumerate(meta["controlled_by"]):
        out = run(backend, 4, [(g["name"], g["targets"], g["params"], g["controls"])], psi0)
        assert np.max(np.abs(out - data[f"ctrl_{i}"])) < TOL128, g


@pytest.mark.parametrize("n", [5, 9, 12])
def test_every_position_every_kind(backend, n):
    """Each gate kind on many qubit placements (low bits exercise the
    warp-shuffle path, high bits the pair path), against the oracle."""
    rng = np.random.default_rng(n)
    names1 = ["H", "X", "Y", "Z", "S", "T", "RX", "RY", "RZ", "U1", "U2", "U3", "SX"]
    names2 = ["CNOT", "CZ", "CU1", "CU3", "SWAP", "iSWAP", "fSim", "RXX", "RZZ", "CRZ", "FSWAP"]
    nparams = {"RX": 1, "RY": 1, "RZ": 1, "U1": 1, "U2": 2, "U3": 3, "CU1": 1, "CU3": 3, "fSim": 2,
               "RXX": 1, "RZZ": 1, "CRZ": 1}
    ops = []
    for q in range(n):
        for nm in names1:
            ops.append((nm, (q,), tuple(rng.uniform(0, 2 * np.pi, nparams.get(nm, 0)))))
    for _ in range(4 * n):
        a, b = rng.choice(n, 2, replace=False)
        nm = names2[rng.integers(len(names2))]
        ops.append((nm, (int(a), int(b)), tuple(rng.uniform(0, 2 * np.pi, nparams.get(nm, 0)))))
    for _ in range(n):
        a, b, c = rng.choice(n, 3, replace=False)
        ops.append(("TOFFOLI", (int(a), int(b), int(c)), ()))
        ops.append(("U3", (int(c),), (0.3, 0.2, 0.1), (int(a), int(b))))
    psi = rand_state(n, 100 + n)
    want = ref.execute(ops, n, psi)
    # per-gate kernels (IEEE FP64), shared-memory passes in double-float, and
    # shared-memory passes in IEEE FP64
    for blocked, strict in ((False, False), (True, False), (True, True)):
        got = run(backend, n, ops, psi, blocked=blocked, strict=strict)
        assert np.max(np.abs(got - want)) < TOL128, (blocked, strict)
    want64 = ref.execute(ops, n, psi.astype(np.complex64), dtype="complex64")
    for blocked in (False, True):
        got = run(backend, n, ops, psi.astype(np.complex64), dtype="complex64", blocked=blocked)
        assert np.max(np.abs(got - want64)) < TOL64 * 10, blocked


@pytest.mark.parametrize("n", [16, 20])
def test_deep_random_circuit_c128_passes(backend, n):
    """890-gate-scale accuracy of the double-float passes (engine fusion off)
    and of the default engine-fused path: a depth-30 U3+CZ brickwork plus
    QFT against the FP64 oracle."""
    ops = ref.brickwork_ops(n, 30, 5) + ref.qft_ops(n)
    psi = rand_state(n, 77)
    want = ref.execute(ops, n, psi)
    got = run(backend, n, ops, psi, blocked=True, fuse=False)
    assert np.max(np.abs(got - want)) < TOL128
    # the default: engine fusion, 5-qubit blocks on the tensor cores
    got = run(backend, n, ops, psi, blocked=True, fuse=True)
    assert np.max(np.abs(got - want)) < TOL128


def test_direct_entry_points(backend):
    """qgb_apply_1q / _2q / _phase / _swap against the oracle."""
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceState

    rt = backend.rt
    n = 9
    psi = rand_state(n, 44)
    u1 = ref.gate_matrix("U3", (0.3, 1.2, -0.7))
    u2 = ref.gate_matrix("fSim", (0.4, 0.9))
    for dt in (np.complex128, np.complex64):
        st = DeviceState.from_numpy(psi.astype(dt))
        m1 = np.ascontiguousarray(u1).view(np.float64).ravel()
        m2 = np.ascontiguousarray(u2).view(np.float64).ravel()
        check(rt.lib.qgb_apply_1q(st.ptr, n, st.code, 6, m1.ctypes.data_as(_lib.dp), rt.stream))
        check(rt.lib.qgb_apply_2q(st.ptr, n, st.code, 7, 2, m2.ctypes.data_as(_lib.dp), rt.stream))
        check(rt.lib.qgb_apply_phase(st.ptr, n, st.code, _lib.int_array([1, 5]), 2, 0.6, -0.8, rt.stream))
        check(rt.lib.qgb_apply_swap(st.ptr, n, st.code, 0, 8, _lib.int_array([3]), 1, rt.stream))
        want = ref.apply_gate(psi.astype(dt).astype(np.complex128), u1, [6], n)
        want = ref.apply_gate(want, u2, [7, 2], n)
        ph = np.eye(4, dtype=complex)
        ph[3, 3] = 0.6 - 0.8j
        want = ref.apply_gate(want, ph, [1, 5], n)
        want = ref.apply_gate_controlled_by(want, ref.gate_matrix("SWAP"), (3,), (0, 8), n)
        tol = TOL128 if dt == np.complex128 else TOL64
        assert np.max(np.abs(np.asarray(st) - want)) < tol, dt
    with pytest.raises(ValueError):
        check(rt.lib.qgb_apply_phase(st.ptr, n, st.code, _lib.int_array([1, 1]), 2, 1.0, 0.0, rt.stream))
    with pytest.raises(ValueError):
        check(rt.lib.qgb_apply_swap(st.ptr, n, st.code, 0, 0, None, 0, rt.stream))


def test_unitary_gates_up_to_5_qubits(backend):
    from scipy.stats import unitary_group

    n = 9
    ops = []
    for k, qs in [(1, (4,)), (2, (8, 0)), (3, (2, 7, 5)), (4, (0, 3, 6, 8)), (5, (1, 8, 4, 2, 6))]:
        u = unitary_group.rvs(2**k, random_state=k)
        ops.append(("Unitary", qs, u))
    psi = rand_state(n, 5)
    want = psi.copy()
    for _, qs, u in ops:
        want = ref.apply_gate(want, u, list(qs), n)
    from qibo_gb300 import Circuit, gates

    c = Circuit(n)
    for _, qs, u in ops:
        c.add(gates.Unitary(u, *qs))
    got = np.asarray(backend.execute_circuit(c, psi.copy()).state())
    assert np.max(np.abs(got - want)) < TOL128


# ----------------------------------------------------------------- QFT --
@pytest.mark.parametrize("n", [4, 5, 6, 10])
def test_qft_golden(backend, gold, n):
    data, _ = gold
    got = run(backend, n, ref.qft_ops(n), data[f"qft{n}_init"])
    assert np.max(np.abs(got - data[f"qft{n}_final"])) < TOL128


def test_qft20_c128_matches_oracle(backend):
    """QFT(20) on a seeded complex Gaussian state: max-abs <= 1e-12."""
    n = 20
    psi = rand_state(n, 20)
    want = ref.execute(ref.qft_ops(n), n, psi)
    got = run(backend, n, ref.qft_ops(n), psi)
    assert np.max(np.abs(got - want)) < TOL128


# ----------------------------------------------------------- brickwork --
def test_brickwork_golden(backend, gold):
    data, _ = gold
    ops = ref.brickwork_ops(8, 6, 30)
    got = run(backend, 8, ops)
    assert np.max(np.abs(got - data["brick8_c128"])) < TOL128
    got64 = run(backend, 8, ops, dtype="complex64")
    assert np.max(np.abs(got64 - data["brick8_c64"])) < TOL64


def test_brickwork_fused_equals_unfused(backend):
    n = 14
    ops = ref.brickwork_ops(n, 10, 3)
    c = make_circuit(n, ops)
    want = ref.execute(ops, n)
    for maxq in (2, 3, 5):
        got = np.asarray(backend.execute_circuit(c.fuse(maxq)).state())
        assert np.max(np.abs(got - want)) < TOL128, maxq


# --------------------------------------------------------- measurement --
def test_probabilities_golden(backend, gold):
    data, meta = gold
    from qibo_gb300.device import DeviceState

    st = DeviceState.from_numpy(data["brick8_c128"])
    for i, qs in enumerate(meta["prob_sets"]):
        p = np.asarray(backend.calculate_probabilities(st, qs, 8))
        assert np.max(np.abs(p - data[f"probs_{i}"])) < 1e-14, qs


@pytest.mark.parametrize("n,qs", [(16, [3, 1]), (16, list(range(16))), (16, [15, 0, 7, 2, 9]),
                                  (18, list(range(0, 18, 2))), (14, [13]), (17, list(range(17))[::-1])])
def test_probabilities_vs_oracle(backend, n, qs):
    from qibo_gb300.device import DeviceState

    psi = rand_state(n, n)
    for dt in (np.complex128, np.complex64):
        st = DeviceState.from_numpy(psi.astype(dt))
        p = np.asarray(backend.calculate_probabilities(st, qs, n))
        want = ref.calculate_probabilities(psi.astype(dt).astype(np.complex128), qs, n)
        assert np.max(np.abs(p - want)) < 1e-14


def test_norm_is_fp64(backend):
    from qibo_gb300.device import DeviceState

    psi = rand_state(22, 1)
    st = DeviceState.from_numpy(psi)
    assert abs(backend.engine_gb.norm2(st) - 1.0) < 1e-13


def _wide_range_state(n, seed, dtype):
    """Amplitudes log-uniform over 1e-30..1 (floats: some subnormal), random
    signs, about 1/8 exact zeros: exercises every range branch of the
    reductions."""
    rng = np.random.default_rng(seed)
    mag = 10.0 ** rng.uniform(-30, 0, (2, 2**n))
    if dtype == np.complex64:
        mag[:, : 2**n // 64] *= 1e-12  # below the smallest normal float for some
    sgn = rng.choice([-1.0, 1.0], (2, 2**n))
    v = (sgn * mag)[0] + 1j * (sgn * mag)[1]
    v[rng.random(2**n) < 0.125] = 0
    return v.astype(dtype)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_reductions_fp64_accuracy(backend, dtype):
    """Norm and marginal probabilities (all qubits, a few qubits, one qubit)
    against sums in extended precision of the same stored values: relative
    error below 1e-13 (the complex64 partials are double-float, the complex128
    ones half FP64, half double-float)."""
    from qibo_gb300.device import DeviceState

    n = 22
    psi = _wide_range_state(n, 7, dtype)
    p_exact = (psi.real.astype(np.longdouble) ** 2 + psi.imag.astype(np.longdouble) ** 2)
    st = DeviceState.from_numpy(psi)
    nrm = backend.engine_gb.norm2(st)
    want = float(np.sum(p_exact))
    assert abs(nrm - want) <= 1e-13 * want
    for qs in ([0, 1, 2], [21], [5, 17, 0, 11, 3, 20, 8, 14, 2, 19], list(range(n))):
        got = np.asarray(backend.calculate_probabilities(st, qs, n))
        w = ref.order_probabilities(np.sum(p_exact.reshape((2,) * n),
                                           axis=tuple(q for q in range(n) if q not in qs)), qs, n).ravel()
        w = np.asarray(w, dtype=np.float64)
        assert np.all(np.abs(got - w) <= 1e-13 * np.maximum(w, 1e-300)), qs


def test_philox_known_answers():
    """Random123 known-answer vectors for philox4x32-10."""
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray, Runtime

    rt = Runtime.get()
    out = DeviceArray((4,), np.uint32, rt)
    cases = [((0, 0, 0, 0), (0, 0), [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD])]
    for ctr, key, want in cases:
        # qgb_philox_fill uses counter (t_lo, t_hi, c2, c3) with t = 0 only
        if ctr[0] or ctr[1]:
            continue
        check(rt.lib.qgb_philox_fill(out.ptr, 1, ctr[2], ctr[3], key[0], key[1], rt.stream))
        assert out.to_numpy().tolist() == want


def chi2_pvalue(counts, probs):
    from scipy.stats import chi2

    nshots = counts.sum()
    exp = probs * nshots
    mask = exp > 5
    stat = np.sum((counts[mask] - exp[mask]) ** 2 / exp[mask])
    rest_o, rest_e = counts[~mask].sum(), exp[~mask].sum()
    dof = mask.sum() - 1
    if rest_e > 0:
        stat += (rest_o - rest_e) ** 2 / rest_e
        dof += 1
    return chi2.sf(stat, dof)


def test_sampling_chi_square(backend):
    n = 10
    psi = rand_state(n, 3)
    probs = np.abs(psi) ** 2
    from qibo_gb300.device import DeviceState

    st = DeviceState.from_numpy(psi)
    dp = backend.calculate_probabilities(st, list(range(n)), n)
    backend.set_seed(1234)
    f = backend.sample_frequencies(dp, 1_000_000)
    counts = np.array([f.get(i, 0) for i in range(2**n)])
    assert counts.sum() == 1_000_000
    assert chi2_pvalue(counts, probs) > 1e-4
    s = backend.sample_shots(dp, 200_000)
    assert s.min() >= 0 and s.max() < 2**n
    assert chi2_pvalue(np.bincount(s, minlength=2**n), probs) > 1e-4


def test_sample_state_equals_probability_sampling(backend):
    """Shots drawn straight from the state (no 2^n probability vector) are the
    same draws as shots from the FP64 probability vector."""
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray, DeviceState

    rt = backend.rt
    for n, dt in ((18, np.complex128), (17, np.complex64)):
        st = DeviceState.from_numpy(rand_state(n, 31).astype(dt))
        probs = backend.engine_gb.probabilities(st, list(range(n)))
        a = DeviceArray((50000,), np.int64, rt)
        b = DeviceArray((50000,), np.int64, rt)
        check(rt.lib.qgb_sample(probs.ptr, n, 50000, 99, a.ptr, None, rt.scratch(rt.lib.qgb_sample_scratch_bytes(n)),
                                rt.stream))
        check(rt.lib.qgb_sample_state(st.ptr, n, st.code, 50000, 99, b.ptr,
                                      rt.scratch(rt.lib.qgb_sample_state_scratch_bytes(n)), rt.stream))
        np.testing.assert_array_equal(a.to_numpy(), b.to_numpy())


def test_mixed_precision_overlap(backend):
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray, DeviceState

    rt = backend.rt
    psi = rand_state(16, 8)
    a = DeviceState.from_numpy(psi)
    b = DeviceState.from_numpy(psi.astype(np.complex64))
    out = DeviceArray((2,), np.float64, rt)
    check(rt.lib.qgb_inner_mixed(a.ptr, a.code, b.ptr, b.code, 16, out.ptr,
                                 rt.scratch(rt.lib.qgb_inner_scratch_bytes()), rt.stream))
    re, im = out.to_numpy()
    want = np.vdot(psi, psi.astype(np.complex64).astype(np.complex128))
    assert abs(re - want.real) < 1e-12 and abs(im - want.imag) < 1e-12


def test_sampling_seed_protocol(backend):
    """Same seed -> same draws; zero-probability outcomes never drawn."""
    p = np.array([0.5, 0.0, 0.25, 0.0, 0.0, 0.25, 0.0, 0.0])
    backend.set_seed(7)
    a = backend.sample_shots(p, 10000)
    backend.set_seed(7)
    b = backend.sample_shots(p, 10000)
    np.testing.assert_array_equal(a, b)
    assert set(np.unique(a)) <= {0, 2, 5}
    backend.set_seed(7)
    f = backend.sample_frequencies(p, 100000)
    assert set(f) <= {0, 2, 5} and sum(f.values()) == 100000


def test_deterministic_outcome_reference_case(backend):
    """tests/test_measurements.py:63-78: X on qubits, 1e6 shots give one outcome."""
    from qibo_gb300 import Circuit, gates

    c = Circuit(4)
    c.add(gates.X(0)); c.add(gates.X(2)); c.add(gates.M(0, 1, 2, 3))
    res = backend.execute_circuit(c, nshots=1_000_000)
    assert res.frequencies() == {"1010": 1_000_000}
    s = res.samples()
    assert s.shape == (1_000_000, 4) and (s == [1, 0, 1, 0]).all()


def test_frequencies_match_reference_distribution(backend, gold):
    """The reference's seeded 1e5-shot histogram and ours come from the same
    distribution (two-sample chi-square); bit-equality is not expected
    because the reference draws from numpy's MT19937."""
    data, _ = gold
    from qibo_gb300 import Circuit, gates

    c = Circuit(3)
    c.add(gates.H(0)); c.add(gates.RY(1, 0.7)); c.add(gates.CNOT(0, 2)); c.add(gates.M(0, 1, 2))
    backend.set_seed(1234)
    res = backend.execute_circuit(c, nshots=100000)
    np.testing.assert_allclose(np.asarray(res.probabilities([0, 1, 2])), data["freq3_probs"], atol=1e-15)
    f = res.frequencies(binary=False)
    ours = np.array([f.get(i, 0) for i in range(8)])
    theirs = data["freq3_counts"]
    from scipy.stats import chi2_contingency

    keep = (ours + theirs) > 0
    assert chi2_contingency(np.stack([ours[keep], theirs[keep]]))[1] > 1e-4


# --------------------------------------------------------- expectation --
@pytest.mark.parametrize("n", [6, 8])
def test_tfim_expectation_golden(backend, gold, n):
    data, _ = gold
    from qibo_gb300.device import DeviceState

    st = DeviceState.from_numpy(data[f"tfim{n}_state"])
    t, q, c = ref.tfim_terms(n)
    from qibo_gb300.engine import pauli_masks

    xs, zs = zip(*[pauli_masks(tt, qq) for tt, qq in zip(t, q)])
    e = backend.engine_gb.expect_pauli(st, xs, zs, c)
    assert abs(e - float(data[f"tfim{n}_energy"])) < 1e-12


def test_pauli_strings_with_y_vs_oracle(backend):
    n = 12
    psi = rand_state(n, 9)
    rng = np.random.default_rng(4)
    terms, qubits, coefs = [], [], []
    for _ in range(40):
        k = rng.integers(1, 5)
        qs = tuple(int(x) for x in rng.choice(n, k, replace=False))
        terms.append("".join(rng.choice(list("XYZ"), k)))
        qubits.append(qs)
        coefs.append(float(rng.normal()))
    want = ref.exp_value_observable_symbolic(psi, terms, qubits, coefs, n)
    from qibo_gb300.device import DeviceState
    from qibo_gb300.engine import pauli_masks

    st = DeviceState.from_numpy(psi)
    xs, zs = zip(*[pauli_masks(t, q) for t, q in zip(terms, qubits)])
    got = backend.engine_gb.expect_pauli(st, xs, zs, coefs)
    assert abs(got - want) < 1e-12


@pytest.mark.parametrize("n", [10, 14])
@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-12)])
def test_z_strings_vs_oracle(n, dtype, tol):
    """Diagonal terms through the Walsh-Hadamard kernel (2^10 amplitudes or
    more): 100 random Z strings, so two launches of at most 64 terms, with
    masks on every index bit including bits 5..9 that the transform spans.
    The transform runs in double-float, so complex64 states too match the
    exact value of their stored amplitudes to 1e-12."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState
    from qibo_gb300.engine import pauli_masks

    b = GB300Backend(dtype)
    psi = rand_state(n, 31)
    rng = np.random.default_rng(8)
    terms, qubits, coefs = [], [], []
    for _ in range(100):
        k = int(rng.integers(1, 6))
        qs = tuple(int(x) for x in rng.choice(n, k, replace=False))
        terms.append("Z" * k)
        qubits.append(qs)
        coefs.append(float(rng.normal()))
    st = DeviceState.from_numpy(psi.astype(dtype), dtype)
    want = ref.exp_value_observable_symbolic(np.asarray(st).astype(np.complex128), terms, qubits, coefs, n)
    xs, zs = zip(*[pauli_masks(t, q) for t, q in zip(terms, qubits)])
    assert abs(b.engine_gb.expect_pauli(st, xs, zs, coefs) - want) < tol


@pytest.mark.parametrize("n", [16, 20])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_flip_tiles_vs_oracle(n, dtype):
    """X/Y terms batched per shared-memory tile (k_expect_flip_tile: states of
    2^13 amplitudes or more, masks on up to 7 index bits above bit 4 per
    batch): 60 random Pauli strings on 1-4 qubits plus the transverse-field
    terms, against the oracle on the stored amplitudes, to 1e-12."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState
    from qibo_gb300.engine import pauli_masks

    b = GB300Backend(dtype)
    psi = rand_state(n, 5 + n).astype(dtype)
    rng = np.random.default_rng(n)
    terms, qubits, coefs = [], [], []
    for _ in range(60):
        k = int(rng.integers(1, 5))
        qs = tuple(int(x) for x in rng.choice(n, k, replace=False))
        terms.append("".join(rng.choice(list("XYZ"), k)))
        qubits.append(qs)
        coefs.append(float(rng.normal()))
    for q in range(n):
        terms.append("X")
        qubits.append((q,))
        coefs.append(float(rng.normal()))
    st = DeviceState.from_numpy(psi)
    want = ref.exp_value_observable_symbolic(psi.astype(np.complex128), terms, qubits, coefs, n)
    xs, zs = zip(*[pauli_masks(t, q) for t, q in zip(terms, qubits)])
    assert abs(b.engine_gb.expect_pauli(st, xs, zs, coefs) - want) < 1e-12


@pytest.mark.parametrize("n", [12, 18])
def test_single_term_flips_complex64(n):
    """One X or Y term per flip mask (the transverse-field terms of TFIM),
    complex64: the double-float pair kernel against the exact value of the
    stored amplitudes, to 1e-12."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState
    from qibo_gb300.engine import pauli_masks

    b = GB300Backend("complex64")
    psi = rand_state(n, 77).astype(np.complex64)
    rng = np.random.default_rng(12)
    terms, qubits, coefs = [], [], []
    for q in range(n):
        f = "X" if q % 3 else "Y"
        extra = [] if q % 2 else [int((q + 5) % n)]
        terms.append(f + "Z" * len(extra))
        qubits.append(tuple([q] + extra))
        coefs.append(float(rng.normal()))
    st = DeviceState.from_numpy(psi)
    want = ref.exp_value_observable_symbolic(psi.astype(np.complex128), terms, qubits, coefs, n)
    xs, zs = zip(*[pauli_masks(t, q) for t, q in zip(terms, qubits)])
    assert abs(b.engine_gb.expect_pauli(st, xs, zs, coefs) - want) < 1e-12


def test_dense_expectation_vs_oracle(backend):
    n = 8
    psi = rand_state(n, 2)
    h = np.random.default_rng(1).normal(size=(2**n, 2**n)) + 1j * np.random.default_rng(2).normal(size=(2**n, 2**n))
    h = h + h.conj().T
    want = ref.expectation_value(h, psi * 1.7, normalize=True)
    from qibo_gb300.device import DeviceState

    got = backend.expectation_value(h, DeviceState.from_numpy(psi * 1.7), normalize=True)
    assert abs(got - want) < 1e-10


# ------------------------------------------------ full-size properties --
def test_n26_qft_roundtrip_and_norm(backend):
    """At 26 qubits: QFT then its inverse returns the initial state, and the
    norm stays 1 (size-independent properties; the oracle at this size would
    take minutes)."""
    n = 26
    psi = rand_state(n, 26)
    from qibo_gb300 import QFT
    from qibo_gb300.device import DeviceState

    st = DeviceState.from_numpy(psi)
    c = QFT(n)
    backend.execute_circuit(c, st)
    assert abs(backend.engine_gb.norm2(st) - 1.0) < 1e-12
    backend.execute_circuit(c.invert(), st)
    assert np.max(np.abs(np.asarray(st) - psi)) < 1e-12


def test_errors_are_exceptions(backend):
    from qibo_gb300.device import DeviceState

    st = DeviceState.zero(4)
    with pytest.raises(ValueError):
        backend.engine_gb.apply(st, [7], np.eye(2))
    with pytest.raises(ValueError):
        backend.engine_gb.apply(st, [1, 1], np.eye(4))
    with pytest.raises(RuntimeError):
        backend.execute_circuit(make_circuit(40, []))  # 16 TiB: device OOM -> RuntimeError


@pytest.mark.parametrize("n", [8, 14])
def test_per_gate_double_float_vs_oracle(n):
    """complex128 gate by gate (qgb_apply_circuit without QGB_PLAN_BLOCKED):
    dense 1- and 2-qubit gates in double-float, the doubles split and joined
    with integer operations.  Depth-30 brickwork plus random dense 2-qubit
    gates (some controlled) against the FP64 oracle to 1e-12, and against the
    IEEE FP64 per-gate path (QGB_PLAN_STRICT_FP64)."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    b = GB300Backend("complex128")
    ops = ref.brickwork_ops(n, 30, 40 + n)
    rng = np.random.default_rng(n)
    descs = [(q, (), ref.gate_matrix(name, p)) for name, q, p in ops]
    for _ in range(12):
        q = tuple(int(x) for x in rng.choice(n, 3, replace=False))
        u, _ = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
        ctrl = (q[2],) if rng.random() < 0.5 else ()
        descs.append((q[:2], ctrl, u))
        ops.append(("__dense2", q, u, ctrl))
    psi0 = rand_state(n, 70 + n)
    want = psi0.copy()
    for op in ops:
        if op[0] == "__dense2":
            _, q, u, ctrl = op
            want = ref.apply_gate_controlled_by(want, u, ctrl, q[:2], n) if ctrl else ref.apply_gate(want, u, q[:2], n)
        else:
            want = ref.apply_gate(want, ref.gate_matrix(op[0], op[2]), op[1], n)
    for strict in (False, True):
        st = DeviceState.from_numpy(psi0)
        b.engine_gb.apply_many(st, descs, blocked=False, strict_fp64=strict)
        assert np.max(np.abs(np.asarray(st) - want)) < 1e-12, strict
    # dense 1-qubit gates share their pairs between FP64 and double-float
    # warps; every share (all double-float to all FP64) meets the same bar
    for w in ("0", "5", "8"):
        os.environ["QIBO_GB300_DF_FP64_WARPS"] = w
        try:
            st = DeviceState.from_numpy(psi0)
            b.engine_gb.apply_many(st, descs, blocked=False)
        finally:
            del os.environ["QIBO_GB300_DF_FP64_WARPS"]
        assert np.max(np.abs(np.asarray(st) - want)) < 1e-12, w


def test_backend_apply_gate_c128(backend):
    """Backend.apply_gate (the reference's per-gate entry point,
    backends/abstract.py:2322-2361) in complex128: dense 1- and 2-qubit gates
    in the FP64 / double-float warp mix by default, IEEE FP64 with
    strict_fp64; other gates through their own kernels.  Against the FP64
    oracle to 1e-12."""
    from qibo_gb300 import gates
    from qibo_gb300.device import DeviceState

    n = 12
    psi = rand_state(n, 91)
    ops = [("U3", (0,), (0.3, 1.1, -0.4)), ("H", (n - 1,), ()), ("RY", (3,), (0.7,)), ("CNOT", (2, 9), ()),
           ("fSim", (5, 1), (0.4, 0.9)), ("CZ", (4, 7), ()), ("TOFFOLI", (0, 6, 11), ()), ("SWAP", (8, 10), ()),
           ("U3", (n - 2,), (1.3, -0.2, 0.6)), ("CU3", (6, 3), (0.5, 0.1, -0.8))]
    want = ref.execute(ops, n, psi)
    for strict in (False, True):
        backend.strict_fp64 = strict
        try:
            st = DeviceState.from_numpy(psi)
            for name, qs, params in ops:
                st = backend.apply_gate(getattr(gates, name)(*qs, *params), st, n)
            got = np.asarray(st)
        finally:
            backend.strict_fp64 = False
        assert np.max(np.abs(got - want)) < TOL128, strict
