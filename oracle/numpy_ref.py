"""numpy restatement of qibo 0.3.5's NumpyBackend state-vector hot path.

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
product path never imports this module.

Every function names the reference file:line it restates.  Paths are relative
to the reference project's ``src/qibo/``.  The arithmetic is the reference's:
per gate a transpose that moves the gate's qubit axes to the front, a reshape
to (2^k, -1), one ``matrix @ state`` product (OpenBLAS zgemm/cgemm) and the
inverse transpose.

Bit order (reference convention): qubit 0 is the most significant bit of the
amplitude index; the state reshaped to ``nqubits * (2,)`` has axis ``q`` for
qubit ``q`` (``backends/abstract.py:2327-2355``).
"""

from __future__ import annotations

import cmath
import math
from collections import Counter
from string import ascii_letters
from typing import Dict, List, Sequence, Tuple

import numpy as np

SHOT_BATCH_SIZE = 2**18  # config.py:41


# --------------------------------------------------------------------------
# Gate matrices: backends/npmatrices.py (closed forms, computed in complex128
# and then cast to the backend dtype, ``NumpyMatrices._cast`` :20-23)
# --------------------------------------------------------------------------

def _c(rows, dtype):
    return np.array(rows, dtype=dtype)


def gate_matrix(name: str, params: Sequence[float] = (), dtype="complex128") -> np.ndarray:
    """Matrix of a named gate, restating ``backends/npmatrices.py``.

    H :27, X :31, Y :35, Z :39, SX :43, SXDG :47, S :51, SDG :55, T :59,
    TDG :65, RX :79, RY :84, RZ :89, U1 :113, U2 :117, U3 :125, CNOT :144,
    CY :150, CZ :162, CSX :176, CSXDG :190, CRX :203, CRY :214, CRZ :220,
    CU1 :230, CU2 :240, CU3 :251, SWAP :265, iSWAP :271, FSWAP :307,
    fSim :312, RXX :353, RYY :366, RZZ :379, TOFFOLI :457, CCZ :473.
    """
    p = list(params)
    s2 = 1 / math.sqrt(2)
    if name == "I":
        return np.eye(2 ** int(p[0]) if p else 2, dtype=dtype)
    if name == "H":
        return _c([[1, 1], [1, -1]], dtype) / math.sqrt(2)
    if name == "X":
        return _c([[0, 1], [1, 0]], dtype)
    if name == "Y":
        return _c([[0j, -1j], [1j, 0j]], dtype)
    if name == "Z":
        return _c([[1, 0], [0, -1]], dtype)
    if name == "SX":
        return _c([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]], dtype) / 2
    if name == "SXDG":
        return _c([[1 - 1j, 1 + 1j], [1 + 1j, 1 - 1j]], dtype) / 2
    if name == "S":
        return _c([[1, 0], [0, 1j]], dtype)
    if name == "SDG":
        return _c([[1, 0], [0, -1j]], dtype)
    if name == "T":
        return _c([[1, 0], [0, cmath.exp(1j * math.pi / 4.0)]], dtype)
    if name == "TDG":
        return _c([[1, 0], [0, cmath.exp(-1j * math.pi / 4.0)]], dtype)
    if name == "RX":
        c, s = np.cos(p[0] / 2.0) + 0j, -1j * np.sin(p[0] / 2.0)
        return _c([[c, s], [s, c]], dtype)
    if name == "RY":
        c, s = np.cos(p[0] / 2.0) + 0j, np.sin(p[0] / 2.0) + 0j
        return _c([[c, -s], [s, c]], dtype)
    if name == "RZ":
        ph = np.exp(0.5j * p[0])
        return _c([[np.conj(ph), 0], [0, ph]], dtype)
    if name == "U1":
        return _c([[1, 0], [0, np.exp(1j * p[0])]], dtype)
    if name == "U2":
        ep, em = np.exp(1j * (p[0] + p[1]) / 2.0), np.exp(1j * (p[0] - p[1]) / 2.0)
        return _c([[np.conj(ep), -np.conj(em)], [em, ep]], dtype) / math.sqrt(2)
    if name == "U3":
        ct, st = np.cos(p[0] / 2), np.sin(p[0] / 2)
        ep, em = np.exp(1j * (p[1] + p[2]) / 2.0), np.exp(1j * (p[1] - p[2]) / 2.0)
        return _c([[np.conj(ep) * ct, -np.conj(em) * st], [em * st, ep * ct]], dtype)
    if name in ("CNOT", "CY", "CZ", "CRX", "CRY", "CRZ", "CU1", "CU2", "CU3", "CSX", "CSXDG"):
        base = {"CNOT": "X", "CY": "Y", "CZ": "Z", "CRX": "RX", "CRY": "RY", "CRZ": "RZ",
                "CU1": "U1", "CU2": "U2", "CU3": "U3", "CSX": "SX", "CSXDG": "SXDG"}[name]
        m = np.eye(4, dtype="complex128")
        m[2:, 2:] = gate_matrix(base, p, "complex128")
        return m.astype(dtype)
    if name == "SWAP":
        return _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype)
    if name == "iSWAP":
        return _c([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]], dtype)
    if name == "FSWAP":
        return _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, -1]], dtype)
    if name == "fSim":
        ct, ist, ph = np.cos(p[0]) + 0j, -1j * np.sin(p[0]), np.exp(-1j * p[1])
        return _c([[1, 0, 0, 0], [0, ct, ist, 0], [0, ist, ct, 0], [0, 0, 0, ph]], dtype)
    if name == "RXX":
        c, s = np.cos(p[0] / 2.0) + 0j, -1j * np.sin(p[0] / 2.0)
        return _c([[c, 0, 0, s], [0, c, s, 0], [0, s, c, 0], [s, 0, 0, c]], dtype)
    if name == "RYY":
        c, s = np.cos(p[0] / 2.0) + 0j, -1j * np.sin(p[0] / 2.0)
        return _c([[c, 0, 0, -s], [0, c, s, 0], [0, s, c, 0], [-s, 0, 0, c]], dtype)
    if name == "RZZ":
        ph = np.exp(0.5j * p[0])
        return _c(np.diag([np.conj(ph), ph, ph, np.conj(ph)]), dtype)
    if name == "TOFFOLI":
        m = np.eye(8, dtype="complex128")
        m[6:, 6:] = [[0, 1], [1, 0]]
        return m.astype(dtype)
    if name == "CCZ":
        m = np.eye(8, dtype="complex128")
        m[7, 7] = -1
        return m.astype(dtype)
    raise KeyError(f"oracle has no matrix for gate {name}")


# --------------------------------------------------------------------------
# Gate application: backends/abstract.py:2322-2361, einsum_utils.py:94-110
# --------------------------------------------------------------------------

def permutations(qubits: Tuple[int, ...], nqubits: int):
    """``einsum_utils.permutations`` (backends/einsum_utils.py:94-110)."""
    fwd = list(qubits) + [q for q in range(nqubits) if q not in qubits]
    inv = [0] * nqubits
    for i, q in enumerate(fwd):
        inv[q] = i
    return fwd, inv


def apply_gate(state: np.ndarray, matrix: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """``Backend.apply_gate`` state-vector branch (backends/abstract.py:2322-2361).

    transpose(fwd) -> reshape(2^k, -1) -> ``matrix @ state`` -> reshape ->
    transpose(inv) (:2350-2355).  ``qubits`` is ``gate.qubits`` = controls
    then targets (gates/abstract.py:440), the row order of the matrix.
    """
    shape = nqubits * (2,)
    st = np.reshape(state, shape)
    fwd, inv = permutations(tuple(qubits), nqubits)
    st = np.transpose(st, fwd)
    st = np.reshape(st, (2 ** len(qubits), -1))
    st = matrix @ st
    st = np.reshape(st, shape)
    st = np.transpose(st, inv)
    return np.reshape(st, (2**nqubits,))


def control_order(controls: Sequence[int], targets: Sequence[int], nqubits: int):
    """``einsum_utils.control_order`` (backends/einsum_utils.py:58-72)."""
    loop_start = 0
    order = list(controls)
    tg = list(targets)
    for control in controls:
        for i in range(loop_start, control):
            order.append(i)
        loop_start = control + 1
        for i, t in enumerate(targets):
            if t > control:
                tg[i] -= 1
    for i in range(loop_start, nqubits):
        order.append(i)
    return order, tg


def apply_gate_string(targets: Sequence[int], nqubits: int) -> str:
    """``einsum_utils.apply_gate_string`` with ``prepare_strings``
    (backends/einsum_utils.py:13-33): the matrix is indexed (out, in)."""
    inp = list(ascii_letters[:nqubits])
    out = list(inp)
    trans = list(ascii_letters[nqubits: nqubits + len(targets)])
    for i, t in enumerate(targets):
        trans.append(inp[t])
        out[t] = trans[i]
    return "{},{}->{}".format("".join(inp), "".join(trans), "".join(out))


def apply_gate_controlled_by(state, matrix, controls, targets, nqubits) -> np.ndarray:
    """``Backend._apply_gate_controlled_by`` (backends/abstract.py:3176-3197).

    The target matrix acts only on the slice where every control is 1.
    """
    k = len(targets)
    m = np.reshape(matrix, 2 * k * (2,))
    ncontrol = len(controls)
    nactive = nqubits - ncontrol
    order, tg = control_order(sorted(controls), targets, nqubits)
    st = np.transpose(np.reshape(state, nqubits * (2,)), order)
    st = np.reshape(st, (2**ncontrol,) + nactive * (2,))
    opstring = apply_gate_string(tg, nactive)
    updates = np.einsum(opstring, st[-1], m)
    st = np.concatenate([st[:-1], updates[None]], axis=0)
    st = np.reshape(st, nqubits * (2,))
    rorder = [0] * len(order)
    for i, r in enumerate(order):
        rorder[r] = i
    st = np.transpose(st, rorder)
    return np.reshape(st, (2**nqubits,))


def zero_state(nqubits: int, dtype="complex128") -> np.ndarray:
    """``Backend.zero_state`` (backends/abstract.py:2243-2273)."""
    st = np.zeros(2**nqubits, dtype=dtype)
    st[0] = 1
    return st


def execute(ops, nqubits: int, initial_state=None, dtype="complex128") -> np.ndarray:
    """Gate loop of ``Backend._execute_circuit`` (backends/abstract.py:3306-3322).

    ``ops`` is a list of ``(name, qubits, params)`` or
    ``(name, targets, params, controls)`` tuples; ``qubits`` follows the
    reference's ``gate.qubits`` order (controls first, then targets).  For the
    four-tuple form (``gate.controlled_by``) the matrix is that of the target
    gate and is applied on the all-controls-1 slice.  ``name`` may also be
    ``"Unitary"`` with ``params`` holding the matrix.
    """
    st = zero_state(nqubits, dtype) if initial_state is None else np.asarray(initial_state, dtype=dtype).copy()
    for op in ops:
        name, qubits, params = op[0], tuple(op[1]), op[2]
        m = np.asarray(params, dtype=dtype) if name == "Unitary" else gate_matrix(name, params, dtype)
        if len(op) > 3 and op[3]:
            st = apply_gate_controlled_by(st, m, tuple(op[3]), qubits, nqubits)
        else:
            st = apply_gate(st, m, qubits, nqubits)
    return st


# --------------------------------------------------------------------------
# Fusion matrix: backends/abstract.py:2680-2717
# --------------------------------------------------------------------------

def matrix_fused(target_qubits: Sequence[int], gates) -> np.ndarray:
    """``Backend.matrix_fused`` (backends/abstract.py:2680-2717), dense numpy.

    ``gates`` is a list of ``(qubits, matrix)``; ``target_qubits`` is the
    sorted qubit list of the fused block (gates/special.py:38).  Each gate
    matrix is kron'd with identity, its axes permuted onto the block's qubits
    and left-multiplied into the accumulated matrix.
    """
    rank = len(target_qubits)
    total = np.eye(2**rank, dtype=np.complex128)
    for qubits, gm in gates:
        gm = np.kron(gm, np.eye(2 ** (rank - len(qubits))))
        shp = gm.shape
        gm = np.reshape(gm, 2 * rank * (2,))
        indices = list(qubits) + [q for q in target_qubits if q not in qubits]
        indices = list(np.argsort(indices))
        trans = indices + [i + rank for i in indices]
        gm = np.reshape(np.transpose(gm, trans), shp)
        total = gm @ total
    return total


# --------------------------------------------------------------------------
# Probabilities and sampling: backends/abstract.py:2734-2801, :3371-3381
# --------------------------------------------------------------------------

def order_probabilities(probs: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """``Backend._order_probabilities`` (backends/abstract.py:3371-3381)."""
    unmeasured, reduced = [], {}
    for q in range(nqubits):
        if q in qubits:
            reduced[q] = q - len(unmeasured)
        else:
            unmeasured.append(q)
    return np.transpose(probs, [reduced.get(q) for q in qubits])


def calculate_probabilities(state: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """``Backend.calculate_probabilities`` state-vector branch (:2749-2758).

    Probabilities are in the state's real dtype (float32 for complex64).
    """
    rtype = np.real(state).dtype
    unmeasured = tuple(set(range(nqubits)) ^ set(qubits))
    probs = np.reshape(np.abs(state) ** 2, nqubits * (2,)).astype(rtype)
    if unmeasured:
        probs = np.sum(probs, axis=unmeasured)
    return order_probabilities(probs, qubits, nqubits).ravel()


def sample_shots(probabilities: np.ndarray, nshots: int, rng=None) -> np.ndarray:
    """``Backend.sample_shots`` -> ``random_choice`` (:2774-2781, :1265-1309).

    The reference draws from numpy's legacy global MT19937 stream
    (``np.random.choice``); ``rng`` lets a test pass a seeded generator.
    """
    choice = (rng or np.random).choice
    return choice(np.arange(len(probabilities)), size=nshots, p=probabilities).astype(np.int64)


def sample_frequencies(probabilities: np.ndarray, nshots: int, rng=None) -> Counter:
    """``Backend.sample_frequencies`` + ``update_frequencies`` (:2760-2772, :2795-2801)."""
    nprobs = probabilities / np.sum(probabilities)
    freqs = np.zeros(len(nprobs), dtype=np.int64)
    batches = [SHOT_BATCH_SIZE] * (nshots // SHOT_BATCH_SIZE) + [nshots % SHOT_BATCH_SIZE]
    for b in batches:
        s = sample_shots(nprobs, b, rng)
        res, counts = np.unique(s, return_counts=True)
        freqs[res] += counts
    return Counter({i: int(f) for i, f in enumerate(freqs) if f > 0})


def samples_to_binary(samples: np.ndarray, nqubits: int) -> np.ndarray:
    """``Backend.samples_to_binary`` (backends/abstract.py:2783-2786)."""
    qrange = np.arange(nqubits - 1, -1, -1, dtype=np.int32)
    return np.right_shift(samples[:, None], qrange) % 2


# --------------------------------------------------------------------------
# Collapse: backends/abstract.py:2424-2440, :3236-3247, :3279-3304
# --------------------------------------------------------------------------

def collapse_statevector(state: np.ndarray, qubits: Sequence[int], shot: int, nqubits: int,
                         normalize: bool = True) -> np.ndarray:
    """``Backend._collapse_statevector`` (:3279-3304) with ``_append_zeros``
    (:3236-3247): transpose the measured qubits to the front, keep the slice
    of outcome ``shot`` (qubits[0] the most significant bit), divide it by its
    norm, and put the measured axes back with zeros on the other outcomes.
    The axes go back in the order of ``qubits``, which is only the inverse
    of the transpose for an ascending list (the reference's caller,
    ``M.apply`` in gates/measurements.py:199-204, sorts them)."""
    shape = state.shape
    binshot = list(samples_to_binary(np.array([shot], dtype=np.int64), len(qubits))[0])
    st = np.reshape(state, nqubits * (2,))
    order = list(qubits) + [q for q in range(nqubits) if q not in qubits]
    st = np.transpose(st, order)
    subshape = (2 ** len(qubits),) + (nqubits - len(qubits)) * (2,)
    st = np.reshape(st, subshape)[int(shot)]
    if normalize:
        st = st / np.sqrt(np.sum(np.abs(st) ** 2))
    for q, r in zip(qubits, binshot):
        st = np.expand_dims(st, q)
        st = np.concatenate([np.zeros_like(st), st], axis=q) if r == 1 else np.concatenate([st, np.zeros_like(st)], axis=q)
    return np.reshape(st, shape)


# --------------------------------------------------------------------------
# Expectation values from samples: backends/abstract.py:2873-2926, :3056-3140
# --------------------------------------------------------------------------

def exp_value_from_frequencies(frequencies: Dict[str, int], terms_qubits, terms_coefficients, qubit_map,
                               constant: float = 0.0) -> float:
    """``Backend.exp_value_diagonal_observable_symbolic_from_samples``
    (:2873-2926) on a frequency table of bitstrings over ``qubit_map``: each
    term is its coefficient times the frequency-weighted mean of
    (-1)^(number of 1 bits on the term's qubits)."""
    keys = list(frequencies.keys())
    counts = np.array(list(frequencies.values()), dtype=np.float64)
    counts = counts / counts.sum()
    qubit_map = list(qubit_map)
    expvals = []
    for qubits, coefficient in zip(terms_qubits, terms_coefficients):
        expvals.extend([coefficient * (-1) ** [k[qubit_map.index(q)] for q in qubits].count("1") for k in keys])
    expvals = np.array(expvals, dtype=counts.dtype).reshape(len(terms_coefficients), len(frequencies))
    return float(np.sum(expvals @ counts) + constant)


def basis_rotation(factor: str):
    """Matrix of ``basis_rotation()`` of the Pauli gate ``factor``
    (gates/gates.py:191-292): X -> H, Y -> (Y + Z)/sqrt(2), Z -> none."""
    if factor == "X":
        return gate_matrix("H")
    if factor == "Y":
        return (gate_matrix("Y") + gate_matrix("Z")) / math.sqrt(2)
    return None


def exp_value_observable_symbolic_from_samples(state: np.ndarray, groups, nqubits: int, constant: float, nshots: int,
                                               rng=None) -> float:
    """``Backend.exp_value_observable_symbolic_from_samples`` (:3056-3140) on a
    final state: for each group ``(coefficients, observables, qubits)`` the
    state is rotated by the basis rotations of the group's measured qubits
    (first non-identity factor per qubit), ``nshots`` outcomes of those
    qubits are drawn, and their frequencies give the group's terms."""
    total = 0.0
    for coefs, observables, terms_qubits in groups:
        measured = {}
        for qubits, observable in zip(terms_qubits, observables):
            for q, f in zip(qubits, observable):
                if f != "I" and q not in measured:
                    measured[q] = f
        st = state
        for q, f in measured.items():
            m = basis_rotation(f)
            if m is not None:
                st = apply_gate(st, m.astype(state.dtype), (q,), nqubits)
        qmap = list(measured)
        probs = calculate_probabilities(st, qmap, nqubits)
        freq = sample_frequencies(probs, nshots, rng)
        bfreq = {f"{k:b}".zfill(len(qmap)): v for k, v in freq.items()}
        total += exp_value_from_frequencies(bfreq, terms_qubits, coefs, qmap)
    return total + constant


# --------------------------------------------------------------------------
# Expectation values: backends/abstract.py:2807-2825, :2946-3054
# --------------------------------------------------------------------------

def expectation_value(hamiltonian: np.ndarray, state: np.ndarray, normalize: bool) -> float:
    """``Backend.expectation_value`` state-vector branch (:2807-2825)."""
    ev = np.real(np.sum(np.conj(state) * (hamiltonian @ state)))
    if normalize:
        ev /= np.sum(np.abs(state) ** 2)
    return ev


def exp_value_observable_symbolic(state, terms: Sequence[str], term_qubits, term_coefficients, nqubits: int) -> float:
    """``Backend.exp_value_observable_symbolic`` state-vector branch (:2946-3054).

    One einsum over the whole state per term: conj(state), the per-qubit
    Pauli factors, and the state.
    """
    shape = nqubits * (2,)
    st = np.reshape(state, shape)
    idx = [ascii_letters[e] for e in range(2 * nqubits)]
    dag_idx, st_idx = idx[:nqubits], idx[nqubits:]
    dag_s, st_s = "".join(dag_idx), "".join(st_idx)
    pauli = {"X": gate_matrix("X", (), state.dtype), "Y": gate_matrix("Y", (), state.dtype),
             "Z": gate_matrix("Z", (), state.dtype)}
    expval = 0.0
    for term, qubits, coeff in zip(terms, term_qubits, term_coefficients):
        tm = {q: pauli[f] for f, q in zip(term, qubits) if f != "I"}
        if not tm:
            expval += np.real(coeff * np.sum(np.abs(state) ** 2))
            continue
        qs, mats = zip(*tm.items())
        obs_s = ",".join(dag_idx[q] + st_idx[q] for q in qs)
        new_s = st_s
        for q in set(range(nqubits)) - set(qs):
            new_s = new_s[:q] + dag_s[q] + new_s[q + 1:]
        expval += np.real(coeff * np.einsum(f"{dag_s},{obs_s},{new_s}->", np.conj(st), *mats, st))
    return float(expval)


def tfim_terms(nqubits: int, h: float = 1.0):
    """Pauli terms of ``hamiltonians.models.TFIM(n, h, dense=False)``
    (hamiltonians/models.py:649-662): -sum Z_i Z_{i+1} - h sum X_i with the
    periodic wrap Z_{n-1} Z_0.  Returned as (terms, qubits, coefficients)."""
    terms, qubits, coeffs = [], [], []
    for i in range(nqubits):
        terms.append("ZZ"); qubits.append((i, (i + 1) % nqubits)); coeffs.append(-1.0)
    for i in range(nqubits):
        terms.append("X"); qubits.append((i,)); coeffs.append(-h)
    return terms, qubits, coeffs


# --------------------------------------------------------------------------
# Circuit factories used by the workloads
# --------------------------------------------------------------------------

def qft_ops(nqubits: int, with_swaps: bool = True):
    """Gate list of ``models.QFT`` (models/qft.py:47-58)."""
    ops = []
    for i1 in range(nqubits):
        ops.append(("H", (i1,), ()))
        for i2 in range(i1 + 1, nqubits):
            ops.append(("CU1", (i2, i1), (math.pi / 2 ** (i2 - i1),)))
    if with_swaps:
        for q in range(nqubits // 2):
            ops.append(("SWAP", (q, nqubits - q - 1), ()))
    return ops


def brickwork_ops(nqubits: int, depth: int, seed: int):
    """Random U3 + CZ brickwork: per layer U3 on every qubit with angles from
    ``default_rng(seed).uniform(0, 2*pi, (depth, nqubits, 3))``, then CZ on
    pairs (l%2, l%2+1), (l%2+2, ...)."""
    ang = np.random.default_rng(seed).uniform(0, 2 * np.pi, (depth, nqubits, 3))
    ops = []
    for l in range(depth):
        for q in range(nqubits):
            ops.append(("U3", (q,), tuple(float(a) for a in ang[l, q])))
        for q in range(l % 2, nqubits - 1, 2):
            ops.append(("CZ", (q, q + 1), ()))
    return ops


def vqe_ops(nqubits: int, layers: int, params: Sequence[float]):
    """Hardware-efficient ansatz: per layer RY then RZ on every qubit, then a
    CNOT ladder (i, i+1).  ``params`` in ``Circuit.get_parameters`` order."""
    ops, k = [], 0
    for _ in range(layers):
        for q in range(nqubits):
            ops.append(("RY", (q,), (float(params[k]),))); k += 1
            ops.append(("RZ", (q,), (float(params[k]),))); k += 1
        for q in range(nqubits - 1):
            ops.append(("CNOT", (q, q + 1), ()))
    return ops


def parameter_shift_grad(build_ops, nqubits, params, terms, term_qubits, coeffs, scale_factor=1.0):
    """``derivative.parameter_shift`` (derivative.py:7-156) for rotation
    gates (``_Rn_``, generator eigenvalue 0.5, gates/gates.py:633-634):
    shift s = pi/(4*eig) (derivative.py:118), derivative =
    eig * (E(theta+s) - E(theta-s)) * scale_factor (derivative.py:153).
    ``build_ops(params)`` returns the op list for a parameter vector."""
    params = np.asarray(params, dtype=np.float64)
    eig = 0.5
    s = np.pi / (4 * eig)
    grads = np.zeros_like(params)

    def energy(p):
        st = execute(build_ops(p), nqubits)
        return exp_value_observable_symbolic(st, terms, term_qubits, coeffs, nqubits)

    for i in range(len(params)):
        p = params.copy(); p[i] += s
        ep = energy(p)
        p[i] -= 2 * s
        em = energy(p)
        grads[i] = eig * (ep - em) * scale_factor
    return grads


# --------------------------------------------------------------------------
# Density matrices: backends/abstract.py:2095-2241, :2297-2361, :2734-2748,
# :2807-2816, :2975-3054, :3199-3277
# --------------------------------------------------------------------------

def apply_gate_density(rho: np.ndarray, matrix: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """``Backend.apply_gate`` density branch (:2339-2349) with
    ``einsum_utils.apply_gate_density_matrix_string``
    (backends/einsum_utils.py:36-44): conj(U) contracted into the column
    axes ("right" string), then U into the row axes ("left" string)."""
    n, k = nqubits, len(qubits)
    m = np.reshape(matrix, 2 * k * (2,))
    inp = list(ascii_letters[:n])
    out = list(inp)
    trans = list(ascii_letters[n:n + k])
    for i, q in enumerate(qubits):
        trans.append(inp[q])
        out[q] = trans[i]
    rest = ascii_letters[n + k:n + k + n]
    inp, out, trans = "".join(inp), "".join(out), "".join(trans)
    st = np.reshape(rho, 2 * n * (2,))
    st = np.einsum(f"{rest}{inp},{trans}->{rest}{out}", st, np.conj(m))
    st = np.einsum(f"{inp}{rest},{trans}->{out}{rest}", st, m)
    return np.reshape(st, (2**n, 2**n))


def controlled_matrix(matrix: np.ndarray, ncontrols: int) -> np.ndarray:
    """U with ``ncontrols`` controls as one matrix on controls + targets: the
    identity except the all-ones control block."""
    d = matrix.shape[0] * 2**ncontrols
    full = np.eye(d, dtype=np.complex128)
    full[d - matrix.shape[0]:, d - matrix.shape[0]:] = matrix
    return full


def apply_gate_controlled_by_density(rho, matrix, controls, targets, nqubits) -> np.ndarray:
    """``Backend._apply_gate_controlled_by_density_matrix`` (:3199-3234)
    computes V rho V^dagger for V = U controlled on ``controls`` block by
    block; here V is formed and applied whole (the same map)."""
    return apply_gate_density(rho, controlled_matrix(matrix, len(controls)), list(sorted(controls)) + list(targets),
                              nqubits)


def apply_channel_density(rho: np.ndarray, coefficients, gates, coefficient_sum, nqubits: int) -> np.ndarray:
    """``Backend.apply_channel`` density branch (:2304-2312):
    (1 - sum c) rho + sum_k c_k K_k rho K_k^dagger; ``gates`` are
    (qubits, matrix) pairs."""
    new = (1 - coefficient_sum) * rho
    for c, (qs, m) in zip(coefficients, gates):
        new = new + c * apply_gate_density(rho, m, qs, nqubits)
    return new


def partial_trace_keep(rho: np.ndarray, traced: Sequence[int], nqubits: int) -> np.ndarray:
    """Tr over ``traced`` qubits, the others kept in ascending order."""
    keep = [q for q in range(nqubits) if q not in traced]
    st = np.reshape(rho, 2 * nqubits * (2,))
    inp = list(ascii_letters[:2 * nqubits])
    for q in traced:
        inp[q + nqubits] = inp[q]
    outs = "".join(inp[q] for q in keep) + "".join(inp[q + nqubits] for q in keep)
    red = np.einsum("".join(inp) + "->" + outs, st)
    d = 2 ** len(keep)
    return np.reshape(red, (d, d))


def _with_factor(reduced: np.ndarray, factor: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """reduced (on the qubits not in ``qubits``, ascending) (x) factor (on
    ``qubits`` in that order), axes put back in qubit order."""
    keep = [q for q in range(nqubits) if q not in qubits]
    t = np.tensordot(np.reshape(reduced, 2 * len(keep) * (2,)), np.reshape(factor, 2 * len(qubits) * (2,)), 0)
    # t's axes: kept rows, kept columns, factor rows, factor columns
    axes = keep + [q + nqubits for q in keep] + list(qubits) + [q + nqubits for q in qubits]
    perm = [axes.index(a) for a in range(2 * nqubits)]
    return np.reshape(np.transpose(t, perm), (2**nqubits, 2**nqubits))


def depolarizing_density(rho: np.ndarray, qubits: Sequence[int], lam: float, nqubits: int) -> np.ndarray:
    """``Backend.depolarizing_error_density_matrix`` (:2095-2132):
    (1 - lam) rho + lam Tr_T(rho) (x) I / 2^|T|."""
    d = 2 ** len(qubits)
    mixed = _with_factor(partial_trace_keep(rho, qubits, nqubits), np.eye(d) / d, qubits, nqubits)
    return (1 - lam) * rho + lam * mixed


def reset_density(rho: np.ndarray, qubit: int, p0: float, p1: float, nqubits: int) -> np.ndarray:
    """``Backend.reset_error_density_matrix`` (:2212-2232):
    (1 - p0 - p1) rho + p0 Tr_q(rho) (x) |0><0| + p1 X_q (that) X_q."""
    zero = _with_factor(partial_trace_keep(rho, [qubit], nqubits), np.diag([1.0, 0.0]), [qubit], nqubits)
    x = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    return (1 - p0 - p1) * rho + p0 * zero + p1 * apply_gate_density(zero, x, [qubit], nqubits)


def thermal_density(rho: np.ndarray, qubit: int, t_1: float, t_2: float, kw: dict, nqubits: int) -> np.ndarray:
    """``ThermalRelaxationChannel.apply`` (gates/channels.py:678-707): for
    T1 < T2 a 4 x 4 matrix on (q, q + n) of the flattened density matrix
    (thermal_error_density_matrix, :2234-2241); otherwise the reset map
    minus p_z rho plus p_z Z rho Z with Z on qubit 0, as the reference
    writes it (gates/channels.py:702-706)."""
    p0, p1 = kw["p_0"], kw["p_1"]
    if t_1 < t_2:
        e = kw["e_t2"]
        m = np.array([[1 - p1, 0, 0, p0], [0, e, 0, 0], [0, 0, e, 0], [p1, 0, 0, 1 - p0]], dtype=np.complex128)
        v = apply_gate(np.ravel(rho), m, [qubit, qubit + nqubits], 2 * nqubits)
        return np.reshape(v, rho.shape)
    pz = kw["p_z"]
    z = np.diag([1.0, -1.0]).astype(np.complex128)
    return reset_density(rho, qubit, p0, p1, nqubits) - pz * rho + pz * apply_gate_density(rho, z, [0], nqubits)


def calculate_probabilities_density(rho: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """``Backend.calculate_probabilities`` density branch (:2741-2748):
    measured qubits (sorted) to the front on both sides, "abab->a", then
    ``_order_probabilities``."""
    order = tuple(sorted(qubits))
    order += tuple(q for q in range(nqubits) if q not in qubits)
    order = order + tuple(q + nqubits for q in order)
    shape = 2 * (2 ** len(qubits), 2 ** (nqubits - len(qubits)))
    st = np.reshape(np.transpose(np.reshape(rho, 2 * nqubits * (2,)), order), shape)
    probs = np.abs(np.einsum("abab->a", st))
    probs = np.reshape(probs, len(qubits) * (2,))
    return order_probabilities(probs, qubits, nqubits).ravel()


def collapse_density(rho: np.ndarray, qubits: Sequence[int], shot: int, nqubits: int,
                     normalize: bool = True) -> np.ndarray:
    """``Backend._collapse_density_matrix`` (:3249-3277): the block of
    outcome ``shot`` on rows and columns, divided by its trace, with zeros
    elsewhere."""
    qubits = list(qubits)
    binshot = list(samples_to_binary(np.array([shot], dtype=np.int64), len(qubits))[0])
    order = qubits + [q + nqubits for q in qubits]
    order += [q for q in range(nqubits) if q not in qubits]
    order += [q + nqubits for q in range(nqubits) if q not in qubits]
    st = np.transpose(np.reshape(rho, 2 * nqubits * (2,)), order)
    sub = 2 * (2 ** len(qubits),) + 2 * (nqubits - len(qubits)) * (2,)
    st = np.reshape(st, sub)[int(shot), int(shot)]
    if normalize:
        dims = 2 ** (len(st.shape) // 2)
        st = st / np.trace(np.reshape(st, (dims, dims)))
    for q, r in zip(qubits + [q + nqubits for q in qubits], 2 * binshot):
        st = np.expand_dims(st, q)
        st = np.concatenate([np.zeros_like(st), st], axis=q) if r == 1 else np.concatenate([st, np.zeros_like(st)], axis=q)
    return np.reshape(st, rho.shape)


_PAULI = {"X": np.array([[0, 1], [1, 0]], dtype=np.complex128), "Y": np.array([[0, -1j], [1j, 0]]),
          "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128), "I": np.eye(2, dtype=np.complex128)}


def exp_value_observable_symbolic_density(rho, terms: Sequence[str], term_qubits, term_coefficients,
                                          nqubits: int) -> float:
    """``Backend.exp_value_observable_symbolic`` density branch
    (:3009-3030): per term, Re(c Tr(P rho)) contracted factor by factor."""
    total = 0.0
    for term, qubits, c in zip(terms, term_qubits, term_coefficients):
        st = np.array(rho, dtype=np.complex128)
        for f, q in zip(term, qubits):
            if f != "I":
                st = np.reshape(apply_gate(np.ravel(st), _PAULI[f], [q], 2 * nqubits), st.shape)  # P acting on rows
        total += float(np.real(c * np.trace(st)))
    return total


def expectation_value_density(hamiltonian: np.ndarray, rho: np.ndarray, normalize: bool) -> float:
    """``Backend.expectation_value`` density branch (:2810-2816)."""
    ev = float(np.real(np.trace(hamiltonian @ rho)))
    if normalize:
        ev /= float(np.real(np.trace(rho)))
    return ev


def thermal_parameters(t_1: float, t_2: float, time: float, excited_population: float = 0.0) -> dict:
    """``ThermalRelaxationChannel.__init__`` (gates/channels.py:601-660):
    p_0 = (1 - e^(-t/T1)) (1 - eta), p_1 = (1 - e^(-t/T1)) eta, and e_t2 =
    e^(-t/T2) for T1 < T2, else p_z = (e^(-t/T1) - e^(-t/T2)) / 2."""
    p_reset = 1 - math.exp(-time / t_1)
    kw = {"p_0": p_reset * (1 - excited_population), "p_1": p_reset * excited_population}
    if t_1 < t_2:
        kw["e_t2"] = math.exp(-time / t_2)
    else:
        kw["p_z"] = (math.exp(-time / t_1) - math.exp(-time / t_2)) / 2
    return kw


_NQ = {"H": 1, "X": 1, "Y": 1, "Z": 1, "RX": 1, "RY": 1, "RZ": 1, "U3": 1, "CNOT": 2, "CZ": 2, "fSim": 2,
       "SWAP": 2, "TOFFOLI": 3}


def _pauli_string(s: str) -> np.ndarray:
    m = np.eye(1, dtype=np.complex128)
    for f in s:
        m = np.kron(m, _PAULI[f])
    return m


def execute_density(ops, nqubits: int, rho=None) -> np.ndarray:
    """A density-matrix circuit given as (gate or channel name, constructor
    arguments, controlled_by qubits) in the reference's constructor
    conventions (gates/gates.py, gates/channels.py), applied as the
    reference's NumpyBackend does: gates by ``apply_gate_density``, Kraus /
    unitary / Pauli / amplitude- and phase-damping / readout channels by
    ``apply_channel_density``, depolarizing, reset and thermal relaxation by
    their special forms."""
    n = nqubits
    if rho is None:
        rho = np.zeros((2**n, 2**n), dtype=np.complex128)
        rho[0, 0] = 1
    rho = np.array(rho, dtype=np.complex128)
    for name, args, controls in ops:
        if name == "DepolarizingChannel":
            qs = (args[0],) if isinstance(args[0], int) else tuple(args[0])
            rho = depolarizing_density(rho, qs, args[1], n)
        elif name == "ResetChannel":
            rho = reset_density(rho, args[0], args[1][0], args[1][1], n)
        elif name == "ThermalRelaxationChannel":
            p = list(args[1])
            rho = thermal_density(rho, args[0], p[0], p[1], thermal_parameters(*p), n)
        elif name == "PauliNoiseChannel":
            qs = (args[0],) if isinstance(args[0], int) else tuple(args[0])
            probs = [pr for _, pr in args[1]]
            rho = apply_channel_density(rho, probs, [(qs, _pauli_string(s)) for s, _ in args[1]], sum(probs), n)
        elif name in ("AmplitudeDampingChannel", "PhaseDampingChannel"):
            g = args[1]
            k1 = [[0, math.sqrt(g)], [0, 0]] if name == "AmplitudeDampingChannel" else [[0, 0], [0, math.sqrt(g)]]
            ks = [np.array([[1, 0], [0, math.sqrt(1 - g)]], dtype=np.complex128), np.array(k1, dtype=np.complex128)]
            rho = apply_channel_density(rho, [1, 1], [((args[0],), k) for k in ks], 1, n)
        elif name == "ReadoutErrorChannel":
            P = np.asarray(args[1])
            qs = (args[0],) if isinstance(args[0], int) else tuple(args[0])
            ks = []
            for j in range(len(P)):
                for k in range(len(P)):
                    m = np.zeros((len(P), len(P)), dtype=np.complex128)
                    m[j, k] = math.sqrt(P[k, j])
                    ks.append((qs, m))
            rho = apply_channel_density(rho, [1] * len(ks), ks, 1, n)
        elif name == "KrausChannel":
            rho = apply_channel_density(rho, [1] * len(args[1]), list(zip(args[0], args[1])), 1, n)
        elif name == "UnitaryChannel":
            probs = [p for p, _ in args[1]]
            rho = apply_channel_density(rho, probs, list(zip(args[0], [u for _, u in args[1]])), sum(probs), n)
        else:
            k = _NQ[name]
            qs, params = tuple(args[:k]), tuple(args[k:])
            m = gate_matrix(name, params)
            if controls:
                rho = apply_gate_controlled_by_density(rho, m, controls, qs, n)
            else:
                rho = apply_gate_density(rho, m, qs, n)
    return rho
