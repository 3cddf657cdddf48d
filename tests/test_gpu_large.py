"""Parity at 31 to 34 qubits, where amplitude indices need 64 bits and the
states take 34-137 GB, against answers known in closed form (no
self-comparison):

* a product state (U3 on every qubit from |0...0>): each amplitude is the
  product of the single-qubit amplitudes;
* that state through a random U3+CZ brickwork and its inverse, with engine
  fusion (5-qubit tensor-core blocks, the complex128 fixed-point chains),
  must come back;
* shots drawn straight from the state (qgb_sample_state) follow the product
  state's independent marginals; a collapse leaves a product state;
* QFT of a basis state |k> is column k of the DFT matrix, amplitude
  exp(2 pi i j k / 2^n) / 2^(n/2) (tests/test_models_qft.py:11-77 of the
  reference checks QFT against the same matrix).

Amplitudes are read back at 4096 sampled indices (plus the first and last
ones) with 16-byte copies; the tolerances are the ones the other parity
tests use: 1e-12 max-abs in complex128, 1e-5 in complex64.
"""

from __future__ import annotations

import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"complex128": 1e-12, "complex64": 1e-5}


def _u3_layer(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 2 * np.pi, (n, 3))


def _single_qubit_columns(angles):
    from qibo_gb300 import gates

    return np.array([gates.U3(0, *a).matrix()[:, 0] for a in angles])  # u_q = U3 |0>


def _product_amplitudes(u, n, idx):
    bits = (idx[:, None] >> (n - 1 - np.arange(n))[None, :]) & 1
    return np.prod(u[np.arange(n)[None, :], bits], axis=1)


def _indices(n, count=4096, seed=5):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, 2**n, size=count, dtype=np.int64)
    return np.unique(np.concatenate([idx, [0, 1, 2**n - 2, 2**n - 1]]))


def _gather(st, idx):
    """Amplitudes of device state ``st`` at ``idx`` (one small copy each)."""
    return st.take(idx)


def _brickwork(n, depth, seed):
    from qibo_gb300 import gates

    ang = np.random.default_rng(seed).uniform(0, 2 * np.pi, (depth, n, 3))
    gl = []
    for layer in range(depth):
        gl += [gates.U3(q, *ang[layer, q]) for q in range(n)]
        gl += [gates.CZ(q, q + 1) for q in range(layer % 2, n - 1, 2)]
    return gl


def _inverse(gl):
    from qibo_gb300 import gates

    inv = []
    for g in reversed(gl):
        if type(g).__name__ == "U3":
            th, ph, la = g.parameters
            inv.append(gates.U3(g.target_qubits[0], -th, -la, -ph))
        else:
            inv.append(g)  # CZ is its own inverse
    return inv


def _run(n, dtype, gl):
    from qibo_gb300 import Circuit
    from qibo_gb300.backend import GB300Backend

    b = GB300Backend(dtype)
    c = Circuit(n)
    c.add(gl)
    return b, b.execute_circuit(c).state()


def _u3_inverse_is_inverse():
    from qibo_gb300 import gates

    m = gates.U3(0, 0.3, 1.1, -0.7).matrix()
    mi = gates.U3(0, -0.3, 0.7, -1.1).matrix()
    return np.allclose(mi @ m, np.eye(2), atol=1e-15)


def test_u3_inverse_parameters():
    assert _u3_inverse_is_inverse()


@pytest.mark.parametrize("n,dtype", [(31, "complex128"), (32, "complex64")])
def test_product_state_and_brickwork_inverse(n, dtype):
    """U3 on every qubit, then a depth-4 brickwork and its inverse, engine
    fusion on: the product state comes back, at every sampled index."""
    from qibo_gb300 import gates

    ang = _u3_layer(n, 31)
    u = _single_qubit_columns(ang)
    idx = _indices(n)
    want = _product_amplitudes(u, n, idx)
    layer = [gates.U3(q, *ang[q]) for q in range(n)]
    b, st = _run(n, dtype, layer)
    err0 = np.max(np.abs(_gather(st, idx) - want))
    assert err0 < TOL[dtype], f"product state, n={n} {dtype}: {err0}"
    del st
    gc.collect()
    bw = _brickwork(n, 4, 7)
    b, st = _run(n, dtype, layer + bw + _inverse(bw))
    err = np.max(np.abs(_gather(st, idx) - want))
    assert err < TOL[dtype], f"brickwork then its inverse, n={n} {dtype}: {err}"
    del st, b
    gc.collect()


def test_sample_state_and_collapse_n31():
    """Shots on all 31 qubits drawn straight from the complex128 product
    state (qgb_sample_state): every qubit's frequency of 1 within 5 sigma of
    |u_q[1]|^2, and pairs of qubits uncorrelated.  Then a collapse of qubits
    0 and 30 onto outcome 1 leaves the product state with those factors
    replaced by their normalised |1> amplitudes."""
    from qibo_gb300 import gates
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray

    n, dtype = 31, "complex128"
    ang = _u3_layer(n, 131)
    u = _single_qubit_columns(ang)
    b, st = _run(n, dtype, [gates.U3(q, *ang[q]) for q in range(n)])
    rt, lib = b.rt, b.rt.lib
    nshots = 1_000_000
    samples = DeviceArray((nshots,), np.int64, rt)
    scratch = rt.scratch(lib.qgb_sample_state_scratch_bytes(n))
    check(lib.qgb_sample_state(st.ptr, n, st.code, nshots, 20261204, samples.ptr, scratch, rt.stream))
    s = samples.to_numpy()
    assert s.min() >= 0 and s.max() < 2**n
    ones = np.array([((s >> (n - 1 - q)) & 1).mean() for q in range(n)])
    p1 = np.abs(u[:, 1]) ** 2
    sig = np.sqrt(p1 * (1 - p1) / nshots)
    assert np.all(np.abs(ones - p1) < 5 * sig + 1e-12), np.max(np.abs(ones - p1) / sig)
    b0, b1 = (s >> (n - 1)) & 1, s & 1  # qubits 0 and n-1
    cov = (b0 * b1).mean() - b0.mean() * b1.mean()
    assert abs(cov) < 5 * np.sqrt(p1[0] * (1 - p1[0]) * p1[-1] * (1 - p1[-1]) / nshots)
    del samples
    b.engine_gb.collapse(st, [0, n - 1], 3, True)
    uc = u.copy()
    for q in (0, n - 1):
        uc[q] = [0.0, u[q, 1] / abs(u[q, 1])]
    idx = _indices(n, seed=9)
    err = np.max(np.abs(_gather(st, idx) - _product_amplitudes(uc, n, idx)))
    assert err < TOL[dtype], f"collapsed product state: {err}"
    assert abs(b.engine_gb.norm2(st) - 1.0) < 1e-12
    del st, b
    gc.collect()


def test_qft_of_a_basis_state_n31():
    """QFT(31) with swaps on |k>: amplitude j is exp(2 pi i j k / 2^31) /
    2^15.5 (the exact DFT, tests/test_models_qft.py:11-77), compared with
    integer phase arithmetic at every sampled index."""
    from qibo_gb300 import QFT
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState
    from qibo_gb300._lib import check

    n, N = 31, 2**31
    k = 0x5A3C96E1 % N
    b = GB300Backend("complex128")
    st = DeviceState(n, "complex128")
    check(b.rt.lib.qgb_state_basis(st.ptr, n, st.code, k, b.rt.stream))
    res = b.execute_circuit(QFT(n), initial_state=st)
    idx = _indices(n, seed=13)
    phase = np.array([(int(j) * k) % N for j in idx], dtype=np.float64) / N
    want = np.exp(2j * np.pi * phase) / np.sqrt(N)
    err = np.max(np.abs(_gather(res.state(), idx) - want))
    assert err < 1e-12, f"QFT(31)|{k}>: {err}"
    del st, res, b
    gc.collect()


@pytest.mark.parametrize("n,dtype", [(33, "complex128"), (34, "complex64")])
def test_memory_limit_product_state_brickwork_inverse(n, dtype):
    """The memory-limit sizes (137 GB states): U3 on every qubit, a depth-2
    brickwork and its inverse with engine fusion; the product state comes
    back at every sampled index."""
    from qibo_gb300 import gates
    from qibo_gb300.device import Runtime

    free, _ = Runtime.get().mem_info()
    if free < 2**n * (16 if dtype == "complex128" else 8) + (8 << 30):
        pytest.skip(f"needs {2**n * (16 if dtype == 'complex128' else 8) / 1e9:.0f} GB of device memory")
    ang = _u3_layer(n, n)
    u = _single_qubit_columns(ang)
    idx = _indices(n, count=1024)
    want = _product_amplitudes(u, n, idx)
    layer = [gates.U3(q, *ang[q]) for q in range(n)]
    bw = _brickwork(n, 2, n)
    b, st = _run(n, dtype, layer + bw + _inverse(bw))
    err = np.max(np.abs(_gather(st, idx) - want))
    assert err < TOL[dtype], f"n={n} {dtype}: {err}"
    del st, b
    gc.collect()
