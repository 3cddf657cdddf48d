"""Tensor-core fused 5-qubit blocks (tcgen05, 3xTF32) against the FP64 oracle.

Tolerance: 3xTF32 with FP32 accumulation reproduces FP32 arithmetic, so the
complex64 result of one block matches the FP64 product to 2e-6 max-abs on a
normalised state (and the kernel's own timeout flag stays clear)."""

import ctypes as C

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu


def _unitary(seed):
    from scipy.stats import unitary_group

    return unitary_group.rvs(32, random_state=seed)


def _apply_tc(psi, qubits, u):
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceState, Runtime

    rt = Runtime.get()
    n = int(len(psi)).bit_length() - 1
    st = DeviceState.from_numpy(psi.astype(np.complex64))
    m = np.ascontiguousarray(u, dtype=np.complex128).view(np.float64).ravel()
    check(rt.lib.qgb_apply_fused5_tc(st.ptr, n, _lib.int_array(qubits), m.ctypes.data_as(_lib.dp), rt.stream))
    out = np.asarray(st)
    flag = C.c_int(-1)
    check(rt.lib.qgb_tc_status(C.byref(flag)))
    assert flag.value == 0, "tensor-core launch timed out"
    return out


@pytest.mark.parametrize("n,qubits", [(7, (2, 3, 4, 5, 6)), (10, (0, 1, 2, 3, 4)), (12, (11, 3, 7, 0, 5)),
                                      (14, (9, 10, 11, 12, 13)), (16, (1, 15, 8, 4, 12))])
def test_fused5_tc_matches_oracle(n, qubits):
    rng = np.random.default_rng(n)
    psi = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    psi /= np.linalg.norm(psi)
    psi = psi.astype(np.complex64).astype(np.complex128)
    u = _unitary(n)
    got = _apply_tc(psi, qubits, u)
    want = ref.apply_gate(psi, u, list(qubits), n)
    assert np.max(np.abs(got - want)) < 2e-6


def test_fused5_tc_block_of_a_brickwork():
    """A real fused block (U3 + CZ gates packed by the fusion pass)."""
    from qibo_gb300 import Circuit, gates

    n = 12
    c = Circuit(n)
    for nm, q, p in ref.brickwork_ops(n, 6, 4):
        c.add(getattr(gates, nm)(*q, *p))
    blocks = [g for g in c.fuse(5).queue if len(g.qubits) == 5]
    assert blocks
    psi = np.zeros(2**n, dtype=np.complex128)
    psi[0] = 1
    g = blocks[0]
    got = _apply_tc(psi, g.qubits, g.matrix())
    want = ref.apply_gate(psi, g.matrix(), list(g.qubits), n)
    assert np.max(np.abs(got - want)) < 2e-6
