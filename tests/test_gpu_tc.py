"""Tensor-core fused 5-qubit blocks (tcgen05) against the FP64 oracle.

Tolerances: complex64 (3xTF32, FP32 accumulation) reproduces FP32 arithmetic,
so one block matches the FP64 product to 2e-6 max-abs on a normalised state.
complex128 (Ozaki scheme on BF16: 47-bit fixed point per tile and gate row,
exact level accumulators) is bounded by 2^(E + F - 41) per output, with 2^E
<= 2 x the largest |amplitude| and 2^F <= 2 x the largest |matrix entry|;
the tests check that bound and 1e-13 absolute on normalised states, and
1e-12 (the complex128 bar) on deep fused circuits.  The kernels' timeout
flag must stay clear."""

import ctypes as C

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu


def _unitary(seed):
    from scipy.stats import unitary_group

    return unitary_group.rvs(32, random_state=seed)


def _apply_tc(psi, qubits, u, dtype=np.complex64):
    from qibo_gb300 import _lib
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceState, Runtime

    rt = Runtime.get()
    n = int(len(psi)).bit_length() - 1
    st = DeviceState.from_numpy(psi.astype(dtype))
    m = np.ascontiguousarray(u, dtype=np.complex128).view(np.float64).ravel()
    check(rt.lib.qgb_apply_fused5_tc(st.ptr, n, st.code, _lib.int_array(qubits), m.ctypes.data_as(_lib.dp), rt.stream))
    out = np.asarray(st)
    flag = C.c_int(-1)
    check(rt.lib.qgb_tc_status(C.byref(flag)))
    assert flag.value == 0, "tensor-core launch timed out"
    return out


@pytest.mark.parametrize("n,qubits", [(7, (2, 3, 4, 5, 6)), (10, (0, 1, 2, 3, 4)), (12, (11, 3, 7, 0, 5)),
                                      (14, (9, 10, 11, 12, 13)), (16, (1, 15, 8, 4, 12)),
                                      # A in tensor memory: no block qubit on index bits 0..4, then
                                      # strided lanes (index bits 0, 2 / 3, 4 in the block)
                                      (12, (0, 1, 2, 3, 4)), (13, (7, 0, 2, 5, 6)), (16, (10, 0, 3, 6, 9)),
                                      (20, (14, 2, 13, 7, 11)), (15, (14, 12, 7, 3, 0)), (18, (14, 13, 2, 9, 5)),
                                      # shared-memory A on a full tile: index bits 0 and 1 in the block
                                      (14, (13, 12, 5, 2, 0))])
def test_fused5_tc_matches_oracle(n, qubits):
    rng = np.random.default_rng(n)
    psi = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    psi /= np.linalg.norm(psi)
    psi = psi.astype(np.complex64).astype(np.complex128)
    u = _unitary(n)
    got = _apply_tc(psi, qubits, u)
    want = ref.apply_gate(psi, u, list(qubits), n)
    assert np.max(np.abs(got - want)) < 2e-6


@pytest.mark.parametrize("mode", ["smem", "tmem-strided", "tmem-shfl"])
def test_fused5_tc_every_kernel_every_placement(mode):
    """Full tiles in each complex64 block kernel and lane layout
    (QIBO_GB300_TC64_KERNEL), on placements with 0-5 block qubits on index
    bits 0..4, against the FP64 oracle."""
    import os

    placements = [(12, (0, 1, 2, 3, 4)), (12, (11, 10, 9, 8, 7)), (13, (12, 4, 9, 1, 6)), (14, (13, 12, 5, 2, 0)),
                  (14, (9, 10, 11, 12, 13)), (15, (14, 12, 7, 3, 0)), (16, (15, 14, 13, 12, 4)),
                  (16, (1, 15, 8, 4, 12)), (17, (16, 15, 14, 13, 2)), (18, (14, 13, 2, 9, 5))]
    os.environ["QIBO_GB300_TC64_KERNEL"] = mode
    try:
        for n, qubits in placements:
            rng = np.random.default_rng(n + sum(qubits))
            psi = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
            psi /= np.linalg.norm(psi)
            psi = psi.astype(np.complex64).astype(np.complex128)
            u = _unitary(n + 3)
            got = _apply_tc(psi, qubits, u)
            want = ref.apply_gate(psi, u, list(qubits), n)
            assert np.max(np.abs(got - want)) < 2e-6, (mode, n, qubits)
    finally:
        del os.environ["QIBO_GB300_TC64_KERNEL"]


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


def _rand_state(n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    return psi / np.linalg.norm(psi)


def _oz_bound(psi, u):
    return 4 * np.max(np.abs(psi)) * np.max(np.abs(u)) * 2.0**-41


@pytest.mark.parametrize("n,qubits", [(12, (11, 3, 7, 0, 5)), (12, (0, 1, 2, 3, 4)), (13, (12, 11, 10, 9, 8)),
                                      (16, (1, 15, 8, 4, 12)), (16, (2, 0, 14, 3, 9)), (17, (16, 13, 0, 7, 12))])
def test_fused5_oz_complex128_matches_oracle(n, qubits):
    psi = _rand_state(n, 100 + n)
    u = _unitary(200 + n)
    got = _apply_tc(psi, qubits, u, np.complex128)
    want = ref.apply_gate(psi, u, list(qubits), n)
    err = np.max(np.abs(got - want))
    assert err < _oz_bound(psi, u) and err < 1e-13, err


def test_fused5_oz_complex128_wide_range_and_zeros():
    """Amplitudes over 2^-60..1 in one state, plus all-zero tiles."""
    n = 14
    rng = np.random.default_rng(9)
    psi = (rng.normal(size=2**n) + 1j * rng.normal(size=2**n)) * 2.0 ** -rng.integers(0, 60, size=2**n)
    psi[: 2**12] = 0  # whole tiles of zeros
    u = _unitary(31)
    got = _apply_tc(psi, (13, 2, 6, 9, 0), u, np.complex128)
    want = ref.apply_gate(psi, u, [13, 2, 6, 9, 0], n)
    assert np.max(np.abs(got - want)) < _oz_bound(psi, u)


def test_fused5_oz_deep_fused_circuit():
    """A depth-30 brickwork + QFT, fused into 5-qubit blocks, in complex128
    through the blocked engine (tensor-core blocks + passes) against the FP64
    oracle at the complex128 bar."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend

    n = 16
    ops = ref.brickwork_ops(n, 30, 5) + ref.qft_ops(n)
    c = Circuit(n)
    for nm, q, p in ops:
        c.add(getattr(gates, nm)(*q, *p))
    fused = c.fuse(5)
    assert sum(1 for g in fused.queue if len(g.qubits) == 5) >= 20
    psi = _rand_state(n, 77)
    b = GB300Backend("complex128")
    b.blocked = True
    got = np.asarray(b.execute_circuit(fused, psi.copy()).state())
    want = ref.execute(ops, n, psi)
    assert np.max(np.abs(got - want)) < 1e-12
    flag = C.c_int(-1)
    check_status = b.rt.lib.qgb_tc_status(C.byref(flag))
    assert check_status == 0 and flag.value == 0


def test_fused5_oz_needs_twelve_qubits():
    from qibo_gb300 import _lib
    from qibo_gb300.device import DeviceState, Runtime

    rt = Runtime.get()
    st = DeviceState.from_numpy(_rand_state(11, 1))
    m = np.ascontiguousarray(_unitary(3), dtype=np.complex128).view(np.float64).ravel()
    with pytest.raises(NotImplementedError):
        _lib.check(rt.lib.qgb_apply_fused5_tc(st.ptr, 11, st.code, _lib.int_array((0, 1, 2, 3, 4)),
                                              m.ctypes.data_as(_lib.dp), rt.stream))


@pytest.mark.parametrize("scale_last", [1.0, 0.5])
def test_oz_chain_unnormalised_state(scale_last):
    """Three blocks through qgb_apply_circuit on a complex128 state of norm
    7.3.  All unitary: one fixed-point chain whose scale comes from the
    state's norm.  Last block scaled by 0.5 (not unitary): the run goes
    through the IEEE-double block path instead.  Both against the FP64
    oracle, 1e-12 relative to the norm."""
    from qibo_gb300.backend import GB300Backend
    from qibo_gb300.device import DeviceState

    n = 13
    psi = _rand_state(n, 5) * 7.3
    blocks = [((0, 4, 9, 12, 2), _unitary(41)), ((3, 7, 1, 11, 6), _unitary(42)),
              ((12, 10, 8, 5, 0), _unitary(43) * scale_last)]
    b = GB300Backend("complex128")
    st = DeviceState.from_numpy(psi)
    b.engine_gb.apply_many(st, [(q, [], u) for q, u in blocks], blocked=True)
    got = np.asarray(st)
    want = psi
    for q, u in blocks:
        want = ref.apply_gate(want, u, list(q), n)
    assert np.max(np.abs(got - want)) < 1e-12 * 7.3


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
def test_engine_fusion_matches_oracle(dtype, tol):
    """The backend's default path for n >= 12: the engine fuses the gate
    list (qgb_fuse5) and runs its 5-qubit blocks on the tensor cores; a
    depth-20 brickwork plus QFT (controlled phases and swaps) against the
    FP64 oracle."""
    from qibo_gb300 import Circuit, gates
    from qibo_gb300.backend import GB300Backend, describe_gate

    n = 16
    ops = ref.brickwork_ops(n, 20, 8) + ref.qft_ops(n)
    c = Circuit(n)
    for nm, q, p in ops:
        c.add(getattr(gates, nm)(*q, *p))
    b = GB300Backend(dtype)
    assert b.fuse
    nops, n5 = b.engine_gb.fuse_stats([describe_gate(g, b) for g in c.queue])
    assert n5 >= 20 and nops < len(ops) // 5
    psi = _rand_state(n, 3)
    got = np.asarray(b.execute_circuit(c, psi.copy()).state())
    want = ref.execute(ops, n, psi)
    assert np.max(np.abs(got - want)) < tol
