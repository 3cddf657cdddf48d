"""Observable helpers over the C-ABI."""

from __future__ import annotations

import numpy as np

from ._lib import check
from .device import DeviceArray


def dense_expectation(engine, hamiltonian, state, normalize: bool) -> float:
    """Backend.expectation_value (backends/abstract.py:2807-2825) on the device:
    Re <psi|H|psi> for a dense Hermitian matrix H (uploaded once per call),
    divided by <psi|psi> when ``normalize``."""
    h = np.ascontiguousarray(np.asarray(getattr(hamiltonian, "matrix", hamiltonian), dtype=np.complex128))
    n = state.nqubits
    if h.shape != (2**n, 2**n):
        raise ValueError(f"observable of shape {h.shape} for a {n}-qubit state")
    rt = engine.rt
    dh = DeviceArray(h.shape, np.complex128, rt)
    rt.h2d(dh.ptr, h)
    out = DeviceArray((1,), np.float64, rt)
    scratch = rt.scratch(engine.lib.qgb_expect_scratch_bytes(n, 1))
    check(engine.lib.qgb_expect_dense(state.ptr, n, state.code, dh.ptr, out.ptr, scratch, rt.stream))
    ev = float(out.to_numpy()[0])
    if normalize:
        ev /= engine.norm2(state)
    return ev
