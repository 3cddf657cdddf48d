"""Observable helpers over the C-ABI."""

from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import check
from .device import DeviceArray, DeviceDensity


def dense_expectation(engine, hamiltonian, state, normalize: bool) -> float:
    """Backend.expectation_value (backends/abstract.py:2807-2825) on the device:
    Re <psi|H|psi> for a dense Hermitian matrix H (uploaded once per call),
    divided by <psi|psi> when ``normalize``."""
    h = np.ascontiguousarray(np.asarray(getattr(hamiltonian, "matrix", hamiltonian), dtype=np.complex128))
    if isinstance(state, DeviceDensity):
        return _density_expectation(engine, h, state, normalize)
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


def _density_expectation(engine, h: np.ndarray, rho, normalize: bool) -> float:
    """Re Tr(H rho) (backends/abstract.py:2810-2816) for Hermitian H: the
    inner product <H|rho> of the two matrices flattened, sum_ij
    conj(H_ij) rho_ij = sum_ij H_ji rho_ij, on the device (H uploaded in
    complex128); divided by the real trace when ``normalize``."""
    n = rho.nsys
    if h.shape != (2**n, 2**n):
        raise ValueError(f"observable of shape {h.shape} for a {n}-qubit density matrix")
    rt = engine.rt
    dh = DeviceArray(h.shape, np.complex128, rt)
    rt.h2d(dh.ptr, h)
    out = DeviceArray((2,), np.float64, rt)
    scratch = rt.scratch(engine.lib.qgb_inner_scratch_bytes())
    check(engine.lib.qgb_inner_mixed(dh.ptr, _lib.QGB_C128, rho.ptr, rho.code, rho.nqubits, out.ptr, scratch,
                                     rt.stream))
    ev = float(out.to_numpy()[0])
    if normalize:
        ev /= engine.density_trace(rho)
    return ev
