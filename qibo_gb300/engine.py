"""Thin host-side driver of the C-ABI: gates, probabilities, sampling and
expectations on ``DeviceState`` objects.

Gate descriptors are ``(qubits, controls, matrix)``: ``qubits`` in matrix
order (``qubits[0]`` is the most significant matrix-index bit, the order of
the reference's ``gate.qubits``), ``controls`` the ``controlled_by`` qubits
(the matrix then acts on ``qubits`` only where all controls are 1,
backends/abstract.py:3176-3197), ``matrix`` a complex 2^k x 2^k array.
"""

from __future__ import annotations

import ctypes as C
from typing import Iterable, List, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import QgbOp, check, double_array, int_array
from .device import DeviceArray, DeviceDensity, DeviceState, Runtime

GateDesc = Tuple[Sequence[int], Sequence[int], np.ndarray]


def _matrix_doubles(m) -> np.ndarray:
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    return m.view(np.float64).ravel()


class Engine:
    def __init__(self, rt: Runtime | None = None):
        self.rt = rt or Runtime.get()
        self.lib = self.rt.lib

    # -- gates -----------------------------------------------------------
    def apply(self, state: DeviceState, qubits: Sequence[int], matrix, controls: Sequence[int] = ()):
        qubits, controls = list(qubits), list(controls)
        m = _matrix_doubles(matrix)
        if m.size != 2 * 4 ** len(qubits):
            raise ValueError(f"matrix of {m.size // 2} entries for {len(qubits)} qubits")
        check(self.lib.qgb_apply_gate(state.ptr, state.nqubits, state.code, int_array(qubits), len(qubits),
                                      int_array(controls), len(controls),
                                      m.ctypes.data_as(_lib.dp), self.rt.stream))

    def apply_many(self, state: DeviceState, descs: Iterable[GateDesc], blocked: bool = False,
                   strict_fp64: bool = False, fuse: bool = False):
        """Apply a gate list with one C call (``qgb_apply_circuit``).

        ``blocked`` plans shared-memory passes (many gates per read+write of
        the state); complex128 passes then compute in double-float unless
        ``strict_fp64``.  ``fuse`` (with ``blocked``) first fuses the list into
        blocks of at most 5 qubits, whose uncontrolled 5-qubit blocks run on
        the tensor cores."""
        descs = list(descs)
        if not descs:
            return
        ops, allc = self.pack_ops(descs)
        flags = (_lib.QGB_PLAN_BLOCKED if blocked else 0) | (_lib.QGB_PLAN_STRICT_FP64 if strict_fp64 else 0)
        if blocked and fuse:
            flags |= _lib.QGB_PLAN_FUSE
        check(self.lib.qgb_apply_circuit(state.ptr, state.nqubits, state.code, ops, len(descs),
                                         allc.ctypes.data_as(_lib.dp), flags, self.rt.stream))

    def fuse_stats(self, descs: Iterable[GateDesc], pad_nqubits: int = 0):
        """(ops after engine fusion, uncontrolled 5-qubit blocks among them);
        ``pad_nqubits``: the state's size when the engine widens blocks to 5
        qubits (tensor cores in use, 12 qubits or more)."""
        descs = list(descs)
        if not descs:
            return 0, 0
        ops, allc = self.pack_ops(descs)
        a, b = C.c_int(0), C.c_int(0)
        check(self.lib.qgb_fuse_stats(ops, len(descs), allc.ctypes.data_as(_lib.dp), pad_nqubits, C.byref(a),
                                      C.byref(b)))
        return a.value, b.value

    def count_passes(self, nqubits: int, dtype_code: int, descs: Iterable[GateDesc]) -> int:
        """State passes the shared-memory planner makes for this gate list."""
        descs = list(descs)
        if not descs:
            return 0
        ops, allc = self.pack_ops(descs)
        n = C.c_int(0)
        check(self.lib.qgb_plan_passes(nqubits, dtype_code, ops, len(descs), allc.ctypes.data_as(_lib.dp),
                                       C.byref(n)))
        return n.value

    @staticmethod
    def pack_ops(descs: List[GateDesc]):
        """``qgb_op`` records plus the concatenated matrix coefficients."""
        ops = (QgbOp * len(descs))()
        coefs: List[np.ndarray] = []
        off = 0
        for i, (qubits, controls, matrix) in enumerate(descs):
            qubits, controls = list(qubits), list(controls)
            if len(qubits) > 5 or len(controls) > 8:
                raise NotImplementedError(f"gate on {len(qubits)} qubits with {len(controls)} controls")
            m = _matrix_doubles(matrix)
            if m.size != 2 * 4 ** len(qubits):
                raise ValueError(f"matrix of {m.size // 2} entries for {len(qubits)} qubits")
            op = ops[i]
            op.k = len(qubits)
            op.ncontrols = len(controls)
            for j, q in enumerate(qubits):
                op.qubits[j] = q
            for j, q in enumerate(controls):
                op.controls[j] = q
            op.coef_offset = off
            coefs.append(m)
            off += m.size
        return ops, np.concatenate(coefs)

    # -- reductions -------------------------------------------------------
    def probabilities(self, state: DeviceState, qubits: Sequence[int]) -> DeviceArray:
        """Marginal probabilities (FP64, device) of ``qubits`` in that order."""
        qubits = list(qubits)
        out = DeviceArray((2 ** len(qubits),), np.float64, self.rt)
        nbytes = self.lib.qgb_probs_scratch_bytes(state.nqubits, len(qubits))
        scratch = self.rt.scratch(nbytes)
        check(self.lib.qgb_probabilities(state.ptr, state.nqubits, state.code, int_array(qubits), len(qubits),
                                         out.ptr, scratch or None, self.rt.stream))
        return out

    def norm2(self, state: DeviceState) -> float:
        out = DeviceArray((1,), np.float64, self.rt)
        scratch = self.rt.scratch(self.lib.qgb_norm_scratch_bytes())
        check(self.lib.qgb_norm2(state.ptr, state.nqubits, state.code, out.ptr, scratch, self.rt.stream))
        return float(out.to_numpy()[0])

    def renormalize(self, state: DeviceState) -> float:
        """Scale the state to unit norm; the norm is accumulated in FP64.
        Returns the norm before scaling."""
        nrm = self.norm2(state) ** 0.5
        if nrm > 0 and abs(nrm - 1.0) > 0:
            self.scale(state, 1.0 / nrm)
        return nrm

    def scale(self, state: DeviceState, factor: float):
        check(self.lib.qgb_state_scale(state.ptr, state.nqubits, state.code, float(factor), self.rt.stream))

    def sample(self, probs: DeviceArray, nshots: int, seed: int, counts: bool = True) -> np.ndarray:
        """Draw ``nshots`` outcomes from device FP64 ``probs`` (length 2^m).

        Returns host int64 counts (length 2^m) or samples (length nshots)."""
        m = int(probs.shape[0]).bit_length() - 1
        if 2**m != probs.shape[0]:
            raise ValueError("probability vector length must be a power of two")
        scratch = self.rt.scratch(self.lib.qgb_sample_scratch_bytes(m))
        if counts:
            out = DeviceArray((2**m,), np.int64, self.rt)
            check(self.lib.qgb_memset_zero(out.ptr, out.nbytes, self.rt.stream))
            check(self.lib.qgb_sample(probs.ptr, m, int(nshots), int(seed) & (2**64 - 1), None, out.ptr,
                                      scratch, self.rt.stream))
        else:
            out = DeviceArray((int(nshots),), np.int64, self.rt)
            check(self.lib.qgb_sample(probs.ptr, m, int(nshots), int(seed) & (2**64 - 1), out.ptr, None,
                                      scratch, self.rt.stream))
        return out.to_numpy()

    def sample_device(self, probs: DeviceArray, nshots: int, seed: int) -> DeviceArray:
        """``nshots`` outcome indices drawn from device FP64 ``probs`` (length
        2^m), left on the device (int64)."""
        m = int(probs.shape[0]).bit_length() - 1
        if 2**m != probs.shape[0]:
            raise ValueError("probability vector length must be a power of two")
        scratch = self.rt.scratch(self.lib.qgb_sample_scratch_bytes(m))
        out = DeviceArray((max(1, int(nshots)),), np.int64, self.rt)
        check(self.lib.qgb_sample(probs.ptr, m, int(nshots), int(seed) & (2**64 - 1), out.ptr, None, scratch,
                                  self.rt.stream))
        return out

    def parity_means(self, samples: DeviceArray, nshots: int, masks: Sequence[int]) -> np.ndarray:
        """Per mask, the mean over the shots of (-1)^(number of 1 bits of the
        outcome under the mask), from integer parity counts on the device."""
        masks = [int(m) for m in masks]
        out = np.ones(len(masks), dtype=np.float64)
        if nshots <= 0:
            return out
        for lo in range(0, len(masks), _lib.QGB_PARITY_MAX_TERMS):
            chunk = masks[lo:lo + _lib.QGB_PARITY_MAX_TERMS]
            odd = DeviceArray((len(chunk),), np.int64, self.rt)
            mp = (C.c_uint64 * len(chunk))(*chunk)
            check(self.lib.qgb_parity_counts(samples.ptr, int(nshots), mp, len(chunk), odd.ptr, self.rt.stream))
            out[lo:lo + len(chunk)] = (nshots - 2 * odd.to_numpy()) / nshots
        return out

    def collapse(self, state: DeviceState, qubits: Sequence[int], outcome, normalize: bool = True):
        """Project ``state`` in place onto ``outcome`` of measuring ``qubits``
        (``qubits[0]`` the most significant outcome bit); ``outcome`` is an
        int or a device int64 array whose first element is the outcome."""
        qubits = list(qubits)
        outcome = self._outcome_array(outcome, len(qubits))
        scratch = self.rt.scratch(self.lib.qgb_norm_scratch_bytes())
        check(self.lib.qgb_collapse(state.ptr, state.nqubits, state.code, int_array(qubits), len(qubits),
                                    outcome.ptr, int(bool(normalize)), scratch, self.rt.stream))

    def _outcome_array(self, outcome, nq: int) -> DeviceArray:
        if isinstance(outcome, DeviceArray):
            return outcome
        k = int(outcome)
        if not 0 <= k < 2**nq:
            raise ValueError(f"outcome {k} outside the {2 ** nq} outcomes of {nq} qubits")
        dev = DeviceArray((1,), np.int64, self.rt)
        self.rt.h2d(dev.ptr, np.array([k], dtype=np.int64))
        return dev

    # -- density matrices --------------------------------------------------
    def density_probabilities(self, rho: DeviceDensity, qubits: Sequence[int]) -> DeviceArray:
        """Marginal probabilities (FP64, device) of ``qubits`` (in that
        order) from the diagonal of ``rho``."""
        qubits = list(qubits)
        out = DeviceArray((2 ** len(qubits),), np.float64, self.rt)
        scratch = self.rt.scratch(self.lib.qgb_density_scratch_bytes())
        check(self.lib.qgb_density_probabilities(rho.ptr, rho.nsys, rho.code, int_array(qubits), len(qubits),
                                                 out.ptr, scratch, self.rt.stream))
        return out

    def density_trace(self, rho: DeviceDensity) -> float:
        return float(self.density_probabilities(rho, []).to_numpy()[0])

    def density_collapse(self, rho: DeviceDensity, qubits: Sequence[int], outcome, normalize: bool = True):
        """Project rows and columns of ``rho`` onto ``outcome`` of ``qubits``
        (int or device int64 array), divided by the kept trace."""
        qubits = list(qubits)
        dev = self._outcome_array(outcome, len(qubits))
        scratch = self.rt.scratch(self.lib.qgb_density_scratch_bytes())
        check(self.lib.qgb_density_collapse(rho.ptr, rho.nsys, rho.code, int_array(qubits), len(qubits), dev.ptr,
                                            int(bool(normalize)), scratch, self.rt.stream))

    def density_expect_pauli(self, rho: DeviceDensity, xmask: Sequence[int], zmask: Sequence[int],
                             coef: Sequence[float]) -> float:
        """sum_t coef[t] Re Tr(P_t rho), P_t given by qubit bit masks."""
        n = len(coef)
        xm = (C.c_uint64 * max(1, n))(*[int(x) for x in xmask])
        zm = (C.c_uint64 * max(1, n))(*[int(z) for z in zmask])
        out = DeviceArray((1,), np.float64, self.rt)
        scratch = self.rt.scratch(self.lib.qgb_density_scratch_bytes())
        check(self.lib.qgb_density_expect_pauli(rho.ptr, rho.nsys, rho.code, xm, zm, double_array(coef), n, out.ptr,
                                                scratch, self.rt.stream))
        return float(out.to_numpy()[0])

    def axpby(self, y: DeviceState, x: DeviceState, a: float, b: float):
        """y = a x + b y (same size and precision)."""
        if y.nqubits != x.nqubits or y.code != x.code:
            raise ValueError("axpby needs arrays of the same size and precision")
        check(self.lib.qgb_state_axpby(y.ptr, x.ptr, y.nqubits, y.code, float(a), float(b), self.rt.stream))

    def expect_pauli(self, state: DeviceState, xmask: Sequence[int], zmask: Sequence[int],
                     coef: Sequence[float]) -> float:
        """sum_t coef[t] <psi|P_t|psi>, P_t given by qubit bit masks (bit q = qubit q)."""
        n = len(coef)
        xm = (C.c_uint64 * max(1, n))(*[int(x) for x in xmask])
        zm = (C.c_uint64 * max(1, n))(*[int(z) for z in zmask])
        cf = double_array(coef)
        out = DeviceArray((1,), np.float64, self.rt)
        scratch = self.rt.scratch(self.lib.qgb_expect_scratch_bytes(state.nqubits, n))
        check(self.lib.qgb_expect_pauli(state.ptr, state.nqubits, state.code, xm, zm, cf, n, out.ptr, scratch,
                                        self.rt.stream))
        return float(out.to_numpy()[0])


def pauli_masks(term: str, qubits: Sequence[int]) -> Tuple[int, int]:
    """(xmask, zmask) of a Pauli string such as ``"XZY"`` on ``qubits``."""
    x = z = 0
    for f, q in zip(term, qubits):
        if f in ("X", "Y"):
            x |= 1 << q
        if f in ("Z", "Y"):
            z |= 1 << q
        if f not in ("X", "Y", "Z", "I"):
            raise ValueError(f"unknown Pauli factor {f!r}")
    return x, z
