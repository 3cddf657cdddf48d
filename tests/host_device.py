"""Host stand-in for ``libqgb300`` (test infrastructure only).

``HostLib`` implements, on host memory, the ``qgb_*`` entry points that the
package's Python layer (``Runtime``, ``DeviceArray``/``DeviceState``,
``Engine``, the backend's direct calls) makes through ctypes.  A "device
pointer" is the address of a host numpy buffer owned here, so pointer
arithmetic and ``memmove`` copies behave as on the device.  Gates,
probabilities, collapses and expectations follow the oracle (the reference
NumpyBackend algorithms restated in ``oracle/numpy_ref.py``); shots are drawn
with numpy from the given seed.

It lets CPU tests drive qibo's own front end (``Circuit``, results,
Hamiltonians) through ``QiboGB300Backend`` without a GPU: the C-ABI calls
are the only thing replaced.  ``calls`` counts each entry point.
"""

from __future__ import annotations

import collections
import ctypes as C

import numpy as np

from oracle import numpy_ref as ref

_CDT = {0: np.complex64, 1: np.complex128}  # QGB_C64, QGB_C128


def _ival(x) -> int:
    """An integer argument: a Python int, a ctypes scalar, or None (0)."""
    if x is None:
        return 0
    return int(getattr(x, "value", x) or 0)


class HostLib:
    def __init__(self):
        self._bufs = {}
        self.calls = collections.Counter()
        self.error = b""

    # -- memory -------------------------------------------------------------
    def _alloc(self, nbytes: int) -> int:
        buf = np.zeros(max(int(nbytes), 1) + 64, dtype=np.uint8)
        addr = buf.ctypes.data
        self._bufs[addr] = buf
        return addr

    def _view(self, addr, dtype, count) -> np.ndarray:
        dtype = np.dtype(dtype)
        raw = (C.c_char * (int(count) * dtype.itemsize)).from_address(_ival(addr))
        return np.frombuffer(raw, dtype=dtype)

    def _state(self, ptr, n, code) -> np.ndarray:
        return self._view(ptr, _CDT[code], 2**n)

    def __getattr__(self, name):
        raise AttributeError(f"the host stand-in has no entry point {name}")

    # -- runtime --------------------------------------------------------------
    def qgb_last_error(self):
        return self.error

    def qgb_device_init(self, device, sms):
        sms._obj.value = 152
        return 0

    def qgb_mem_info(self, free, total):
        free._obj.value = 1 << 40
        total._obj.value = 1 << 40
        return 0

    def qgb_malloc(self, pp, nbytes):
        pp._obj.value = self._alloc(nbytes)
        return 0

    def qgb_free(self, p):
        self._bufs.pop(_ival(p), None)
        return 0

    def qgb_memcpy_h2d(self, dst, src, nbytes, stream):
        C.memmove(_ival(dst), _ival(src), int(nbytes))
        return 0

    qgb_memcpy_d2h = qgb_memcpy_h2d
    qgb_memcpy_d2d = qgb_memcpy_h2d

    def qgb_memset_zero(self, ptr, nbytes, stream):
        C.memset(_ival(ptr), 0, int(nbytes))
        return 0

    def qgb_stream_sync(self, stream):
        return 0

    timed_out = 0  # set by a test to stand for a kernel whose bounded wait gave up

    def qgb_tc_status(self, flag):
        flag._obj.value, self.timed_out = self.timed_out, 0
        return 0

    # -- states ---------------------------------------------------------------
    def qgb_state_zero(self, ptr, n, code, stream):
        self.calls["qgb_state_zero"] += 1
        st = self._state(ptr, n, code)
        st[:] = 0
        st[0] = 1
        return 0

    def qgb_state_cast(self, src, scode, dst, dcode, n, stream):
        self._state(dst, n, dcode)[:] = self._state(src, n, scode)
        return 0

    def qgb_state_scale(self, ptr, n, code, factor, stream):
        st = self._state(ptr, n, code)
        st *= factor
        return 0

    # -- gates ------------------------------------------------------------------
    def _apply(self, st, n, qubits, controls, m):
        work = st.astype(np.complex128)
        if controls:
            out = ref.apply_gate_controlled_by(work, m, list(controls), list(qubits), n)
        else:
            out = ref.apply_gate(work, m, list(qubits), n)
        st[:] = out

    def qgb_apply_gate(self, ptr, n, code, qubits, k, controls, nc, matrix, stream):
        self.calls["qgb_apply_gate"] += 1
        m = np.ctypeslib.as_array(matrix, shape=(2 * 4**k,)).view(np.complex128).reshape(2**k, 2**k)
        self._apply(self._state(ptr, n, code), n, list(qubits)[:k], list(controls)[:nc], m)
        return 0

    def qgb_apply_circuit(self, ptr, n, code, ops, nops, coefs, flags, stream):
        self.calls["qgb_apply_circuit"] += 1
        st = self._state(ptr, n, code)
        for i in range(nops):
            op = ops[i]
            k = op.k
            flat = np.ctypeslib.as_array(coefs, shape=(op.coef_offset + 2 * 4**k,))[op.coef_offset:]
            m = flat.view(np.complex128).reshape(2**k, 2**k)
            self._apply(st, n, list(op.qubits)[:k], list(op.controls)[: op.ncontrols], m)
        return 0

    # -- reductions and sampling ----------------------------------------------------
    def qgb_probs_scratch_bytes(self, n, nq):
        return 0

    def qgb_norm_scratch_bytes(self):
        return 0

    def qgb_sample_scratch_bytes(self, m):
        return 0

    def qgb_expect_scratch_bytes(self, n, nterms):
        return 0

    def qgb_probabilities(self, ptr, n, code, qubits, nq, out, scratch, stream):
        self.calls["qgb_probabilities"] += 1
        st = self._state(ptr, n, code).astype(np.complex128)
        p = ref.calculate_probabilities(st, list(qubits)[:nq], n)
        self._view(out, np.float64, 2**nq)[:] = p
        return 0

    def qgb_norm2(self, ptr, n, code, out, scratch, stream):
        st = self._state(ptr, n, code).astype(np.complex128)
        self._view(out, np.float64, 1)[0] = float(np.vdot(st, st).real)
        return 0

    def qgb_sample(self, probs, m, nshots, seed, samples, counts, scratch, stream):
        self.calls["qgb_sample"] += 1
        p = np.array(self._view(probs, np.float64, 2**m))
        draws = np.random.default_rng(_ival(seed)).choice(2**m, size=int(nshots), p=p / p.sum())
        if _ival(samples):
            self._view(samples, np.int64, int(nshots))[:] = draws
        if _ival(counts):
            self._view(counts, np.int64, 2**m)[:] += np.bincount(draws, minlength=2**m)
        return 0

    def qgb_collapse(self, ptr, n, code, qubits, nq, outcome, normalize, scratch, stream):
        self.calls["qgb_collapse"] += 1
        st = self._state(ptr, n, code)
        shot = int(self._view(outcome, np.int64, 1)[0])
        out = ref.collapse_statevector(st.astype(np.complex128), list(qubits)[:nq], shot, n, bool(normalize))
        st[:] = out
        return 0

    def qgb_expect_pauli(self, ptr, n, code, xmask, zmask, coef, nterms, out, scratch, stream):
        self.calls["qgb_expect_pauli"] += 1
        st = self._state(ptr, n, code).astype(np.complex128)
        terms, tq, cf = [], [], []
        for t in range(nterms):
            x, z = int(xmask[t]), int(zmask[t])
            qs = [q for q in range(n) if ((x | z) >> q) & 1]
            terms.append("".join("Y" if (x >> q) & (z >> q) & 1 else "X" if (x >> q) & 1 else "Z" for q in qs))
            tq.append(tuple(qs))
            cf.append(float(coef[t]))
        self._view(out, np.float64, 1)[0] = ref.exp_value_observable_symbolic(st, terms, tq, cf, n)
        return 0

    def qgb_parity_counts(self, samples, nshots, masks, nterms, odd, stream):
        self.calls["qgb_parity_counts"] += 1
        s = np.array(self._view(samples, np.int64, int(nshots)))
        o = self._view(odd, np.int64, nterms)
        for t in range(nterms):
            o[t] = int(sum(bin(int(v) & int(masks[t])).count("1") & 1 for v in s))
        return 0

    def qgb_expect_dense(self, ptr, n, code, ham, out, scratch, stream):
        self.calls["qgb_expect_dense"] += 1
        st = self._state(ptr, n, code).astype(np.complex128)
        h = np.array(self._view(ham, np.complex128, 4**n)).reshape(2**n, 2**n)
        self._view(out, np.float64, 1)[0] = float(np.vdot(st, h @ st).real)
        return 0

    # -- density matrices (the 2n-qubit vector of rho) ---------------------------
    def _rho(self, ptr, n, code) -> np.ndarray:
        return self._state(ptr, 2 * n, code).reshape(2**n, 2**n)

    def qgb_density_scratch_bytes(self):
        return 0

    def qgb_density_probabilities(self, ptr, n, code, qubits, nq, out, scratch, stream):
        self.calls["qgb_density_probabilities"] += 1
        rho = self._rho(ptr, n, code).astype(np.complex128)
        if nq == 0:
            p = [float(np.real(np.trace(rho)))]
        else:
            p = ref.calculate_probabilities_density(rho, list(qubits)[:nq], n)
        self._view(out, np.float64, 2**nq)[:] = p
        return 0

    def qgb_density_collapse(self, ptr, n, code, qubits, nq, outcome, normalize, scratch, stream):
        self.calls["qgb_density_collapse"] += 1
        rho = self._rho(ptr, n, code)
        shot = int(self._view(outcome, np.int64, 1)[0])
        rho[:] = ref.collapse_density(rho.astype(np.complex128), list(qubits)[:nq], shot, n, bool(normalize))
        return 0

    def qgb_density_expect_pauli(self, ptr, n, code, xmask, zmask, coef, nterms, out, scratch, stream):
        self.calls["qgb_density_expect_pauli"] += 1
        rho = self._rho(ptr, n, code).astype(np.complex128)
        terms, tq, cf = [], [], []
        for t in range(nterms):
            x, z = int(xmask[t]), int(zmask[t])
            qs = [q for q in range(n) if ((x | z) >> q) & 1]
            terms.append("".join("Y" if (x >> q) & (z >> q) & 1 else "X" if (x >> q) & 1 else "Z" for q in qs))
            tq.append(tuple(qs))
            cf.append(float(coef[t]))
        self._view(out, np.float64, 1)[0] = ref.exp_value_observable_symbolic_density(rho, terms, tq, cf, n)
        return 0

    def qgb_state_axpby(self, y, x, n, code, a, b, stream):
        self.calls["qgb_state_axpby"] += 1
        yv, xv = self._state(y, n, code), self._state(x, n, code)
        yv[:] = a * xv if b == 0 else a * xv + b * yv
        return 0

    def qgb_inner_scratch_bytes(self):
        return 0

    def qgb_inner_mixed(self, a, code_a, b, code_b, n, out, scratch, stream):
        v = np.vdot(self._state(a, n, code_a).astype(np.complex128), self._state(b, n, code_b).astype(np.complex128))
        self._view(out, np.float64, 2)[:] = [v.real, v.imag]
        return 0

