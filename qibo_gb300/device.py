"""Device runtime: the GPU, its stream, device buffers and state vectors.

A ``DeviceState`` owns a device buffer of ``2**nqubits`` complex amplitudes
(complex128: 16 B, complex64: 8 B) laid out exactly like the reference's
numpy state vector (index bit ``n-1-q`` is qubit ``q``).  It quacks like a
1-D numpy array where qibo's result objects need it (``shape``, ``dtype``,
``__array__``, ``tolist``), and is copied to the host only when asked.  A
``DeviceDensity`` is a density matrix stored the same way as the 2n-qubit
vector of its row-major entries.
"""

from __future__ import annotations

import ctypes as C
import threading
import weakref

import numpy as np

from . import _lib
from ._lib import check

_DTYPES = {"complex128": (_lib.QGB_C128, 16), "complex64": (_lib.QGB_C64, 8)}


def dtype_code(dtype) -> int:
    name = np.dtype(dtype).name
    if name not in _DTYPES:
        raise TypeError(f"qibo_gb300 states are complex64 or complex128, not {name}")
    return _DTYPES[name][0]


class Runtime:
    """Process-wide device context: device id, SM count, stream, scratch."""

    _instance = None
    _lock = threading.Lock()

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        sms = C.c_int(0)
        check(self.lib.qgb_device_init(device, C.byref(sms)))
        self.device = device
        self.sm_count = sms.value
        self.stream = None  # cudaStream_t handle (int) or None for the legacy default stream
        self._scratch = None
        self._scratch_bytes = 0

    @classmethod
    def get(cls) -> "Runtime":
        with cls._lock:
            if cls._instance is None:
                cls._instance = Runtime()
            return cls._instance

    # -- memory ---------------------------------------------------------
    def malloc(self, nbytes: int) -> int:
        p = C.c_void_p()
        check(self.lib.qgb_malloc(C.byref(p), int(nbytes)))
        return p.value or 0

    def free(self, ptr: int):
        if ptr:
            self.lib.qgb_free(C.c_void_p(ptr))

    def scratch(self, nbytes: int) -> int:
        """A grow-only scratch buffer shared by stream-ordered calls."""
        if nbytes <= 0:
            return 0
        if nbytes > self._scratch_bytes:
            if self._scratch:
                self.synchronize()
                self.free(self._scratch)
                self._scratch = None
            self._scratch = self.malloc(nbytes)
            self._scratch_bytes = nbytes
        return self._scratch

    def synchronize(self):
        """Wait for the stream, then raise ``DeviceTimeout`` if a tensor-core
        kernel gave up one of its bounded waits since the last check (its
        output is invalid)."""
        check(self.lib.qgb_stream_sync(self.stream))
        self.check_waits()

    def check_waits(self):
        flag = C.c_int(0)
        check(self.lib.qgb_tc_status(C.byref(flag)))
        if flag.value:
            raise _lib.DeviceTimeout(_lib.QGB_ERR_TIMEOUT, "a tensor-core kernel gave up waiting for its MMAs or "
                                     "copies (bounded wait); the state it wrote is invalid")

    def mem_info(self):
        f, t = C.c_size_t(), C.c_size_t()
        check(self.lib.qgb_mem_info(C.byref(f), C.byref(t)))
        return f.value, t.value

    def h2d(self, dst: int, arr: np.ndarray):
        arr = np.ascontiguousarray(arr)
        check(self.lib.qgb_memcpy_h2d(dst, arr.ctypes.data, arr.nbytes, self.stream))
        self.synchronize()  # the host array may be released after return

    def d2h(self, arr: np.ndarray, src: int):
        check(self.lib.qgb_memcpy_d2h(arr.ctypes.data, src, arr.nbytes, self.stream))
        self.synchronize()


class DeviceArray:
    """A plain device array (e.g. FP64 probabilities, int64 counts)."""

    def __init__(self, shape, dtype, rt: Runtime | None = None, ptr: int | None = None, owner=None):
        self.rt = rt or Runtime.get()
        self.shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self._owner = owner
        if ptr is None:
            self.ptr = self.rt.malloc(max(self.nbytes, 1))
            self._fin = weakref.finalize(self, self.rt.free, self.ptr)
        else:
            self.ptr = ptr
            self._fin = None

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def size(self):
        return int(np.prod(self.shape))

    def __len__(self):
        return self.shape[0]

    def to_numpy(self) -> np.ndarray:
        out = np.empty(self.shape, dtype=self.dtype)
        if self.nbytes:
            self.rt.d2h(out, self.ptr)
        return out

    def __array__(self, dtype=None, copy=None):
        a = self.to_numpy()
        return a if dtype is None else a.astype(dtype)

    def tolist(self):
        return self.to_numpy().tolist()

    def __getitem__(self, item):
        return self.to_numpy()[item]

    def take(self, indices) -> np.ndarray:
        """Elements at ``indices`` of the flat array, read with one small
        copy each (a few amplitudes of a state too large to copy whole)."""
        idx = np.asarray(indices, dtype=np.int64).ravel()
        if idx.size and (idx.min() < 0 or idx.max() >= self.size):
            raise IndexError(f"index out of range for {self.size} elements")
        out = np.empty(idx.size, dtype=self.dtype)
        item = self.dtype.itemsize
        for k, i in enumerate(idx):
            check(self.rt.lib.qgb_memcpy_d2h(out.ctypes.data + k * item, self.ptr + int(i) * item, item,
                                             self.rt.stream))
        self.rt.synchronize()
        return out

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype.name})"

    def free(self):
        if self._fin is not None:
            self._fin()


class DeviceState(DeviceArray):
    """State vector of ``nqubits`` qubits resident in device memory."""

    def __init__(self, nqubits: int, dtype="complex128", rt: Runtime | None = None, ptr: int | None = None):
        self.nqubits = int(nqubits)
        self.code = dtype_code(dtype)
        super().__init__((2**self.nqubits,), dtype, rt, ptr)

    # -- creation ---------------------------------------------------------
    @classmethod
    def zero(cls, nqubits: int, dtype="complex128") -> "DeviceState":
        st = cls(nqubits, dtype)
        check(st.rt.lib.qgb_state_zero(st.ptr, st.nqubits, st.code, st.rt.stream))
        return st

    @classmethod
    def from_numpy(cls, arr, dtype=None) -> "DeviceState":
        arr = np.asarray(arr)
        if arr.ndim != 1 or arr.shape[0] & (arr.shape[0] - 1) or arr.shape[0] < 2:
            raise ValueError(f"a state vector has shape (2**n,), got {arr.shape}")
        dtype = np.dtype(dtype or (arr.dtype if arr.dtype in (np.complex64, np.complex128) else np.complex128))
        n = int(arr.shape[0]).bit_length() - 1
        st = cls(n, dtype)
        st.rt.h2d(st.ptr, arr.astype(dtype, copy=False))
        return st

    def copy(self) -> "DeviceState":
        out = DeviceState(self.nqubits, self.dtype, self.rt)
        check(self.rt.lib.qgb_memcpy_d2d(out.ptr, self.ptr, self.nbytes, self.rt.stream))
        return out

    def astype(self, dtype, copy: bool = True) -> "DeviceState":
        dtype = np.dtype(dtype)
        if dtype == self.dtype:
            return self.copy() if copy else self
        out = DeviceState(self.nqubits, dtype, self.rt)
        check(self.rt.lib.qgb_state_cast(self.ptr, self.code, out.ptr, out.code, self.nqubits, self.rt.stream))
        return out

    # -- arithmetic with real scalars and same-shape states (new arrays), as
    #    the reference's channel code combines states (gates/channels.py:702-706)
    def __mul__(self, c):
        if np.iscomplexobj(c) and np.imag(c) != 0:
            return NotImplemented
        if not np.isscalar(c) and np.ndim(c) != 0:
            return NotImplemented
        out = self.copy()
        check(self.rt.lib.qgb_state_scale(out.ptr, out.nqubits, out.code, float(np.real(c)), self.rt.stream))
        return out

    __rmul__ = __mul__

    def __neg__(self):
        return self * -1.0

    def _combine(self, other, a: float):
        if not isinstance(other, DeviceState) or other.nqubits != self.nqubits or other.shape != self.shape:
            return NotImplemented
        out = self.copy()
        if other.code != out.code:
            other = other.astype(out.dtype)
        check(self.rt.lib.qgb_state_axpby(out.ptr, other.ptr, out.nqubits, out.code, a, 1.0, self.rt.stream))
        return out

    def __add__(self, other):
        return self._combine(other, 1.0)

    def __sub__(self, other):
        return self._combine(other, -1.0)

    def __repr__(self):
        return f"DeviceState(nqubits={self.nqubits}, dtype={self.dtype.name})"


class DeviceDensity(DeviceState):
    """Density matrix of ``nsys`` qubits resident in device memory: the
    (2^n, 2^n) matrix in row-major order, i.e. the 2n-qubit vector
    v[i 2^n + j] = rho[i, j] (the reference's ``rho.ravel()``,
    backends/abstract.py:2234-2241).  ``nqubits`` is the vector's 2n (what
    the state-vector entry points take); ``shape`` is the matrix's, so qibo's
    results see a density matrix (result.py:46)."""

    def __init__(self, nsys: int, dtype="complex128", rt: Runtime | None = None, ptr: int | None = None):
        self.nsys = int(nsys)
        self.nqubits = 2 * self.nsys
        self.code = dtype_code(dtype)
        DeviceArray.__init__(self, (2**self.nsys, 2**self.nsys), dtype, rt, ptr)

    @classmethod
    def zero(cls, nsys: int, dtype="complex128") -> "DeviceDensity":
        """|0...0><0...0|: the 2n-qubit basis vector 0."""
        rho = cls(nsys, dtype)
        check(rho.rt.lib.qgb_state_zero(rho.ptr, rho.nqubits, rho.code, rho.rt.stream))
        return rho

    @classmethod
    def from_numpy(cls, arr, dtype=None) -> "DeviceDensity":
        arr = np.asarray(arr)
        d = arr.shape[0] if arr.ndim == 2 else 0
        if arr.ndim != 2 or arr.shape[1] != d or d < 2 or d & (d - 1):
            raise ValueError(f"a density matrix has shape (2**n, 2**n), got {arr.shape}")
        dtype = np.dtype(dtype or (arr.dtype if arr.dtype in (np.complex64, np.complex128) else np.complex128))
        rho = cls(d.bit_length() - 1, dtype)
        rho.rt.h2d(rho.ptr, np.ascontiguousarray(arr, dtype=dtype))
        return rho

    def copy(self) -> "DeviceDensity":
        out = DeviceDensity(self.nsys, self.dtype, self.rt)
        check(self.rt.lib.qgb_memcpy_d2d(out.ptr, self.ptr, self.nbytes, self.rt.stream))
        return out

    def astype(self, dtype, copy: bool = True) -> "DeviceDensity":
        dtype = np.dtype(dtype)
        if dtype == self.dtype:
            return self.copy() if copy else self
        out = DeviceDensity(self.nsys, dtype, self.rt)
        check(self.rt.lib.qgb_state_cast(self.ptr, self.code, out.ptr, out.code, self.nqubits, self.rt.stream))
        return out

    def __repr__(self):
        return f"DeviceDensity(nqubits={self.nsys}, dtype={self.dtype.name})"
