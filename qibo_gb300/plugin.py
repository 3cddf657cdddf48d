"""qibo plugin: ``qibo.set_backend("qibo_gb300")`` (or ``"qibo-gb300"``).

qibo resolves a non-native backend name by importing the module
``name.replace("-", "_")`` and calling its ``MetaBackend.load(**kwargs)``
(backends/__init__.py:325-350); ``list_available_backends`` calls
``MetaBackend().list_available()`` (:312-322).  When qibo is installed the
loaded object is ``QiboGB300Backend``, a subclass of qibo's own
``NumpyBackend`` whose state-vector hot path runs on the GB300, so qibo's
``Circuit(...)(nshots=...)``, results, Hamiltonians and derivative helpers
work unchanged.
"""

from __future__ import annotations

_CLASS = None


def qibo_backend_class():
    """Build (once) the qibo-derived backend class; needs qibo importable."""
    global _CLASS
    if _CLASS is not None:
        return _CLASS
    from qibo.backends.numpy import NumpyBackend
    from qibo.result import CircuitResult, MeasurementOutcomes, QuantumState

    from .backend import GB300Methods
    from .device import DeviceArray

    class QiboGB300Backend(GB300Methods, NumpyBackend):
        def __init__(self, dtype="complex128"):
            NumpyBackend.__init__(self)
            self.name = "qibo_gb300"
            self.set_dtype(dtype)
            self._gb300_init(dtype)
            self.tensor_types = (self.engine.ndarray, DeviceArray)
            self.versions[self.name] = "1.0"

        def set_device(self, device):
            if not device.startswith("/GPU"):
                raise ValueError(f"Device {device} is not available for {self} backend.")

        def set_threads(self, nthreads):
            self.nthreads = int(nthreads)

        def _result_classes(self):
            return QuantumState, CircuitResult

        def _outcomes_class(self):
            return MeasurementOutcomes

    _CLASS = QiboGB300Backend
    return _CLASS
