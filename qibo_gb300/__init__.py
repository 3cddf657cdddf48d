"""qibo_gb300: a GB300 (sm_103a) state-vector simulation backend for qibo.

Plugin entry (qibo's own surface, backends/__init__.py:325-350)::

    import qibo
    qibo.set_backend("qibo_gb300", dtype="complex128")
    qibo.models.QFT(20)(nshots=1000)

Without qibo installed, the same backend drives the qibo-compatible
``qibo_gb300.Circuit`` / ``qibo_gb300.gates`` mirror::

    from qibo_gb300 import Circuit, gates, set_backend
    c = Circuit(2); c.add(gates.H(0)); c.add(gates.CNOT(0, 1)); c.add(gates.M(0, 1))
    c(nshots=1000).frequencies()

The compute path is ``libqgb300.so`` (hand-written CUDA for sm_103a, built
in-tree by ``qibo_gb300._build``); there is no CPU fallback.
"""

from __future__ import annotations

from . import gates
from .circuit import QFT, Circuit

__version__ = "1.0.0"

_BACKEND = None


def _qibo_available() -> bool:
    try:
        import qibo  # noqa: F401

        return True
    except Exception:
        return False


class MetaBackend:
    """qibo's provider protocol: ``load(**kwargs)`` and ``list_available()``."""

    @staticmethod
    def load(platform=None, dtype="complex128", **kwargs):
        if platform not in (None, "cuda", "gb300"):
            raise ValueError(f"qibo_gb300 has no platform {platform!r} (available: 'cuda')")
        if _qibo_available():
            from .plugin import qibo_backend_class

            return qibo_backend_class()(dtype=dtype)
        from .backend import GB300Backend

        return GB300Backend(dtype=dtype)

    def list_available(self) -> dict:
        try:
            from . import _lib

            _lib.load()
            from .device import Runtime

            Runtime.get()
            ok = True
        except Exception:
            ok = False
        return {"cuda": ok}


def set_backend(backend: str = "qibo_gb300", **kwargs):
    """Select the backend used by the standalone ``Circuit`` mirror."""
    global _BACKEND
    if backend.replace("-", "_") != "qibo_gb300":
        raise ValueError(f"only the qibo_gb300 backend is available here, not {backend}")
    from .backend import GB300Backend

    _BACKEND = GB300Backend(dtype=kwargs.get("dtype", "complex128"))
    return _BACKEND


def get_backend():
    global _BACKEND
    if _BACKEND is None:
        from .backend import GB300Backend

        _BACKEND = GB300Backend()
    return _BACKEND


def set_dtype(dtype: str):
    get_backend().set_dtype(dtype)


def set_seed(seed):
    get_backend().set_seed(seed)
