import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def reference_src():
    """The reference qibo source tree, for the CPU tests that import qibo:
    the directory in QIBO_REFERENCE_SRC, else ``reference/src`` beside this
    repository; None when neither exists (those tests then skip)."""
    for cand in (os.environ.get("QIBO_REFERENCE_SRC"), os.path.join(os.path.dirname(ROOT), "reference", "src")):
        if cand and os.path.isdir(os.path.join(cand, "qibo")):
            return cand
    return None


def import_reference():
    """qibo imported from reference_src() with the import shims of
    tests/golden/make_golden.py, or None."""
    import importlib.util

    src = reference_src()
    if src is None:
        return None
    if "qibo" in sys.modules:
        return sys.modules["qibo"]
    gold = os.path.join(ROOT, "tests", "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", gold)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg._import_reference(src)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
