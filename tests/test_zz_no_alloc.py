"""The allocation-free sampling entry point (qgb_sample_noalloc).

Callers that cannot allocate device memory when they draw shots — a state
vector sized to fill the GPU, or a serving loop that must not call
cudaMalloc/cudaFree because those can synchronise the device — use
``qgb_sample_noalloc``, which keeps its CDF in a fixed array inside the
library instead of a caller scratch buffer.  This test calls it through the
C ABI and checks that it returns exactly what ``qgb_sample`` returns for the
same distribution and seed, on two calls in a row (the second call must not
see anything left over from the first), and that distributions beyond its
2^20-outcome limit are refused.  The file is named to be collected last.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_probs(rt, p):
    from qibo_gb300.device import DeviceArray

    arr = DeviceArray((len(p),), np.float64, rt)
    rt.h2d(arr.ptr, np.ascontiguousarray(p, dtype=np.float64))
    return arr


def _both(rt, probs, m, nshots, seed, counts):
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray

    size = 2**m if counts else nshots
    a = DeviceArray((size,), np.int64, rt)
    b = DeviceArray((size,), np.int64, rt)
    check(rt.lib.qgb_memset_zero(a.ptr, a.nbytes, rt.stream))
    check(rt.lib.qgb_memset_zero(b.ptr, b.nbytes, rt.stream))
    scratch = rt.scratch(rt.lib.qgb_sample_scratch_bytes(m))
    if counts:
        check(rt.lib.qgb_sample(probs.ptr, m, nshots, seed, None, a.ptr, scratch, rt.stream))
        check(rt.lib.qgb_sample_noalloc(probs.ptr, m, nshots, seed, None, b.ptr, rt.stream))
    else:
        check(rt.lib.qgb_sample(probs.ptr, m, nshots, seed, a.ptr, None, scratch, rt.stream))
        check(rt.lib.qgb_sample_noalloc(probs.ptr, m, nshots, seed, b.ptr, None, rt.stream))
    return a.to_numpy(), b.to_numpy()


def test_sample_noalloc_matches_sample_twice():
    from qibo_gb300.device import Runtime

    rt = Runtime.get()
    rng = np.random.default_rng(2024)
    # first call: a wide distribution at the size limit, samples mode
    m1 = 20
    p1 = rng.random(2**m1) ** 4
    a, b = _both(rt, _device_probs(rt, p1), m1, 300_000, 11, counts=False)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0 and a.max() < 2**m1
    # second call right after: a small, sparse distribution, counts mode
    m2 = 9
    p2 = np.zeros(2**m2)
    p2[rng.choice(2**m2, 7, replace=False)] = rng.random(7)
    a, b = _both(rt, _device_probs(rt, p2), m2, 100_000, 12, counts=True)
    np.testing.assert_array_equal(a, b)
    assert a.sum() == 100_000 and set(np.nonzero(b)[0]) <= set(np.nonzero(p2)[0])


def test_sample_noalloc_rejects_oversized_distribution():
    from qibo_gb300._lib import check
    from qibo_gb300.device import DeviceArray, Runtime

    rt = Runtime.get()
    probs = DeviceArray((2**21,), np.float64, rt)
    out = DeviceArray((16,), np.int64, rt)
    with pytest.raises(ValueError, match="exceeds the built-in scratch"):
        check(rt.lib.qgb_sample_noalloc(probs.ptr, 21, 16, 1, out.ptr, None, rt.stream))
