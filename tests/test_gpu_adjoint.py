"""Adjoint-method gradients on the GPU against the reference's parameter-shift
golden values, the reference test KAT, and finite differences.

Tolerances: complex128 gradients match exact parameter shift to 1e-9 and
FP64 central finite differences (h=1e-4, truncation ~1e-8) to 1e-6;
complex64 gradients match complex128 ones to 5e-4.
"""

import json
import os

import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def backend():
    from qibo_gb300.backend import GB300Backend

    return GB300Backend("complex128")


def circuit_of(n, ops):
    from qibo_gb300 import Circuit, gates

    c = Circuit(n)
    for op in ops:
        g = getattr(gates, op[0])(*op[1], *op[2])
        if len(op) > 3 and op[3]:
            g = g.controlled_by(*op[3])
        c.add(g)
    return c


def vqe_circuit(n, layers, params):
    return circuit_of(n, ref.vqe_ops(n, layers, params))


def test_vqe4_matches_reference_parameter_shift(backend):
    data = np.load(os.path.join(ROOT, "tests", "golden", "reference_vectors.npz"))
    from qibo_gb300.adjoint import adjoint_gradient

    p = data["vqe4_params"]
    c = vqe_circuit(4, 2, p)
    e, g = adjoint_gradient(backend, c, ref.tfim_terms(4))
    assert abs(e - float(data["vqe4_energy"])) < 1e-12
    np.testing.assert_allclose(g, data["vqe4_psr_grads"], atol=1e-9)


@pytest.mark.parametrize("scale, kat", [(1.0, [-8.51104358e-02, -5.20075970e-01, 0.0]),
                                         (0.5, [-0.02405061, -0.13560379, 0.0])])
def test_reference_derivative_kat(backend, scale, kat):
    """tests/test_derivative.py:28-31 (observable Z0, RX-RY-RZ on one qubit)."""
    from qibo_gb300.adjoint import adjoint_gradient

    p = np.linspace(0.1, 1, 3) * scale
    c = circuit_of(1, [("RX", (0,), (p[0],)), ("RY", (0,), (p[1],)), ("RZ", (0,), (p[2],))])
    _, g = adjoint_gradient(backend, c, (["Z"], [(0,)], [1.0]))
    np.testing.assert_allclose(g * scale, kat, atol=1e-8)


def _fd_oracle(n, build, params, ham, h=1e-5):
    terms, qubits, coefs = ham
    out = np.zeros(len(params))
    for i in range(len(params)):
        a, b = params.copy(), params.copy()
        a[i] += h
        b[i] -= h
        ea = ref.exp_value_observable_symbolic(ref.execute(build(a), n), terms, qubits, coefs, n)
        eb = ref.exp_value_observable_symbolic(ref.execute(build(b), n), terms, qubits, coefs, n)
        out[i] = (ea - eb) / (2 * h)
    return out


def test_general_parametrised_gates_vs_finite_differences(backend):
    """U3 (3 parameters), CU1, CRY, RZZ, fSim and controlled_by rotations."""
    from qibo_gb300.adjoint import adjoint_gradient

    n = 6
    rng = np.random.default_rng(8)

    def build(x):
        it = iter(x)
        ops = []
        for q in range(n):
            ops.append(("U3", (q,), (next(it), next(it), next(it))))
        ops += [("CNOT", (0, 1), ()), ("CU1", (2, 3), (next(it),)), ("CRY", (4, 1), (next(it),)),
                ("RZZ", (5, 0), (next(it),)), ("fSim", (3, 4), (next(it), next(it))),
                ("RX", (2,), (next(it),), (0, 5)), ("H", (3,), ()), ("RY", (1,), (next(it),))]
        return ops

    npar = 3 * n + 7
    p = rng.uniform(-np.pi, np.pi, npar)
    ham = (["ZZ", "X", "Y", "XZ", "YY", ""], [(0, 1), (2,), (3,), (4, 5), (1, 3), ()], [0.7, -1.1, 0.4, 0.9, 0.3, 0.25])
    c = circuit_of(n, build(p))
    flat = [x for t in c.get_parameters() for x in t]
    np.testing.assert_allclose(flat, p)
    e, g = adjoint_gradient(backend, c, ham)
    want_e = ref.exp_value_observable_symbolic(ref.execute(build(p), n), *ham, n)
    assert abs(e - want_e) < 1e-12
    np.testing.assert_allclose(g, _fd_oracle(n, build, p, ham), atol=1e-7)


def test_vqe_n10_vs_parameter_shift_oracle(backend):
    from qibo_gb300.adjoint import adjoint_gradient

    n, layers = 10, 3
    p = np.random.default_rng(3).uniform(-np.pi, np.pi, 2 * n * layers)
    ham = ref.tfim_terms(n)
    _, g = adjoint_gradient(backend, vqe_circuit(n, layers, p), ham)
    want = ref.parameter_shift_grad(lambda x: ref.vqe_ops(n, layers, x), n, p, *ham)
    np.testing.assert_allclose(g, want, atol=1e-9)


def test_complex64_gradients_close_to_complex128(backend):
    from qibo_gb300.adjoint import adjoint_gradient
    from qibo_gb300.backend import GB300Backend

    n, layers = 12, 4
    p = np.random.default_rng(5).uniform(-np.pi, np.pi, 2 * n * layers)
    ham = ref.tfim_terms(n)
    e128, g128 = adjoint_gradient(backend, vqe_circuit(n, layers, p), ham)
    e64, g64 = adjoint_gradient(GB300Backend("complex64"), vqe_circuit(n, layers, p), ham)
    assert abs(e64 - e128) < 5e-4
    np.testing.assert_allclose(g64, g128, atol=5e-4)


def test_torch_autograd_surface(backend):
    torch = pytest.importorskip("torch")
    from qibo_gb300.adjoint import adjoint_gradient, expectation

    n, layers = 6, 2
    p0 = np.random.default_rng(11).uniform(-np.pi, np.pi, 2 * n * layers)
    c = vqe_circuit(n, layers, p0)
    ham = ref.tfim_terms(n)
    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    e = expectation(params, c, ham, backend)
    e.backward()
    e_ref, g_ref = adjoint_gradient(backend, vqe_circuit(n, layers, p0), ham)
    assert abs(float(e.detach()) - e_ref) < 1e-12
    np.testing.assert_allclose(params.grad.numpy(), g_ref, atol=1e-12)


def test_vqe24_480_parameters_vs_gpu_finite_differences(backend):
    """Config: 24 qubits, 10 layers of RY+RZ and a CNOT ladder (480
    parameters), periodic TFIM h=1; gradients checked on a sample of
    parameters against FP64 central differences (h=1e-4) run on the GPU."""
    from qibo_gb300.adjoint import adjoint_gradient, energy

    n, layers = 24, 10
    p = np.random.default_rng(24).uniform(-np.pi, np.pi, 2 * n * layers)
    ham = ref.tfim_terms(n)
    e, g = adjoint_gradient(backend, vqe_circuit(n, layers, p), ham)
    assert g.shape == (480,)
    h = 1e-4
    for i in (0, 1, 47, 200, 333, 479):
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        ea = energy(backend, vqe_circuit(n, layers, a), ham)
        eb = energy(backend, vqe_circuit(n, layers, b), ham)
        assert abs(g[i] - (ea - eb) / (2 * h)) < 1e-6, i
    assert abs(e - energy(backend, vqe_circuit(n, layers, p), ham)) < 1e-10
