"""Adjoint-method energies and gradients, and their PyTorch autograd surface.

``adjoint_gradient`` returns E = <psi(theta)|H|psi(theta)> and dE/dtheta for
every trainable parameter of a circuit (in ``circuit.get_parameters()``
order) from one forward run and one reverse sweep on the device
(``qgb_adjoint_sweep``), where the reference needs two full circuit runs per
parameter (parameter shift, derivative.py:7-156).

H is a Pauli sum given as ``(terms, term_qubits, coefficients)`` — the form
``SymbolicHamiltonian.simple_terms`` produces (hamiltonians/hamiltonians.py:
413-426) — or any object with those three attributes via
``terms_of_hamiltonian``.

Derivative matrices dU/dtheta come from the gate's own matrix function with
a fourth-order central stencil (step 1e-3, truncation ~1e-13), so any
parametrised gate on one or two qubits is supported without a table of
generators.
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check
from .device import DeviceArray, DeviceState
from .engine import Engine, pauli_masks

_STENCIL_H = 1e-3


def _set_params(gate, values):
    gate.parameters = tuple(float(v) for v in values)


def derivative_matrices(gate, backend) -> list:
    """dU/dtheta_j for each parameter j of ``gate`` (matrix order as
    ``gate.matrix``)."""
    p0 = tuple(float(x) for x in gate.parameters)
    out = []
    h = _STENCIL_H
    try:
        for j in range(len(p0)):
            mats = []
            for s in (2, 1, -1, -2):
                p = list(p0)
                p[j] += s * h
                _set_params(gate, p)
                mats.append(np.asarray(gate.matrix(backend), dtype=np.complex128))
            out.append((-mats[0] + 8 * mats[1] - 8 * mats[2] + mats[3]) / (12 * h))
    finally:
        _set_params(gate, p0)
    return out


def terms_of_hamiltonian(ham) -> Tuple[list, list, list]:
    """(terms, qubits, coefficients) of a qibo ``SymbolicHamiltonian`` —
    ``simple_terms`` is (coefficients, names, qubits) and ``constant`` the
    identity part (hamiltonians/hamiltonians.py:385-426) — or of a triple
    already in that form."""
    if isinstance(ham, (tuple, list)) and len(ham) == 3:
        return list(ham[0]), [tuple(q) for q in ham[1]], [float(np.real(c)) for c in ham[2]]
    coefs, names, qubits = ham.simple_terms
    terms = list(names)
    qubits = [tuple(q) for q in qubits]
    coefs = [float(np.real(c)) for c in coefs]
    const = float(np.real(getattr(ham, "constant", 0.0)))
    if const:
        terms.append("")
        qubits.append(())
        coefs.append(const)
    return terms, qubits, coefs


def _masks(terms, qubits, coefs):
    """X/Z bit masks; an empty string is the identity term."""
    xs, zs, cs = [], [], []
    for t, q, c in zip(terms, qubits, coefs):
        x, z = pauli_masks(t, q)
        xs.append(x)
        zs.append(z)
        cs.append(float(np.real(c)))
    return xs, zs, cs


def _trainable_slots(circuit):
    """id(gate) -> (first flat index, count) in get_parameters() order."""
    slots = {}
    k = 0
    for g in circuit.associate_gates_with_parameters():
        gid = id(g)
        if gid in slots:
            slots[gid] = (slots[gid][0], slots[gid][1] + 1)
        else:
            slots[gid] = (k, 1)
        k += 1
    return slots, k


def adjoint_gradient(backend, circuit, hamiltonian, initial_state=None):
    """(energy, gradients) of <psi|H|psi> for ``circuit`` run on ``backend``."""
    from .backend import describe_gate

    eng: Engine = backend.engine_gb
    rt = eng.rt
    terms, qubits, coefs = terms_of_hamiltonian(hamiltonian)
    xs, zs, cs = _masks(terms, qubits, coefs)
    if len(cs) > 256:
        raise NotImplementedError("adjoint gradients support Pauli sums of up to 256 terms")
    init = None
    if initial_state is not None:
        init = initial_state.copy() if isinstance(initial_state, DeviceState) else initial_state
    res = backend.execute_circuit(circuit, init)
    psi = res.state()
    if not isinstance(psi, DeviceState):
        psi = DeviceState.from_numpy(np.asarray(psi))
    n = psi.nqubits
    lam = DeviceState(n, psi.dtype, rt)
    nt = len(cs)
    xm = (C.c_uint64 * max(1, nt))(*xs)
    zm = (C.c_uint64 * max(1, nt))(*zs)
    cf = _lib.double_array(cs)
    if nt:
        check(rt.lib.qgb_apply_pauli_sum(psi.ptr, lam.ptr, n, psi.code, xm, zm, cf, nt, rt.stream))
    else:
        check(rt.lib.qgb_memset_zero(lam.ptr, lam.nbytes, rt.stream))
    out = DeviceArray((2,), np.float64, rt)
    check(rt.lib.qgb_inner(psi.ptr, lam.ptr, n, psi.code, out.ptr, rt.scratch(rt.lib.qgb_inner_scratch_bytes()),
                           rt.stream))
    energy = float(out.to_numpy()[0])

    slots, nparams = _trainable_slots(circuit)
    descs, nder, der_off, gidx, mats = [], [], [], [], []
    off = 0
    for gate in reversed(circuit.queue):
        d = describe_gate(gate, backend)
        if d is None:
            continue
        q, ctrl, m = d
        udag = np.ascontiguousarray(m.conj().T)
        descs.append((q, ctrl, udag))
        off += udag.size * 2
        slot = slots.get(id(gate))
        if slot is None:
            nder.append(0)
            der_off.append(0)
            gidx.append(0)
            continue
        ders = derivative_matrices(gate, backend)
        if len(ders) != slot[1]:
            raise ValueError(f"gate {gate} has {len(ders)} parameters but {slot[1]} trainable slots")
        nder.append(len(ders))
        gidx.append(slot[0])
        der_off.append(-1)  # filled after packing
        mats.append((len(descs) - 1, ders))
    ops, allc = Engine.pack_ops(descs)
    extra = []
    base = allc.size
    for i, ders in mats:
        der_off[i] = base + sum(e.size for e in extra)
        for dm in ders:
            extra.append(np.ascontiguousarray(dm, dtype=np.complex128).view(np.float64).ravel())
    coefs_all = np.concatenate([allc] + extra) if extra else allc
    grads = DeviceArray((max(1, nparams),), np.float64, rt)
    nd = _lib.int_array(nder)
    do = (C.c_int64 * max(1, len(der_off)))(*der_off)
    gi = _lib.int_array(gidx)
    scratch = rt.scratch(rt.lib.qgb_adjoint_scratch_bytes(nparams))
    check(rt.lib.qgb_adjoint_sweep(psi.ptr, lam.ptr, n, psi.code, ops, len(descs),
                                   coefs_all.ctypes.data_as(_lib.dp), nd, do, gi, nparams, grads.ptr, scratch,
                                   rt.stream))
    g = grads.to_numpy()[:nparams]
    return energy, g


def energy(backend, circuit, hamiltonian, initial_state=None) -> float:
    """<psi|H|psi> of the circuit's final state (one forward run, one
    expectation pass per distinct X/Y pattern)."""
    terms, qubits, coefs = terms_of_hamiltonian(hamiltonian)
    xs, zs, cs = _masks(terms, qubits, coefs)
    res = backend.execute_circuit(circuit, initial_state)
    st = res.state()
    return backend.engine_gb.expect_pauli(st, xs, zs, cs)


def expectation(params, circuit, hamiltonian, backend=None):
    """E(params) as a differentiable ``torch`` scalar: the forward pass runs
    the circuit on the GB300, the backward pass is the adjoint sweep."""
    import torch

    if backend is None:
        from . import get_backend

        backend = get_backend()
    return _Energy.apply(params, circuit, hamiltonian, backend)


def _make_function():
    import torch

    class Energy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, circuit, hamiltonian, backend):
            p = params.detach().cpu().double().numpy()
            circuit.set_parameters(p)
            e, g = adjoint_gradient(backend, circuit, hamiltonian)
            ctx.save_for_backward(torch.as_tensor(g, dtype=params.dtype))
            return torch.tensor(e, dtype=params.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None

    return Energy


class _Lazy:
    fn = None

    def apply(self, *args):
        if _Lazy.fn is None:
            _Lazy.fn = _make_function()
        return _Lazy.fn.apply(*args)


_Energy = _Lazy()
