"""Generate golden vectors by running the reference qibo (NumpyBackend) itself.

Run in a container that holds the reference source tree::

    python tests/golden/make_golden.py /path/to/qibo/src

(or with the source directory in the environment variable
``QIBO_REFERENCE_SRC``).

The reference needs two import shims outside its tree (both written to a
temporary directory here): a ``qibo-<ver>.dist-info/METADATA`` so that
``importlib.metadata.version("qibo")`` resolves, and an empty ``openqasm3``
module (imported unconditionally by ``models/_openqasm.py``; QASM parsing is
not exercised).  The outputs are small ``.npz``/``.json`` fixtures in this
directory; the GPU tests read these fixtures and never the reference itself.
"""

from __future__ import annotations

import json
import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC_ENV = "QIBO_REFERENCE_SRC"


def _import_reference(src: str):
    shim = tempfile.mkdtemp(prefix="qibo_shim_")
    os.makedirs(os.path.join(shim, "qibo-0.3.5.dist-info"))
    with open(os.path.join(shim, "qibo-0.3.5.dist-info", "METADATA"), "w") as f:
        f.write("Metadata-Version: 2.1\nName: qibo\nVersion: 0.3.5\n")
    os.makedirs(os.path.join(shim, "openqasm3"))
    open(os.path.join(shim, "openqasm3", "__init__.py"), "w").close()
    sys.dont_write_bytecode = True
    sys.path[:0] = [src, shim]
    import qibo  # noqa: E402

    qibo.set_backend("numpy")
    return qibo


# gate catalogue exercised by the per-gate known-answer vectors:
# (name, qubits, params).  Qubit tuples follow the reference's constructor
# argument order (for controlled gates: control(s) first, then target).
GATE_CASES = [
    ("H", (0,), ()), ("H", (3,), ()), ("X", (1,), ()), ("Y", (2,), ()), ("Z", (0,), ()),
    ("S", (1,), ()), ("SDG", (3,), ()), ("T", (2,), ()), ("TDG", (0,), ()),
    ("SX", (1,), ()), ("SXDG", (2,), ()),
    ("RX", (0,), (0.1234,)), ("RY", (3,), (1.987,)), ("RZ", (1,), (-2.5,)),
    ("U1", (2,), (0.77,)), ("U2", (0,), (0.3, -1.1)), ("U3", (3,), (0.1, 0.2, 0.3)),
    ("U3", (1,), (4.1, 2.2, 5.3)),
    ("CNOT", (0, 3), ()), ("CNOT", (3, 1), ()), ("CY", (2, 0), ()), ("CZ", (1, 2), ()),
    ("CSX", (0, 2), ()), ("CRX", (3, 0), (0.4,)), ("CRY", (1, 3), (1.3,)),
    ("CRZ", (2, 1), (2.1,)), ("CU1", (3, 0), (0.9,)), ("CU2", (0, 1), (0.5, 1.5)),
    ("CU3", (2, 3), (1.0, 2.0, 3.0)),
    ("SWAP", (0, 3), ()), ("SWAP", (2, 1), ()), ("iSWAP", (1, 3), ()), ("FSWAP", (0, 2), ()),
    ("fSim", (3, 1), (0.6, 0.25)), ("RXX", (0, 1), (0.3,)), ("RYY", (2, 0), (1.7,)),
    ("RZZ", (1, 3), (2.9,)),
    ("TOFFOLI", (0, 1, 3), ()), ("TOFFOLI", (3, 2, 0), ()), ("CCZ", (1, 2, 3), ()),
]

# gate.controlled_by cases: (name, targets, params, controls)
CONTROLLED_BY_CASES = [
    ("X", (2,), (), (0, 1)),
    ("U3", (1,), (0.3, 0.4, 0.5), (3,)),
    ("RY", (0,), (0.8,), (1, 3)),
    ("SWAP", (0, 3), (), (1,)),
    ("Z", (3,), (), (0, 2)),
]


def _gate(qibo, name, qubits, params):
    cls = getattr(qibo.gates, name)
    return cls(*qubits, *params)


def main(src: str):
    qibo = _import_reference(src)
    from qibo import gates, Circuit
    from qibo.models import QFT
    from qibo.hamiltonians import TFIM
    from qibo.derivative import parameter_shift

    out = {}
    meta = {"reference": "qibo " + qibo.__version__, "generator": "tests/golden/make_golden.py"}

    # 1. per-gate known-answer vectors on a seeded random 4-qubit state
    rng = np.random.default_rng(1)
    n = 4
    psi0 = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    psi0 /= np.linalg.norm(psi0)
    out["gates_init"] = psi0
    gate_meta = []
    for i, (name, qubits, params) in enumerate(GATE_CASES):
        c = Circuit(n)
        g = _gate(qibo, name, qubits, params)
        c.add(g)
        out[f"gate_{i}"] = c(psi0.copy()).state()
        out[f"gate_{i}_matrix"] = g.matrix(qibo.get_backend())
        gate_meta.append({"name": name, "qubits": list(qubits), "params": list(params),
                          "gate_qubits": list(g.qubits)})
    ctrl_meta = []
    for i, (name, targets, params, controls) in enumerate(CONTROLLED_BY_CASES):
        c = Circuit(n)
        g = _gate(qibo, name, targets, params).controlled_by(*controls)
        c.add(g)
        out[f"ctrl_{i}"] = c(psi0.copy()).state()
        ctrl_meta.append({"name": name, "targets": list(targets), "params": list(params),
                          "controls": list(controls)})
    meta["gates"] = gate_meta
    meta["controlled_by"] = ctrl_meta

    # 2. QFT on seeded random states, plus the exact DFT check values
    for nq in (4, 5, 6, 10):
        r = np.random.default_rng(nq)
        s = r.normal(size=2**nq) + 1j * r.normal(size=2**nq)
        s /= np.linalg.norm(s)
        out[f"qft{nq}_init"] = s
        out[f"qft{nq}_final"] = QFT(nq)(s.copy()).state()

    # 3. random U3 + CZ brickwork, complex128 and complex64, plus fused
    nq, depth = 8, 6
    ang = np.random.default_rng(30).uniform(0, 2 * np.pi, (depth, nq, 3))
    c = Circuit(nq)
    for l in range(depth):
        for q in range(nq):
            c.add(gates.U3(q, *ang[l, q]))
        for q in range(l % 2, nq - 1, 2):
            c.add(gates.CZ(q, q + 1))
    out["brick8_angles"] = ang
    out["brick8_c128"] = c().state()
    out["brick8_fused5"] = c.fuse(max_qubits=5)().state()
    out["brick8_fused_nblocks"] = np.array(len(c.fuse(max_qubits=5).queue))
    qibo.set_dtype("complex64")
    out["brick8_c64"] = c().state()
    qibo.set_dtype("complex128")

    # 4. probabilities over qubit subsets in caller order (state = brick8_c128)
    st = out["brick8_c128"]
    prob_sets = [[0, 1, 2, 3, 4, 5, 6, 7], [2, 0], [7, 3, 5], [4]]
    res = qibo.result.QuantumState(st)
    for i, qs in enumerate(prob_sets):
        out[f"probs_{i}"] = res.probabilities(qs)
    meta["prob_sets"] = prob_sets

    # 5. seeded frequencies (pins the numpy MT19937 stream only) and probabilities
    c = Circuit(3)
    c.add(gates.H(0)); c.add(gates.RY(1, 0.7)); c.add(gates.CNOT(0, 2)); c.add(gates.M(0, 1, 2))
    qibo.set_backend("numpy")
    qibo.get_backend().set_seed(1234)
    r = c(nshots=100000)
    out["freq3_probs"] = np.asarray(r.probabilities())
    f = r.frequencies(binary=False)
    out["freq3_counts"] = np.array([f.get(i, 0) for i in range(8)])

    # 6. TFIM expectation on the brickwork state and on a 6-qubit state
    for nq in (6, 8):
        ham = TFIM(nq, h=1.0, dense=False)
        r = np.random.default_rng(100 + nq)
        s = r.normal(size=2**nq) + 1j * r.normal(size=2**nq)
        s /= np.linalg.norm(s)
        out[f"tfim{nq}_state"] = s
        out[f"tfim{nq}_energy"] = np.array(ham.expectation(s))

    # 7. variational ansatz energy and parameter-shift gradients (RY, RZ, CNOT ladder)
    nq, layers = 4, 2
    params = np.random.default_rng(24).uniform(-np.pi, np.pi, 2 * nq * layers)
    c = Circuit(nq)
    for _ in range(layers):
        for q in range(nq):
            c.add(gates.RY(q, 0.0)); c.add(gates.RZ(q, 0.0))
        for q in range(nq - 1):
            c.add(gates.CNOT(q, q + 1))
    c.set_parameters(params)
    ham = TFIM(nq, h=1.0, dense=False)
    out["vqe4_params"] = params
    out["vqe4_energy"] = np.array(ham.expectation(c().state()))
    grads = []
    for i in range(len(params)):
        c.set_parameters(params)
        grads.append(parameter_shift(c, ham, parameter_index=i))
    out["vqe4_psr_grads"] = np.array(grads)

    # 8. state collapse (Backend.collapse_state, ascending qubit lists as
    #    M.apply passes them) and an expectation value from frequencies
    #    (exp_value_diagonal_observable_symbolic_from_samples)
    backend = qibo.get_backend()
    st = out["brick8_c128"]
    collapse_cases = [([2], 1), ([0, 5], 2), ([1, 3, 7], 5), ([4, 6], 0)]
    for i, (qs, k) in enumerate(collapse_cases):
        out[f"collapse_{i}"] = backend.collapse_state(st.copy(), qs, np.array([k]), 8)
        out[f"collapse_{i}_unnorm"] = backend.collapse_state(st.copy(), qs, np.array([k]), 8, normalize=False)
    meta["collapse_cases"] = [[list(q), k] for q, k in collapse_cases]
    fs = {"freq": {"0110": 37, "1011": 12, "0001": 80, "1111": 5, "0100": 21}, "qubit_map": [3, 0, 5, 2],
          "terms_qubits": [[3], [0, 5], [2, 3, 0], [5, 2]], "coefs": [0.5, -1.25, 0.75, 2.0], "constant": 0.3}

    class _Frequencies:
        def frequencies(self):
            return dict(fs["freq"])

    c = Circuit(1)
    c._final_state = _Frequencies()
    out["fromsamples_value"] = np.array(backend.exp_value_diagonal_observable_symbolic_from_samples(
        c, 6, [tuple(q) for q in fs["terms_qubits"]], fs["coefs"], nshots=1, qubit_map=fs["qubit_map"],
        constant=fs["constant"]))
    meta["fromsamples"] = fs

    # 9. density matrices: gates and every channel kind, probabilities from
    #    the diagonal, Pauli-sum energy, collapse (density_cases.py)
    sys.path.insert(0, HERE)
    import density_cases as dc

    dm_meta = {}
    for name, (nq, build, seed) in dc.CASES.items():
        c = build(gates, Circuit)
        init = None if seed is None else dc.random_rho(nq, seed)
        res = c(initial_state=None if init is None else init.copy())
        final = np.asarray(res.state())
        if init is not None:
            out[f"{name}_init"] = init
        if name in dc.SAMPLED:
            idx = dc.sample_indices(nq, dc.SAMPLED[name])
            out[f"{name}_idx"] = idx
            out[f"{name}_vals"] = final.ravel()[idx]
        else:
            out[f"{name}_final"] = final
            out[f"{name}_collapse"] = backend.collapse_state(final.copy(), [1], np.array([1]), nq,
                                                             density_matrix=True)
        for i, qs in enumerate(dc.PROB_SETS[name]):
            out[f"{name}_probs_{i}"] = np.asarray(res.probabilities(qs))
        out[f"{name}_tfim"] = np.array(TFIM(nq, h=0.5, dense=False).expectation(c))
        out[f"{name}_purity"] = np.array(np.real(np.trace(final @ final)))
        dm_meta[name] = {"nqubits": nq, "ngates": len(c.queue)}
    meta["density"] = dm_meta

    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **out)
    with open(os.path.join(HERE, "reference_vectors.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(SRC_ENV)
    if not src:
        sys.exit(f"usage: make_golden.py <qibo src directory> (or set {SRC_ENV})")
    main(src)
