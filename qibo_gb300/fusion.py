"""Gate fusion into blocks of at most ``max_qubits`` qubits.

The reference's ``Circuit.fuse`` (models/circuit.py:954-1003, with
``FusedGate.fuse``, gates/special.py:106-153) merges neighbouring gates
pairwise and stops as soon as both sides of a candidate have blocking
neighbours, so on brickwork circuits it yields almost only 2-qubit blocks.
This packer grows each block by a forward scan over the not-yet-placed gates
in circuit order instead:

* a block starts from the earliest unplaced gate;
* a later gate joins the block when every earlier unplaced gate that shares
  a qubit with it has joined too (so moving it forward only crosses gates on
  disjoint qubits, with which it commutes) and the block's qubit set stays
  within ``max_qubits``;
* a gate that cannot join "blocks" its qubits for the rest of the scan.

The output keeps qibo's form: a list of ``FusedGate`` objects whose
``target_qubits`` are sorted (gates/special.py:38); single-gate blocks are
returned as the original gate, as ``_Queue.from_fused`` does
(models/circuit.py:75-94).  Gates that must stay alone (measurements,
gates wider than ``max_qubits``) are emitted unfused in order.
"""

from __future__ import annotations

from typing import Callable, List, Sequence


def gate_qubit_set(g) -> frozenset:
    return frozenset(getattr(g, "qubits", ()))


def pack(gates: Sequence, max_qubits: int, fusable: Callable[[object], bool] = lambda g: True,
         seed_qubits: Sequence[int] = ()) -> List[List[int]]:
    """Group gate indices into blocks.  Returns blocks as lists of indices in
    an execution order equivalent to the input order.

    ``seed_qubits`` pre-populates every block's qubit set (used by the
    shared-memory planner to keep the low-order index bits resident)."""
    n = len(gates)
    qsets = [gate_qubit_set(g) for g in gates]
    placed = [False] * n
    blocks: List[List[int]] = []
    first = 0
    seed = frozenset(seed_qubits)
    while first < n:
        while first < n and placed[first]:
            first += 1
        if first >= n:
            break
        start = first
        if not fusable(gates[start]) or len(qsets[start] | seed) > max_qubits:
            placed[start] = True
            blocks.append([start])
            continue
        members = [start]
        placed[start] = True
        qs = set(qsets[start]) | set(seed)
        blocked = set()
        for i in range(start + 1, n):
            if placed[i]:
                continue
            gq = qsets[i]
            if gq & blocked:
                blocked |= gq
                continue
            if fusable(gates[i]) and len(qs | gq) <= max_qubits:
                members.append(i)
                placed[i] = True
                qs |= gq
            else:
                blocked |= gq
            if len(qs) >= max_qubits and qs <= blocked:
                break  # no later gate can join: every block qubit is blocked
        blocks.append(members)
    return blocks


def fuse_gates(gates: Sequence, max_qubits: int, fused_cls, is_special: Callable[[object], bool]):
    """Return a qibo-style queue: ``fused_cls`` blocks plus unfusable gates."""
    blocks = pack(gates, max_qubits, fusable=lambda g: not is_special(g))
    queue = []
    for b in blocks:
        if len(b) == 1:
            queue.append(gates[b[0]])
            continue
        qs = sorted(set().union(*(gate_qubit_set(gates[i]) for i in b)))
        fg = fused_cls(*qs)
        for i in b:
            fg.append(gates[i])
        queue.append(fg)
    return queue
