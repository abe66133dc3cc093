"""Minimal circuit backend with the protocol the encoder emits into.

The reference injects a ``quick.circuit.Circuit`` subclass
(``qmprs/synthesis/mps_encoding/base.py:50-56``, used at
``qmprs/synthesis/mps_encoding/sequential.py:208``) and calls only
``circuit_framework(num_qubits)`` and ``circuit.unitary(matrix, qubits)``;
its tests read ``get_statevector()`` and ``get_depth()``.  quick-core is not
available here, so this module provides a small class with that protocol;
any class with the same methods (a real quick circuit) can be passed as
``circuit_framework`` instead.

Conventions follow quick/qiskit: qubit 0 is the least significant bit of the
statevector index, and in ``unitary(U, [a, b])`` qubit ``a`` is the least
significant bit of U's row index.

``get_depth()`` reports the depth after a basis translation to one-qubit
gates and CX: each two-qubit unitary costs the minimal number of CX given by
the Shende-Bullock-Markov invariant (0 local, 1, 2 or 3; "Recognizing
small-circuit structure in two-qubit operators", Phys. Rev. A 70, 012310),
interleaved with one-qubit layers, and consecutive one-qubit gates on a wire
merge.  ``get_unitary_depth()`` is the depth counting each unitary as one
operation.
"""

from __future__ import annotations

import numpy as np

_SY = np.array([[0, -1j], [1j, 0]])
_SYY = np.kron(_SY, _SY)


def cx_count(u: np.ndarray, tol: float = 1e-5) -> int:
    """Minimal number of CX gates needed for a 4x4 unitary."""
    u = np.asarray(u, dtype=np.complex128)
    det = np.linalg.det(u)
    u = u / det ** 0.25
    gamma = u @ _SYY @ u.T @ _SYY
    tr = np.trace(gamma)
    eye = np.eye(4)
    if np.allclose(gamma, eye, atol=tol) or np.allclose(gamma, -eye, atol=tol):
        return 0
    if abs(tr) < tol and np.allclose(gamma @ gamma, -eye, atol=tol):
        return 1
    if abs(tr.imag) < tol:
        return 2
    return 3


class Circuit:
    """A list of unitary gates on ``num_qubits`` qubits (little-endian)."""

    def __init__(self, num_qubits: int) -> None:
        if not isinstance(num_qubits, (int, np.integer)) or num_qubits < 1:
            raise ValueError("num_qubits must be a positive integer")
        self.num_qubits = int(num_qubits)
        self.gates: list[tuple[np.ndarray, list[int]]] = []

    def unitary(self, unitary_matrix, qubit_indices) -> None:
        qs = [int(qubit_indices)] if np.isscalar(qubit_indices) else [int(q) for q in qubit_indices]
        u = np.asarray(unitary_matrix, dtype=np.complex128)
        if u.shape != (2 ** len(qs), 2 ** len(qs)):
            raise ValueError(f"unitary of shape {u.shape} does not act on {len(qs)} qubit(s)")
        if any(q < 0 or q >= self.num_qubits for q in qs) or len(set(qs)) != len(qs):
            raise ValueError(f"invalid qubit indices {qs}")
        self.gates.append((u, qs))

    def get_statevector(self) -> np.ndarray:
        n = self.num_qubits
        psi = np.zeros(2 ** n, dtype=np.complex128)
        psi[0] = 1.0
        for u, qs in self.gates:
            k = len(qs)
            # axes of psi reshaped to [2]*n are MSB first: qubit q is axis n-1-q
            t = psi.reshape([2] * n)
            axes = [n - 1 - q for q in reversed(qs)]          # U's MSB is the last listed qubit
            t = np.moveaxis(t, axes, list(range(k)))
            shp = t.shape
            t = (u @ t.reshape(2 ** k, -1)).reshape(shp)
            t = np.moveaxis(t, list(range(k)), axes)
            psi = t.reshape(-1)
        return psi

    def count_ops(self) -> dict:
        ops = {"U3": 0, "CX": 0}
        for u, qs in self.gates:
            if len(qs) == 1:
                ops["U3"] += 1
            else:
                k = cx_count(u)
                ops["CX"] += k
                ops["U3"] += 2 * (k + 1) if k else 2
        return ops

    def get_depth(self) -> int:
        depth = [0] * self.num_qubits
        open1q = [False] * self.num_qubits

        def one(q: int) -> None:
            if not open1q[q]:
                depth[q] += 1
                open1q[q] = True

        def cx(a: int, b: int) -> None:
            d = max(depth[a], depth[b]) + 1
            depth[a] = depth[b] = d
            open1q[a] = open1q[b] = False

        for u, qs in self.gates:
            if len(qs) == 1:
                one(qs[0])
                continue
            a, b = qs
            k = cx_count(u)
            one(a)
            one(b)
            for _ in range(k):
                cx(a, b)
                one(a)
                one(b)
        return max(depth) if depth else 0

    def get_unitary_depth(self) -> int:
        depth = [0] * self.num_qubits
        for _, qs in self.gates:
            d = max(depth[q] for q in qs) + 1
            for q in qs:
                depth[q] = d
        return max(depth) if depth else 0
