"""Statevector wrapper with the behaviour the encoder relies on from quick-core.

The reference wraps inputs in ``quick.primitives.Ket`` (used at
``qmprs/synthesis/mps_encoding/base.py:96-102`` and
``qmprs/primitives/mps.py:170-171,270``).  quick-core is not a dependency
here; this class restates what the path needs: complex128 data padded with
zeros to a power-of-two length, L2-normalised, ``num_qubits``,
``change_indexing`` and ``compress``.
"""

from __future__ import annotations

import numpy as np


class Ket:
    def __init__(self, data, normalize: bool = True) -> None:
        rows = None
        if isinstance(data, Ket):
            rows = data.rows
            data = data.data
        arr = np.asarray(data, dtype=np.complex128)
        if arr.ndim == 2:
            rows = arr.shape[0]      # an image: snake indexing walks its rows
        v = arr.reshape(-1)
        if v.size == 0:
            raise ValueError("a statevector needs at least one amplitude")
        n = max(1, int(np.ceil(np.log2(v.size))))
        if v.size < 2 ** n:
            v = np.concatenate([v, np.zeros(2 ** n - v.size, dtype=np.complex128)])
        if normalize:
            nrm = np.linalg.norm(v)
            if nrm == 0 or not np.isfinite(nrm):
                raise ValueError("The statevector must have a finite, non-zero norm.")
            if not np.isclose(nrm, 1.0):
                v = v / nrm
        self.data = v
        self.num_qubits = n
        # rows of the 2-D view used by snake indexing (the input's own rows
        # for a 2-D array whose size is a power of two)
        self.rows = rows if rows and v.size % rows == 0 and arr.size == v.size else 2 ** ((n + 1) // 2)

    def change_indexing(self, index_type: str) -> None:
        """``"row"`` keeps the amplitude order; ``"snake"`` reverses every odd
        row of the amplitudes viewed as an image: the input's own rows for a
        2-D input, else 2^ceil(n/2) x 2^floor(n/2)."""
        if index_type == "row":
            return
        if index_type == "snake":
            img = self.data.reshape(self.rows, -1).copy()
            img[1::2] = img[1::2, ::-1]
            self.data = img.reshape(-1)
            return
        raise ValueError(f"`index_type` must be 'row' or 'snake'. Received {index_type}.")

    def compress(self, compression_percentage: float) -> None:
        """Zero the given percentage of smallest-magnitude amplitudes, renormalise."""
        if not (0.0 <= compression_percentage <= 100.0):
            raise ValueError("compression percentage must be within [0, 100]")
        k = int(np.floor(self.data.size * compression_percentage / 100.0))
        if k > 0:
            order = np.argsort(np.abs(self.data), kind="stable")
            self.data = self.data.copy()
            self.data[order[:k]] = 0.0
            nrm = np.linalg.norm(self.data)
            if nrm > 0:
                self.data /= nrm

    def __eq__(self, other: object) -> bool:
        if not isinstance(other, Ket):
            return NotImplemented
        return self.data.shape == other.data.shape and bool(np.allclose(self.data, other.data))

    def __repr__(self) -> str:
        return f"Ket(num_qubits={self.num_qubits})"
