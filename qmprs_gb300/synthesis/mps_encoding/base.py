"""Encoder plugin boundary (reference ``qmprs/synthesis/mps_encoding/base.py:32-130``)."""

from __future__ import annotations

from abc import ABC, abstractmethod

from ...ket import Ket
from ...primitives import MPS


class MPSEncoder(ABC):
    """Abstract MPS encoder; ``circuit_framework`` is the circuit class to emit into.

    ``prepare_state`` mirrors the reference step by step (``base.py:96-106``):
    wrap in ``Ket``, change indexing, optional compression, build the ``MPS``
    with the requested bond dimension, dispatch to ``prepare_mps``.
    """

    def __init__(self, circuit_framework) -> None:
        self.circuit_framework = circuit_framework

    def prepare_state(self, statevector, bond_dimension: int, compression_percentage: float = 0.0,
                      index_type: str = "row", **kwargs):
        if not isinstance(statevector, Ket):
            statevector = Ket(statevector)
        statevector.change_indexing(index_type)
        if compression_percentage > 0.0:
            statevector.compress(compression_percentage)
        mps = MPS(statevector, bond_dimension=bond_dimension)
        return self.prepare_mps(mps, **kwargs)

    @abstractmethod
    def prepare_mps(self, mps: MPS, **kwargs):
        """Prepare the quantum state held by ``mps``; returns a circuit."""
