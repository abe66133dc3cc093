"""MPS primitive (reference ``qmprs/primitives/__init__.py:15-17``)."""

from .mps import MPS, MatrixProductState, UnitaryBlock, UnitaryLayer

__all__ = ["MPS", "MatrixProductState", "UnitaryBlock", "UnitaryLayer"]
