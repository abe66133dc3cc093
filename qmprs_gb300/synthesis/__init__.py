"""Synthesis entry points (reference ``qmprs/synthesis/__init__.py:15-17``)."""

from . import mps_encoding

__all__ = ["mps_encoding"]
