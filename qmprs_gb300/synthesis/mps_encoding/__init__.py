"""MPS encoders (reference ``qmprs/synthesis/mps_encoding/__init__.py:15-21``)."""

from .base import MPSEncoder
from .sequential import Sequential

__all__ = ["MPSEncoder", "Sequential"]
