"""qmprs_gb300: the MPS-encoding path of Qualition/qmprs on NVIDIA GB300.

Public API (same names as the reference package):

    from qmprs_gb300.primitives import MPS
    from qmprs_gb300.synthesis.mps_encoding import MPSEncoder, Sequential
    from qmprs_gb300.circuit import Circuit

All numerical work runs in the in-tree CUDA library
``qmprs_gb300/_lib/libqmprs_gb300.so`` (build: ``python -m qmprs_gb300.build``).
"""

__version__ = "0.1.0"

from .ket import Ket  # noqa: F401
from .circuit import Circuit  # noqa: F401
