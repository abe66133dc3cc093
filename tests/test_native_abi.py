"""The CUDA library builds for sm_103a, loads, and exports the C ABI.

No compute call is made here (no GPU is needed to load the library).
"""

import ctypes
import re
from pathlib import Path

from qmprs_gb300 import _native
from qmprs_gb300 import build as qb

HEADER = Path(__file__).resolve().parents[1] / "include" / "qmprs_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(qmprs_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["qmprs_create", "qmprs_plan_create", "qmprs_mps_from_statevector", "qmprs_unitary_layers",
              "qmprs_optimize_layers", "qmprs_circuit_state", "qmprs_overlap"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    lib_path = qb.build_cuda()
    lib = ctypes.CDLL(str(lib_path))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    assert set(declared_functions()) == set(_native.SIGNATURES)


def test_version_call_needs_no_gpu():
    lib = _native.load()
    assert lib.qmprs_version() >= 100


def _declared_arg_counts():
    """Argument count of every declaration in the header."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"\b(qmprs_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_binding_argument_counts_match_header():
    """The ctypes signature table passes exactly the arguments the header
    declares for every entry point (a mismatch would shift pointers)."""
    declared = _declared_arg_counts()
    assert set(declared) == set(_native.SIGNATURES)
    for name, (_, argtypes) in _native.SIGNATURES.items():
        assert len(argtypes) == declared[name], (name, len(argtypes), declared[name])
