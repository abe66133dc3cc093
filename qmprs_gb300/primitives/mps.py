"""``MPS`` primitive with the reference's API, backed by the GPU library.

Mirrors ``qmprs.primitives.MPS`` (reference ``qmprs/primitives/mps.py:50-1138``).
The reference wraps a quimb ``MatrixProductState``; this class keeps the
state as a dense complex64 vector resident on the GPU (the representation
every GPU stage works on) and derives site tensors from it with the library's
truncated-SVD kernel when they are asked for.  Validation messages and
exception types follow the reference.

Numerical methods and the reference lines they replace:

* ``from_statevector``  ``qmprs_mps_from_statevector``     mps.py:219-249
* ``to_statevector``    ``qmprs_mps_to_statevector``       mps.py:252-270
* ``norm``/``normalize``  ``qmprs_overlap``                 mps.py:272-310
* ``canonicalize``/``compress``  truncated SVD (kernel (a)) from the
  right; "left" runs it on the qubit-reversed state     mps.py:348-459
* ``generate_bond_D_unitary_layer``  ``qmprs_unitary_layers`` with one
  layer                                                  mps.py:849-891
* ``apply_unitary_layer(s)``  ``qmprs_apply_layer``         mps.py:893-1018
* ``fidelity_with_zero_state``  amplitude 0 of the state     mps.py:1020-1039
"""

from __future__ import annotations

import copy
from typing import Literal, TypeAlias

import numpy as np
import torch

from .. import engine as _engine
from ..ket import Ket

# (start, end, [gate, ...]) and a list of those (reference mps.py:46-47)
UnitaryBlock: TypeAlias = tuple
UnitaryLayer: TypeAlias = list

_MAX_SVD_BOND = 1024   # largest bond of the GPU statevector -> MPS stage


class Tensor:
    """Site tensor holder exposing ``.data`` like a quimb Tensor."""

    def __init__(self, data: np.ndarray):
        self.data = data

    @property
    def shape(self):
        return self.data.shape


def _quimb_like(obj) -> bool:
    """A quimb ``MatrixProductState``: site ``arrays`` plus either
    ``permute_arrays`` (quimb's own method, which reorders every site's
    indices to a given order such as "lpr") or an index-order string
    ``shape`` (a permutation of "lrp")."""
    if not hasattr(obj, "arrays"):
        return False
    if callable(getattr(obj, "permute_arrays", None)):
        return True
    shape = getattr(obj, "shape", None)
    return isinstance(shape, str) and sorted(shape) == ["l", "p", "r"]


def _from_quimb(obj) -> "MatrixProductState":
    """Site arrays of a quimb MPS as (l, p, r) tensors.  A quimb object is
    copied and brought to index order "lpr" with its own
    ``permute_arrays``, so its stored order never has to be known; an
    object without that method states its order in ``shape``.  The first
    site has no l index and the last no r index (quimb's open boundary
    arrays)."""
    order = getattr(obj, "shape", None)
    if callable(getattr(obj, "permute_arrays", None)):
        obj = obj.copy() if callable(getattr(obj, "copy", None)) else obj
        obj.permute_arrays("lpr")
        order = "lpr"
    arrays = [np.asarray(a) for a in obj.arrays]
    n = len(arrays)
    out = []
    for i, a in enumerate(arrays):
        letters = order
        if n > 1 and i == 0:
            letters = letters.replace("l", "")
        if n > 1 and i == n - 1:
            letters = letters.replace("r", "")
        if n == 1:
            letters = "p"
        if a.ndim != len(letters):
            raise ValueError(f"site {i}: array of rank {a.ndim} does not match the index order {order!r}")
        want = "".join(c for c in "lpr" if c in letters)
        out.append(np.transpose(a, [letters.index(c) for c in want]))
    return MatrixProductState(out, layout="lpr")


class MatrixProductState:
    """Site tensors of an open-boundary MPS with physical dimension 2.

    ``arrays`` holds one array per site in the current index layout:
    ``"lpr"`` (left, phys, right) or ``"lrp"``; the first site has no left
    index and the last no right index, as quimb's arrays.
    """

    def __init__(self, arrays, layout: str = "lpr"):
        arrays = [np.asarray(a, dtype=np.complex128) for a in arrays]
        if len(arrays) == 0:
            raise ValueError("an MPS needs at least one tensor")
        self._t = [self._to_3d(a, i, len(arrays), layout) for i, a in enumerate(arrays)]
        self.layout = layout

    @staticmethod
    def _to_3d(a: np.ndarray, i: int, n: int, layout: str) -> np.ndarray:
        if a.ndim == 3:
            return a if layout == "lpr" else a.transpose(0, 2, 1)
        if n == 1:
            return a.reshape(1, -1, 1)
        if a.ndim == 2:
            if i == 0:
                return (a[None] if layout == "lpr" else a.T[None])      # (p, r) / (r, p)
            if i == n - 1:
                return a[:, :, None]                                     # (l, p)
        raise ValueError("site tensors must be (l, p, r) arrays or quimb-style end tensors")

    @classmethod
    def from_3d(cls, tensors) -> "MatrixProductState":
        m = cls.__new__(cls)
        m._t = [np.asarray(t, dtype=np.complex128) for t in tensors]
        m.layout = "lpr"
        return m

    @property
    def num_tensors(self) -> int:
        return len(self._t)

    @property
    def L(self) -> int:
        return len(self._t)

    def tensors3d(self) -> list:
        return [t.copy() for t in self._t]

    @property
    def arrays(self) -> tuple:
        n = len(self._t)
        out = []
        for i, t in enumerate(self._t):
            a = t if self.layout == "lpr" else t.transpose(0, 2, 1)
            if n > 1 and i == 0:
                a = a[0]
            elif n > 1 and i == n - 1:
                a = a[..., 0] if self.layout == "lpr" else a[:, 0, :]
            out.append(a)
        return tuple(out)

    def __getitem__(self, i: int) -> Tensor:
        return Tensor(self.arrays[i])

    def phys_dim(self) -> int:
        return int(self._t[0].shape[1])

    def bond_sizes(self) -> list:
        return [int(t.shape[2]) for t in self._t[:-1]]

    def max_bond(self) -> int:
        b = self.bond_sizes()
        return max(b) if b else 1

    def permute_arrays(self, shape: str) -> None:
        self.layout = shape


class MPS:
    """Matrix product state of a qubit register (see the module docstring)."""

    def __init__(self, statevector=None, mps=None, bond_dimension: int = 64) -> None:
        if not isinstance(bond_dimension, int) or isinstance(bond_dimension, bool) or bond_dimension < 1:
            raise ValueError(
                "`bond_dimension` must be an integer greater than 0. "
                f"Received {bond_dimension}."
            )
        self._form: str | None = None
        self._layout = "lpr"
        if (statevector is not None) and (mps is None):
            if not isinstance(statevector, Ket):
                statevector = Ket(statevector)
            if statevector.num_qubits == 1:
                raise ValueError(
                    "The statevector must have at least 2 qubits. "
                    f"Received {statevector.num_qubits}."
                )
            self.statevector = statevector
            self._tensors, self._dense = self._from_statevector_dev(statevector, bond_dimension)
            self._form = "right"
            # the complex128 input, for encoders run in the exact precision
            # mode (dropped once the state is changed)
            self._exact_source = statevector.data
        elif (mps is not None) and (statevector is None):
            if not isinstance(mps, MatrixProductState) and _quimb_like(mps):
                mps = _from_quimb(mps)
            if not isinstance(mps, MatrixProductState):
                raise TypeError(
                    "`mps` must be a `MatrixProductState` instance. "
                    f"Received {type(mps)}."
                )
            if mps.num_tensors == 1:
                raise ValueError(
                    "The MPS must have at least 2 tensors. "
                    f"Received {mps.num_tensors}."
                )
            self._tensors = mps.tensors3d()
            self._layout = mps.layout
            self._dense = self._dense_from_tensors(self._tensors)
            self.statevector = self.to_statevector(mps)
        else:
            raise ValueError("Must provide either `statevector` or `mps` not both.")
        self.bond_dimension = bond_dimension
        self.num_sites = self.statevector.num_qubits
        if self.mps.phys_dim() != 2:
            raise ValueError(
                "Only supports MPS with physical dimension of 2. "
                f"Received {self.mps.phys_dim()}."
            )
        self.physical_dimension = 2

    # ---- GPU helpers -----------------------------------------------------------
    @staticmethod
    def _from_statevector_dev(statevector: Ket, chi: int):
        eng = _engine.engine()
        p, sv = eng.upload([statevector.data], 1, chi)
        tensors, bonds, target = eng.stage_mps(p, sv, chi)
        torch.cuda.current_stream().synchronize()
        res = _engine.BatchResult(nqubits=p.nqubits, gates=None, arity=None, num_layers=None,
                                  layer_fidelities=None, sweep_fidelities=None, sweeps_done=None,
                                  fidelity=None, gate_off=p.gate_off,
                                  tensors=tensors.cpu().numpy().view(np.complex128),
                                  tensor_off=p.tensor_off, bonds=bonds.cpu().numpy(),
                                  max_n=p.max_n, max_bond=chi)
        return res.mps_tensors(0), target

    @staticmethod
    def _dense_from_tensors(tensors, precision: str = "fast") -> torch.Tensor:
        """Dense statevector of site tensors (l, p, r) on the GPU: complex64
        (float32 pairs), or complex128 contracted in double-float with
        ``precision="exact"``."""
        n = len(tensors)
        bonds = [1] + [int(t.shape[2]) for t in tensors[:-1]] + [1]
        chi = max(bonds)
        if chi > 1024:
            raise ValueError("MPS bonds above 1024 are not supported on the GPU path")
        eng = _engine.engine()
        p = eng.plan([n], 1, chi, precision)
        ce = p.chi_eff(0)
        store = np.zeros(p.tensor_elems, dtype=np.complex128)
        for s, t in enumerate(tensors):
            flat = np.asarray(t, dtype=np.complex128).reshape(-1)
            off = s * 2 * ce * ce
            store[off: off + flat.size] = flat
        bond_arr = np.zeros(p.max_n + 1, dtype=np.int32)
        bond_arr[: n + 1] = bonds
        dt = torch.from_numpy(store.view(np.float64)).cuda()
        db = torch.from_numpy(bond_arr).cuda()
        out = eng.mps_to_statevector(p, dt, db)
        torch.cuda.current_stream().synchronize()
        return out

    def _dense_np(self) -> np.ndarray:
        return self._dense.cpu().numpy().view(np.complex64).astype(np.complex128)

    def _set_dense(self, dense: torch.Tensor, form: str | None) -> None:
        self._exact_source = None
        self._dense = dense
        self._tensors = None
        self._form = form

    def _recompute_tensors(self, max_bond: int | None, cutoff_form: str) -> None:
        """Site tensors of the dense state by the truncated SVD (right or left form)."""
        n = self.num_sites
        self._exact_source = None
        if max_bond:
            chi = min(int(max_bond), 2 ** (n // 2))
            if chi > _MAX_SVD_BOND:
                raise ValueError(f"bond dimensions above {_MAX_SVD_BOND} are not supported on the GPU path")
        else:
            # no max_bond: only quimb's cutoff truncates (reference
            # qmprs/primitives/mps.py:441-453), so every bond may reach 2^(n/2)
            chi = min(2 ** (n // 2), _MAX_SVD_BOND)
        vec = self._dense_np()
        if cutoff_form == "left":
            vec = vec.reshape([2] * n).transpose(list(range(n))[::-1]).reshape(-1)
        eng = _engine.engine()
        p, sv = eng.upload([vec], 1, max(chi, 1))
        tensors, bonds, target = eng.stage_mps(p, sv, max(chi, 1))
        torch.cuda.current_stream().synchronize()
        res = _engine.BatchResult(nqubits=p.nqubits, gates=None, arity=None, num_layers=None,
                                  layer_fidelities=None, sweep_fidelities=None, sweeps_done=None,
                                  fidelity=None, gate_off=p.gate_off,
                                  tensors=tensors.cpu().numpy().view(np.complex128),
                                  tensor_off=p.tensor_off, bonds=bonds.cpu().numpy(),
                                  max_n=p.max_n, max_bond=max(chi, 1))
        ts = res.mps_tensors(0)
        if not max_bond and 2 ** (n // 2) > _MAX_SVD_BOND and max(t.shape[2] for t in ts[:-1]) >= _MAX_SVD_BOND:
            raise ValueError(f"the state needs bonds above {_MAX_SVD_BOND}, which the GPU path does not support")
        if cutoff_form == "left":
            ts = [t.transpose(2, 1, 0).copy() for t in ts[::-1]]
            tvec = target.cpu().numpy().view(np.complex64).reshape([2] * n)
            tvec = tvec.transpose(list(range(n))[::-1]).reshape(-1).copy()
            target = torch.from_numpy(tvec.view(np.float32)).cuda()
        self._tensors = ts
        self._dense = target
        self._form = cutoff_form

    # ---- data ------------------------------------------------------------------
    @property
    def mps(self) -> MatrixProductState:
        if self._tensors is None:
            self._recompute_tensors(None, self._form or "right")
        m = MatrixProductState.from_3d(self._tensors)
        m.layout = self._layout
        return m

    @staticmethod
    def from_statevector(statevector, max_bond_dimension: int) -> MatrixProductState:
        if not isinstance(statevector, Ket):
            statevector = Ket(statevector)
        tensors, _ = MPS._from_statevector_dev(statevector, max_bond_dimension)
        return MatrixProductState.from_3d(tensors)

    @staticmethod
    def to_statevector(mps: MatrixProductState) -> Ket:
        dense = MPS._dense_from_tensors(mps.tensors3d())
        return Ket(dense.cpu().numpy().view(np.complex64).astype(np.complex128), normalize=False)

    @property
    def norm(self) -> float:
        eng = _engine.engine()
        p = eng.plan([self.num_sites], 1, 1)
        ov = eng.overlap(p, self._dense, self._dense)
        return float(np.sqrt(max(ov.cpu().numpy()[0], 0.0)))

    @property
    def is_normalized(self) -> bool:
        return True if np.isclose(self.norm, 1) else False

    def normalize(self) -> None:
        if not self.is_normalized:
            nrm = self.norm
            self._dense = self._dense / nrm
            if self._tensors is not None:
                k = 0 if self._form != "left" else self.num_sites - 1
                self._tensors[k] = self._tensors[k] / nrm

    @property
    def orthogonal_center_range(self) -> tuple[int, int]:
        if self._form == "right":
            return (0, 0)
        if self._form == "left":
            return (self.num_sites - 1, self.num_sites - 1)
        return (0, self.num_sites - 1)

    @property
    def canonical_form(self) -> Literal["left", "right", "unknown"]:
        if self.orthogonal_center_range == (0, 0):
            return "right"
        elif self.orthogonal_center_range == (self.num_sites - 1, self.num_sites - 1):
            return "left"
        return "unknown"

    def canonicalize(self, mode: Literal["left", "right"], normalize=False) -> None:
        if mode not in ("left", "right"):
            raise ValueError("`mode` must be either 'left' or 'right'.")
        self._recompute_tensors(max(self.mps.max_bond(), 1), mode)
        if normalize:
            nrm = self.norm
            if nrm > 0:
                self._dense = self._dense / nrm
                k = 0 if mode == "right" else self.num_sites - 1
                self._tensors[k] = self._tensors[k] / nrm

    def compress(self, max_bond_dimension: int | None = None,
                 mode: Literal["left", "right"] | None = None) -> None:
        if mode is not None and mode not in ("left", "right"):
            raise ValueError(
                "`mode` must be either 'left', or 'right'. "
                f"Received {mode}."
            )
        self._recompute_tensors(max_bond_dimension, mode or "right")
        if max_bond_dimension:
            self.bond_dimension = max_bond_dimension

    def permute(self, shape: Literal["lrp", "lpr"]) -> None:
        if shape not in ["lrp", "lpr"]:
            raise ValueError(f"`shape` must be either 'lrp' or 'lpr'. Received {shape}.")
        self._layout = shape

    # ---- layers ----------------------------------------------------------------
    def generate_bond_D_unitary_layer(self) -> UnitaryLayer:
        eng = _engine.engine()
        n = self.num_sites
        p = eng.plan([n], 1, 2)
        gates, arity, nl, lf = eng.stage_layers(p, self._dense, 1, 1.0)
        torch.cuda.current_stream().synchronize()
        res = _engine.BatchResult(nqubits=[n], gates=gates.cpu().numpy().view(np.complex128),
                                  arity=arity.cpu().numpy(), num_layers=np.array([1]),
                                  layer_fidelities=None, sweep_fidelities=None, sweeps_done=None,
                                  fidelity=None, gate_off=p.gate_off, max_n=n, max_bond=2)
        return res.layers(0)[0]

    def generate_unitary_layer(self) -> UnitaryLayer:
        if self.mps.max_bond() > 2:
            raise ValueError("`generate_unitary_layer` needs an MPS with bond dimension at most 2; "
                             "use `generate_bond_D_unitary_layer`.")
        return self.generate_bond_D_unitary_layer()

    def _apply(self, unitary_layer: UnitaryLayer, inverse: bool) -> None:
        n = self.num_sites
        eng = _engine.engine()
        p = eng.plan([n], 1, 2)
        store = np.zeros(p.gate_elems, dtype=np.complex128)
        ar = np.zeros(p.gate_elems // 16, dtype=np.int8)
        covered = np.zeros(n, dtype=bool)
        for start, end, gates in unitary_layer:
            for idx in range(start, end + 1):
                g = np.asarray(getattr(gates[idx - start], "data", gates[idx - start]), dtype=np.complex128)
                k = 1 if idx == end else 2
                if g.shape != (2 ** k, 2 ** k):
                    raise ValueError("gate shape does not match its block position")
                store[idx * 16: idx * 16 + g.size] = g.reshape(-1)
                ar[idx] = k
                covered[idx] = True
        if not covered.all():
            raise ValueError("a unitary layer must cover every site exactly once")
        dg = torch.from_numpy(store.view(np.float64)).cuda()
        da = torch.from_numpy(ar).cuda()
        vec = self._dense.clone()
        eng.apply_layer(p, vec, dg, da, 0, inverse)
        torch.cuda.current_stream().synchronize()
        self._set_dense(vec, None)

    def apply_unitary_layer(self, unitary_layer: UnitaryLayer, inverse: bool = False) -> None:
        self._apply(unitary_layer, inverse)

    def apply_unitary_layers(self, unitary_layers: list, inverse: bool = False) -> None:
        for layer in reversed(unitary_layers):
            self.apply_unitary_layer(layer, inverse=inverse)

    def fidelity_with_zero_state(self) -> complex:
        z = self._dense[:2].cpu().numpy().astype(np.float64)
        return complex(z[0], -z[1])

    # ---- misc --------------------------------------------------------------------
    def contract_site(self, sites) -> None:
        raise NotImplementedError("contract_site is not part of the encoding path (quimb-only helper)")

    def contract_index(self, index: str) -> None:
        raise NotImplementedError("contract_index is not part of the encoding path (quimb-only helper)")

    def polar_decompose(self, indices) -> None:
        raise NotImplementedError("polar_decompose is not part of the encoding path (quimb-only helper)")

    def draw(self):
        raise NotImplementedError("draw needs matplotlib/quimb plotting, which is out of scope")

    def __deepcopy__(self, memo):
        new = MPS.__new__(MPS)
        for k, v in self.__dict__.items():
            if isinstance(v, torch.Tensor):
                new.__dict__[k] = v.clone()
            else:
                new.__dict__[k] = copy.deepcopy(v, memo)
        return new

    def __str__(self) -> str:
        return (
            f"{self.__class__.__name__}"
            f"(num_sites={self.num_sites}, "
            f"bond_dimension={self.bond_dimension}, "
            f"normalized={self.is_normalized}, "
            f"canonical_form={self.canonical_form})"
        )

    def __repr__(self) -> str:
        return f"{self.__class__.__name__}(num_sites={self.num_sites}, bond_dimension={self.bond_dimension})"

    def __len__(self) -> int:
        return self.num_sites

    def __eq__(self, value: object) -> bool:
        # The reference compares self's arrays with themselves (mps.py:1136);
        # this compares the two states' structure and tensors.
        if not isinstance(value, MPS):
            raise TypeError("`value` must be an instance of `qmprs.primitives.MPS`.")
        a, b = self.mps, value.mps
        if a.bond_sizes() != b.bond_sizes():
            return False
        return all(np.allclose(x, y) for x, y in zip(a.tensors3d(), b.tensors3d()))
