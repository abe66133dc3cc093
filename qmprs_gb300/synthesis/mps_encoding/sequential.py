"""Sequential (Ran + Rudolph et al.) encoder on the GPU.

Mirrors ``qmprs.synthesis.mps_encoding.Sequential`` (reference
``qmprs/synthesis/mps_encoding/sequential.py:31-600``): the layers of
Ran's analytic decomposition (arXiv:1908.07958) generated until the state
is disentangled or ``num_layers`` is reached, then ``num_sweeps``
environment sweeps (arXiv:2209.00595, "Dall Oall"), emitted into the
injected circuit class with the reference's LSB qubit mapping.  All
arithmetic runs in the GPU library through ``qmprs_gb300.engine``.

Beyond the reference API, ``prepare_states`` encodes a batch of
statevectors (of any qubit counts) in one pass of every GPU stage, and
``last_run`` records the per-layer and per-sweep fidelities of the last
call.
"""

from __future__ import annotations

import numpy as np
import torch

from ... import engine as _engine
from ...ket import Ket
from ...primitives import MPS
from .base import MPSEncoder


def _gate_data(g) -> np.ndarray:
    return np.asarray(getattr(g, "data", g), dtype=np.complex128)


class Sequential(MPSEncoder):
    """Sequential MPS encoder; see the module docstring."""

    def __init__(self, circuit_framework) -> None:
        super().__init__(circuit_framework)
        self._fidelity_threshold = 1 - 1e-6
        self.last_run: dict = {}

    @property
    def fidelity_threshold(self) -> float:
        return self._fidelity_threshold

    @fidelity_threshold.setter
    def fidelity_threshold(self, threshold: float) -> None:
        if not isinstance(threshold, (int, float)) or threshold < 0 or threshold > 1:
            raise ValueError("The fidelity threshold must be a float between 0 and 1.")
        self._fidelity_threshold = threshold

    # ---- circuit emission (sequential.py:156-214) ---------------------------------
    @staticmethod
    def _apply_unitary_layer_to_circuit(circuit, unitary_layer) -> None:
        for start_index, end_index, unitary_block in unitary_layer:
            for index in range(start_index, end_index + 1):
                unitary = _gate_data(unitary_block[index - start_index])
                # LSB mapping of MSB site `index` (sequential.py:173-186)
                if index == end_index:
                    circuit.unitary(unitary, abs(index - circuit.num_qubits + 1))
                else:
                    circuit.unitary(unitary, [abs(index - circuit.num_qubits + 2),
                                              abs(index - circuit.num_qubits + 1)])

    def _circuit_from_unitary_layers(self, mps: MPS, unitary_layers: list):
        circuit = self.circuit_framework(mps.num_sites)
        for layer in unitary_layers:
            Sequential._apply_unitary_layer_to_circuit(circuit, layer)
        return circuit

    # ---- device gate store <-> UnitaryLayer lists -------------------------------------
    @staticmethod
    def _layers_to_store(unitary_layers: list, n: int, p) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        L = len(unitary_layers)
        store = np.zeros(p.gate_elems, dtype=np.complex128)
        ar = np.zeros(p.gate_elems // 16, dtype=np.int8)
        for c, layer in enumerate(unitary_layers):
            g = L - 1 - c                                     # generation index
            covered = np.zeros(n, dtype=bool)
            for start, end, gates in layer:
                for idx in range(start, end + 1):
                    u = _gate_data(gates[idx - start])
                    k = 1 if idx == end else 2
                    if u.shape != (2 ** k, 2 ** k):
                        raise ValueError("gate shape does not match its block position")
                    slot = g * n + idx
                    store[slot * 16: slot * 16 + u.size] = u.reshape(-1)
                    ar[slot] = k
                    covered[idx] = True
            if not covered.all():
                raise ValueError("each unitary layer must cover every site once")
        return (torch.from_numpy(store.view(np.float64)).cuda(), torch.from_numpy(ar).cuda(),
                torch.tensor([L], dtype=torch.int32, device="cuda"))

    @staticmethod
    def _result(p, gates, arity, nl, lf=None, sf=None, sd=None) -> _engine.BatchResult:
        torch.cuda.current_stream().synchronize()
        return _engine.BatchResult(
            nqubits=p.nqubits, gates=gates.cpu().numpy().view(np.complex128), arity=arity.cpu().numpy(),
            num_layers=nl.cpu().numpy(),
            layer_fidelities=None if lf is None else lf.cpu().numpy().view(np.complex128).reshape(p.B, -1),
            sweep_fidelities=None if sf is None else sf.cpu().numpy(), sweeps_done=None if sd is None else sd.cpu().numpy(),
            fidelity=None, gate_off=p.gate_off, max_n=p.max_n, max_bond=p.max_bond)

    # ---- reference stages -----------------------------------------------------------
    def _get_unitary_layers(self, mps: MPS, num_layers: int) -> list:
        """``Sequential._get_unitary_layers`` (sequential.py:330-398) on the GPU."""
        eng = _engine.engine()
        p = eng.plan([mps.num_sites], num_layers, max(mps.bond_dimension, 1))
        gates, arity, nl, lf = eng.stage_layers(p, mps._dense, num_layers, self.fidelity_threshold)
        res = self._result(p, gates, arity, nl, lf)
        self.last_run = {"layer_fidelities": res.layer_fidelities[0, : int(res.num_layers[0])]}
        return res.layers(0)

    def _optimize_unitary_layers(self, mps: MPS, unitary_layers: list, num_sweeps: int) -> list:
        """``Sequential._optimize_unitary_layers`` (sequential.py:509-541) on the GPU."""
        if num_sweeps <= 0 or not unitary_layers:
            return unitary_layers
        eng = _engine.engine()
        n = mps.num_sites
        p = eng.plan([n], len(unitary_layers), max(mps.bond_dimension, 1))
        gates, arity, nl = self._layers_to_store(unitary_layers, n, p)
        sf, sd = eng.stage_sweeps(p, mps._dense, gates, arity, nl, num_sweeps)
        res = self._result(p, gates, arity, nl, sf=sf, sd=sd)
        self.last_run["sweep_fidelities"] = res.sweep_fidelities[:num_sweeps]
        return res.layers(0)

    def _sequential_unitary_circuit(self, mps: MPS, num_layers: int, num_sweeps: int = 0):
        """``_get_unitary_layers`` then ``_optimize_unitary_layers`` without leaving the GPU."""
        eng = _engine.engine()
        p = eng.plan([mps.num_sites], num_layers, max(mps.bond_dimension, 1))
        gates, arity, nl, lf = eng.stage_layers(p, mps._dense, num_layers, self.fidelity_threshold)
        sf = sd = None
        if num_sweeps > 0:
            sf, sd = eng.stage_sweeps(p, mps._dense, gates, arity, nl, num_sweeps)
        res = self._result(p, gates, arity, nl, lf, sf, sd)
        self.last_run = {
            "layer_fidelities": res.layer_fidelities[0, : int(res.num_layers[0])],
            "sweep_fidelities": None if sf is None else res.sweep_fidelities[:num_sweeps],
            "num_layers": int(res.num_layers[0]),
        }
        return self._circuit_from_unitary_layers(mps, res.layers(0))

    def _exact_unitary_circuit(self, mps: MPS, num_layers: int, num_sweeps: int):
        """The same path in the exact precision mode (double-float working
        states): from the MPS's complex128 input when it was built from a
        statevector and not changed since, else from its site tensors
        contracted in double-float."""
        eng = _engine.engine()
        n = mps.num_sites
        sv = getattr(mps, "_exact_source", None)
        if sv is not None:
            chi = max(mps.bond_dimension, 1)
        else:
            ts = mps.mps.tensors3d()
            chi = max([1] + [int(t.shape[2]) for t in ts[:-1]])
            sv = MPS._dense_from_tensors(ts, "exact").cpu().numpy().view(np.complex128)
        res = eng.encode([sv], chi, num_layers, num_sweeps, self.fidelity_threshold, precision="exact")
        L = int(res.num_layers[0])
        self.last_run = {
            "layer_fidelities": res.layer_fidelities[0, :L],
            "sweep_fidelities": res.sweep_fidelities[0] if num_sweeps > 0 else None,
            "num_layers": L,
        }
        return self._circuit_from_unitary_layers(mps, res.layers(0))

    def prepare_mps(self, mps: MPS, **kwargs):
        """``Sequential.prepare_mps`` (sequential.py:588-600).  Extension:
        ``precision="exact"`` runs the double-float mode, whose per-layer and
        per-sweep fidelities follow an FP64 run of the reference's algorithm
        (the default "fast" keeps complex64 states)."""
        num_layers = kwargs.get("num_layers", 1)
        num_sweeps = kwargs.get("num_sweeps", 0)
        precision = kwargs.get("precision", "fast")
        if not isinstance(num_layers, int) or num_layers < 1:
            raise ValueError("The number of layers must be a positive integer.")
        if precision not in ("fast", "exact"):
            raise ValueError("precision must be 'fast' or 'exact'.")
        if precision == "exact":
            return self._exact_unitary_circuit(mps, num_layers, num_sweeps)
        return self._sequential_unitary_circuit(mps, num_layers, num_sweeps)

    # ---- batched extension -------------------------------------------------------------
    def prepare_states(self, statevectors, bond_dimension: int, num_layers: int = 1, num_sweeps: int = 0,
                       stop_fidelity: float = 0.0, emit: bool = True, nqubits=None, *, warm_start=None,
                       schedule: str = "oall", precision: str = "fast"):
        """Encode many statevectors at once (any mix of qubit counts).

        Same result per state as ``prepare_state`` (default
        ``compression_percentage``/``index_type``); with ``stop_fidelity > 0``
        a state stops sweeping once ``|<target|C|0>|`` reaches it.
        ``statevectors`` is a list of arrays, or, with ``nqubits``, one
        packed float32 torch tensor (host, ideally pinned, or device) of the
        complex64 amplitudes of all states back to back; packed inputs are
        normalised on the device.  Returns the list of circuits
        (``emit=True``, else None) and the engine's BatchResult.
        ``warm_start`` (keyword only; a ``qmprs_gb300.warmstart.WarmStartMLP``)
        starts the sweeps from the network's predicted layers; states that
        end below ``stop_fidelity`` fall back to the analytic layers.
        ``precision`` (keyword only): ``"fast"`` or ``"exact"`` (double-float
        working states; a packed buffer is then float64 pairs).
        ``schedule`` (keyword only): ``"oall"`` (the reference's: all layers,
        then ``num_sweeps`` sweeps), ``"iter_dioall"`` (one layer at a time
        from the residual, each followed by ``num_sweeps`` sweeps of all
        layers) or ``"iter_dioi"`` (one layer at a time, each followed by
        ``num_sweeps`` sweeps of that layer alone against the residual);
        arXiv:2209.00595, documented by the reference's sweep.
        """
        if schedule not in ("oall", "iter_dioall", "iter_dioi"):
            raise ValueError("schedule must be 'oall', 'iter_dioall' or 'iter_dioi'.")
        if precision not in ("fast", "exact"):
            raise ValueError("precision must be 'fast' or 'exact'.")
        if not isinstance(num_layers, int) or num_layers < 1:
            raise ValueError("The number of layers must be a positive integer.")
        if not isinstance(bond_dimension, int) or bond_dimension < 1:
            raise ValueError("`bond_dimension` must be an integer greater than 0.")
        eng = _engine.engine()
        if nqubits is not None:
            ns = [int(n) for n in nqubits]
            if any(n < 2 for n in ns):
                raise ValueError("The statevector must have at least 2 qubits.")
            if schedule != "oall":
                res = eng.encode_iterative(statevectors, bond_dimension, num_layers, num_sweeps, nqubits=ns,
                                           schedule=schedule, precision=precision)
            else:
                res = eng.encode(statevectors, bond_dimension, num_layers, num_sweeps, self.fidelity_threshold,
                                 stop_fidelity, nqubits=ns, warm_start=warm_start, precision=precision)
        else:
            kets = [sv if isinstance(sv, Ket) else Ket(sv) for sv in statevectors]
            ns = [k.num_qubits for k in kets]
            if any(n < 2 for n in ns):
                raise ValueError("The statevector must have at least 2 qubits.")
            if schedule != "oall":
                res = eng.encode_iterative([k.data for k in kets], bond_dimension, num_layers, num_sweeps,
                                           schedule=schedule, precision=precision)
            else:
                res = eng.encode([k.data for k in kets], bond_dimension, num_layers, num_sweeps,
                                 self.fidelity_threshold, stop_fidelity, warm_start=warm_start, precision=precision)
        circuits = None
        if emit:
            circuits = []
            for b, n in enumerate(ns):
                c = self.circuit_framework(n)
                for layer in res.layers(b):
                    Sequential._apply_unitary_layer_to_circuit(c, layer)
                circuits.append(c)
        return circuits, res
