"""Batched GPU encoding engine (host side of the C ABI).

``Engine.encode`` runs the reference's whole ``prepare_state`` path for a
batch of statevectors of possibly different qubit counts:

1. ``qmprs_mps_from_statevector``  (a)  ``MPS.from_statevector``
2. ``qmprs_unitary_layers``        (b)+(c) ``Sequential._get_unitary_layers``
3. ``qmprs_optimize_layers``       (d)  ``Sequential._optimize_unitary_layers``
4. ``qmprs_circuit_state`` + ``qmprs_overlap``  fidelity |<sv|C|0>|

PyTorch provides device memory, pinned host memory and the stream; all
arithmetic runs in the library's kernels.
"""

from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native

_tls = threading.local()


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class Handle:
    """One library handle per host thread (handles are not shared)."""

    def __init__(self):
        if not torch.cuda.is_available():
            raise RuntimeError("qmprs_gb300 needs a CUDA device (no CPU fallback)")
        self.lib = _native.load()
        h = ctypes.c_void_p()
        code = self.lib.qmprs_create(ctypes.byref(h))
        if code != 0:
            raise _native.NativeError(code, "qmprs_create failed")
        self.h = h

    def check(self, code: int) -> None:
        _native.raise_for(code, self.h)

    def __del__(self):
        try:
            self.lib.qmprs_destroy(self.h)
        except Exception:
            pass


def handle() -> Handle:
    h = getattr(_tls, "handle", None)
    if h is None:
        h = Handle()
        _tls.handle = h
    return h


class _DeviceBuffer:
    """A float32 device array owned by the library (a plan buffer), exposed
    to torch through the CUDA array interface without a copy."""

    def __init__(self, ptr: int, numel: int, typestr: str = "<f4"):
        self.__cuda_array_interface__ = {"shape": (int(numel),), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


class Plan:
    """A batch layout: offsets of every state in the caller buffers.

    ``precision`` "fast": complex64 statevector buffers (float32 pairs);
    "exact": complex128 buffers (float64 pairs) and double-float working
    states (``QMPRS_PRECISION_EXACT``)."""

    def __init__(self, hd: Handle, nqubits: list[int], max_layers: int, max_bond: int, precision: str = "fast"):
        self.hd = hd
        self.lib = hd.lib
        self.nqubits = [int(n) for n in nqubits]
        self.B = len(self.nqubits)
        self.max_layers = int(max_layers)
        self.max_bond = int(max_bond)
        if precision not in _native.PRECISIONS:
            raise ValueError("precision must be 'fast' or 'exact'.")
        self.precision = precision
        arr = (ctypes.c_int * self.B)(*self.nqubits)
        p = ctypes.c_void_p()
        hd.check(self.lib.qmprs_plan_create(hd.h, self.B, arr, self.max_layers, self.max_bond, ctypes.byref(p)))
        self.p = p
        hd.check(self.lib.qmprs_plan_set_precision(p, _native.PRECISIONS[precision]))
        ve, ge, te = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        vo = (ctypes.c_int64 * self.B)()
        go = (ctypes.c_int64 * self.B)()
        to = (ctypes.c_int64 * self.B)()
        hd.check(self.lib.qmprs_plan_layout(p, ctypes.byref(ve), ctypes.byref(ge), ctypes.byref(te), vo, go, to))
        self.vec_elems, self.gate_elems, self.tensor_elems = ve.value, ge.value, te.value
        self.vec_off = np.array(vo[:], dtype=np.int64)
        self.gate_off = np.array(go[:], dtype=np.int64)
        self.tensor_off = np.array(to[:], dtype=np.int64)
        self.max_n = self.lib.qmprs_plan_max_qubits(p)

    @property
    def vdtype(self):
        """Real dtype of the statevector-sized buffers (two entries per amplitude)."""
        return torch.float64 if self.precision == "exact" else torch.float32

    @property
    def npdtype(self):
        return np.complex128 if self.precision == "exact" else np.complex64

    def vec(self) -> torch.Tensor:
        """An uninitialised statevector-sized device buffer of this plan."""
        return torch.empty(self.vec_elems * 2, dtype=self.vdtype, device="cuda")

    def buf(self, name: str, numel: int, dtype, zero: bool = False) -> torch.Tensor:
        """A device buffer kept on the plan under `name` (reallocated only
        when its size or type changes), so that repeated calls present the
        same addresses to the library and its stage graphs replay."""
        store = self.__dict__.setdefault("_bufs", {})
        t = store.get(name)
        if t is None or t.numel() != numel or t.dtype != dtype:
            t = torch.empty(numel, dtype=dtype, device="cuda")
            store[name] = t
        if zero:
            t.zero_()
        return t

    def chi_eff(self, b: int) -> int:
        return min(self.max_bond, 2 ** (self.nqubits[b] // 2))

    def __del__(self):
        try:
            self.lib.qmprs_plan_destroy(self.p)
        except Exception:
            pass


@dataclass
class BatchResult:
    nqubits: list
    gates: np.ndarray            # complex128 gate store (generation order)
    arity: np.ndarray            # int8
    num_layers: np.ndarray       # int32 [B]
    layer_fidelities: np.ndarray  # complex128 [B, L]
    sweep_fidelities: np.ndarray  # float64 [B, S]
    sweeps_done: np.ndarray      # int32 [B]
    fidelity: np.ndarray         # float64 [B] |<sv|C|0>|
    gate_off: np.ndarray
    tensors: np.ndarray | None = None
    tensor_off: np.ndarray | None = None
    bonds: np.ndarray | None = None
    max_n: int = 0
    max_bond: int = 0
    timings: dict = field(default_factory=dict)

    def layers(self, b: int) -> list:
        """Layers of state b in CIRCUIT order, as the reference's ``UnitaryLayer`` lists.

        Each layer is a list of blocks ``(start, end, [gate, ...])``; the
        gate of the block's last site is 2x2, the others 4x4
        (``qmprs/primitives/mps.py:46-47``).
        """
        n = self.nqubits[b]
        L = int(self.num_layers[b])
        base = int(self.gate_off[b])
        out = []
        for l in range(L - 1, -1, -1):
            blocks = []
            start = 0
            gates = []
            for s in range(n):
                slot = l * n + s
                k = int(self.arity[base // 16 + slot])
                raw = self.gates[base + slot * 16: base + slot * 16 + 16]
                g = raw[:4].reshape(2, 2).copy() if k == 1 else raw.reshape(4, 4).copy()
                gates.append(g)
                if k == 1:
                    blocks.append((start, s, gates))
                    start = s + 1
                    gates = []
            out.append(blocks)
        return out

    def mps_tensors(self, b: int) -> list:
        """Site tensors (l, p, r) of state b's MPS from stage (a)."""
        n = self.nqubits[b]
        ce = min(self.max_bond, 2 ** (n // 2))
        bonds = self.bonds[b * (self.max_n + 1): b * (self.max_n + 1) + n + 1]
        base = int(self.tensor_off[b])
        out = []
        for s in range(n):
            l, r = int(bonds[s]), int(bonds[s + 1])
            off = base + s * 2 * ce * ce
            out.append(self.tensors[off: off + l * 2 * r].reshape(l, 2, r).copy())
        return out


class Engine:
    """Runs the encoding path for batches of states on the current CUDA device."""

    def __init__(self):
        self.hd = handle()
        self.lib = self.hd.lib
        self._plans: dict = {}

    def plan(self, nqubits, max_layers: int, max_bond: int, precision: str = "fast") -> Plan:
        key = (tuple(int(n) for n in nqubits), int(max_layers), int(max_bond), precision)
        p = self._plans.get(key)
        if p is None:
            p = Plan(self.hd, list(key[0]), key[1], key[2], precision)
            self._plans[key] = p
        return p

    @staticmethod
    def pack(statevectors, dtype=np.complex64) -> tuple[list[int], np.ndarray]:
        """Concatenate complex statevectors (already Ket-normalised) as ``dtype``."""
        ns, parts = [], []
        for v in statevectors:
            v = np.asarray(v).reshape(-1)
            n = int(round(np.log2(v.size)))
            if 2 ** n != v.size:
                raise ValueError("statevector length must be a power of two")
            ns.append(n)
            parts.append(v.astype(dtype))
        return ns, np.concatenate(parts)

    # ---- stages --------------------------------------------------------------
    def upload(self, statevectors, max_layers: int, max_bond: int, precision: str = "fast", reuse: bool = False):
        """Plan the batch and copy the (Ket-normalised) statevectors to the device."""
        ns, host = self.pack(statevectors, np.complex128 if precision == "exact" else np.complex64)
        p = self.plan(ns, max_layers, max_bond, precision)
        pinned = torch.from_numpy(host.view(np.float64 if precision == "exact" else np.float32)).pin_memory()
        sv = p.buf("input", p.vec_elems * 2, p.vdtype) if reuse else p.vec()
        sv.copy_(pinned, non_blocking=True)
        return p, sv

    def stage_mps(self, p: Plan, sv: torch.Tensor, bond_dimension: int, stream=None, reuse: bool = False):
        """(a) statevector -> MPS: site tensors, bonds and the dense truncated target.
        ``reuse``: write into the plan's own stage buffers (``Plan.buf``)."""
        sp = self._sp(stream)
        if reuse:
            tensors = p.buf("tensors", max(p.tensor_elems, 1) * 2, torch.float64)
            bonds = p.buf("bonds", p.B * (p.max_n + 1), torch.int32)
            target = p.buf("target", p.vec_elems * 2, p.vdtype)
        else:
            tensors = torch.empty(max(p.tensor_elems, 1) * 2, dtype=torch.float64, device="cuda")
            bonds = torch.empty(p.B * (p.max_n + 1), dtype=torch.int32, device="cuda")
            target = p.vec()
        self.hd.check(self.lib.qmprs_mps_from_statevector(p.p, _ptr(sv), int(bond_dimension), 1e-10,
                                                          _ptr(tensors), _ptr(bonds), _ptr(target), sp))
        return tensors, bonds, target

    def mps_to_statevector(self, p: Plan, tensors: torch.Tensor, bonds: torch.Tensor, stream=None) -> torch.Tensor:
        sp = self._sp(stream)
        out = p.vec()
        self.hd.check(self.lib.qmprs_mps_to_statevector(p.p, _ptr(tensors), _ptr(bonds), _ptr(out), sp))
        return out

    def stage_layers(self, p: Plan, target: torch.Tensor, num_layers: int, fidelity_threshold: float,
                     stream=None, reuse: bool = False):
        """(b)+(c) disentangling layers from the dense target."""
        sp = self._sp(stream)
        if reuse:
            gates = p.buf("gates", p.gate_elems * 2, torch.float64, zero=True)
            arity = p.buf("arity", p.gate_elems // 16, torch.int8, zero=True)
            nl = p.buf("nl", p.B, torch.int32, zero=True)
            lf = p.buf("lf", p.B * num_layers * 2, torch.float64, zero=True)
        else:
            gates = torch.zeros(p.gate_elems * 2, dtype=torch.float64, device="cuda")
            arity = torch.zeros(p.gate_elems // 16, dtype=torch.int8, device="cuda")
            nl = torch.zeros(p.B, dtype=torch.int32, device="cuda")
            lf = torch.zeros(p.B * num_layers * 2, dtype=torch.float64, device="cuda")
        self.hd.check(self.lib.qmprs_unitary_layers(p.p, _ptr(target), int(num_layers), float(fidelity_threshold),
                                                    _ptr(gates), _ptr(arity), _ptr(nl), _ptr(lf), sp))
        return gates, arity, nl, lf

    def stage_sweeps(self, p: Plan, target, gates, arity, nl, num_sweeps: int, stop_fidelity: float = 0.0,
                     stream=None, reuse: str = ""):
        """(d) environment sweeps; returns per-sweep fidelities and sweeps run.
        ``reuse``: a name under which the plan keeps the output buffers."""
        sp = self._sp(stream)
        S = max(int(num_sweeps), 0)
        if reuse:
            sf = p.buf(reuse + "_sf", max(p.B * S, 1), torch.float64, zero=True)
            sd = p.buf(reuse + "_sd", p.B, torch.int32, zero=True)
        else:
            sf = torch.zeros(max(p.B * S, 1), dtype=torch.float64, device="cuda")
            sd = torch.zeros(p.B, dtype=torch.int32, device="cuda")
        if S > 0:
            self.hd.check(self.lib.qmprs_optimize_layers(p.p, _ptr(target), _ptr(gates), _ptr(arity), _ptr(nl), S,
                                                         float(stop_fidelity), _ptr(sf), _ptr(sd), sp))
        return sf, sd

    def environments(self, p: Plan, target, gates, arity, nl, env: torch.Tensor | None = None,
                     stream=None) -> torch.Tensor:
        """Every gate's environment at the fixed circuit (no update), in the
        gate store's layout (complex128 as float64 pairs): at each slot the
        m x m E with <target|C|0> = sum(G * E) for that gate G."""
        if env is None:
            env = torch.empty(p.gate_elems * 2, dtype=torch.float64, device="cuda")
        self.hd.check(self.lib.qmprs_layer_environments(p.p, _ptr(target), _ptr(gates), _ptr(arity), _ptr(nl),
                                                        _ptr(env), self._sp(stream)))
        return env

    def stage_circuit(self, p: Plan, gates, arity, nl, stream=None, reuse: str = "") -> torch.Tensor:
        sp = self._sp(stream)
        circ = p.buf(reuse + "_circ", p.vec_elems * 2, p.vdtype) if reuse else p.vec()
        self.hd.check(self.lib.qmprs_circuit_state(p.p, _ptr(gates), _ptr(arity), _ptr(nl), _ptr(circ), sp))
        return circ

    def overlap(self, p: Plan, a: torch.Tensor, b: torch.Tensor, stream=None, reuse: str = "") -> torch.Tensor:
        sp = self._sp(stream)
        ov = p.buf(reuse + "_ov", p.B * 2, torch.float64) if reuse else torch.zeros(p.B * 2, dtype=torch.float64,
                                                                                       device="cuda")
        self.hd.check(self.lib.qmprs_overlap(p.p, _ptr(a), _ptr(b), _ptr(ov), sp))
        return ov

    def apply_layer(self, p: Plan, vec, gates, arity, layer: int, inverse: bool, stream=None) -> None:
        sp = self._sp(stream)
        self.hd.check(self.lib.qmprs_apply_layer(p.p, _ptr(vec), _ptr(gates), _ptr(arity), int(layer),
                                                 1 if inverse else 0, sp))

    def set_graphs(self, p: Plan, on: bool) -> None:
        """Replay the layer and sweep stages of plan ``p`` as CUDA graphs (the
        default) or launch them one by one."""
        self.hd.check(self.lib.qmprs_plan_set_graphs(p.p, 1 if on else 0))

    def set_autotune(self, p: Plan, on: bool) -> None:
        """Let the sweep stage pick the tile passes' grid by timing (the default)."""
        self.hd.check(self.lib.qmprs_plan_set_autotune(p.p, 1 if on else 0))

    def tuning(self, p: Plan) -> tuple[int, bool]:
        """(grid of the tile passes, chosen by the autotuner) of plan ``p``."""
        g, t = ctypes.c_int(), ctypes.c_int()
        self.hd.check(self.lib.qmprs_plan_tuning(p.p, ctypes.byref(g), ctypes.byref(t)))
        return g.value, bool(t.value)

    def graph_stats(self, p: Plan) -> tuple[int, int]:
        """(graphs cached, graph replays so far) of plan ``p``."""
        c, r = ctypes.c_int(), ctypes.c_int64()
        self.hd.check(self.lib.qmprs_plan_graph_stats(p.p, ctypes.byref(c), ctypes.byref(r)))
        return c.value, r.value

    def wide_stats(self, p: Plan) -> dict:
        """Counters of the eigensolver of Grams wider than 128 (bonds above
        64) in stage (a): Grams solved, FP32 block-Jacobi sweeps, FP64
        refinement steps, largest first-order correction of a last step."""
        g, sw, st, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self.hd.check(self.lib.qmprs_plan_wide_stats(p.p, ctypes.byref(g), ctypes.byref(sw), ctypes.byref(st),
                                                      ctypes.byref(e)))
        return {"grams": g.value, "sweeps": sw.value, "refine_steps": st.value, "last_correction": e.value}

    def set_profiling(self, p: Plan, on: bool) -> None:
        self.hd.check(self.lib.qmprs_plan_set_profiling(p.p, 1 if on else 0))

    def profile(self, p: Plan, kernel: int) -> tuple[int, float, float]:
        """(launches, event milliseconds, algorithmic bytes) of a sweep kernel class."""
        n, ms, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        self.hd.check(self.lib.qmprs_plan_profile(p.p, int(kernel), ctypes.byref(n), ctypes.byref(ms),
                                                  ctypes.byref(by)))
        return n.value, ms.value, by.value

    def launch_count(self) -> int:
        return int(self.lib.qmprs_launch_count())

    def random_mps_states(self, ns, bonds, seed: int) -> torch.Tensor:
        """Random-MPS statevectors (i.i.d. complex Gaussian tensors of bond
        ``bonds[b]``, left-canonicalised, contracted on the GPU, normalised)
        in one packed complex64 device buffer with the plan layout of ``ns``."""
        chi = max(int(x) for x in bonds)
        p = self.plan(ns, 1, chi)
        rng = np.random.default_rng(seed)
        store = np.zeros(p.tensor_elems, dtype=np.complex128)
        bond_arr = np.zeros((p.B, p.max_n + 1), dtype=np.int32)
        for b, (n, bd) in enumerate(zip(ns, bonds)):
            dims = [1] + [min(int(bd), 2 ** min(i, n - i)) for i in range(1, n)] + [1]
            ts = []
            for i in range(n):
                shape = (dims[i], 2, dims[i + 1])
                ts.append((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0))
            for i in range(n - 1):
                l, pp, r = ts[i].shape
                q, rr = np.linalg.qr(ts[i].reshape(l * pp, r))
                ts[i] = q.reshape(l, pp, q.shape[1])
                nl, np_, nr = ts[i + 1].shape
                ts[i + 1] = (rr @ ts[i + 1].reshape(nl, np_ * nr)).reshape(q.shape[1], np_, nr)
            ce = p.chi_eff(b)
            base = int(p.tensor_off[b])
            for s, t in enumerate(ts):
                off = base + s * 2 * ce * ce
                store[off: off + t.size] = t.reshape(-1)
            bond_arr[b, : n + 1] = [1] + [t.shape[2] for t in ts]
        dt = torch.from_numpy(store.view(np.float64)).cuda()
        db = torch.from_numpy(bond_arr.reshape(-1)).cuda()
        vec = self.mps_to_statevector(p, dt, db)
        ov = self.overlap(p, vec, vec)
        torch.cuda.current_stream().synchronize()
        inv = torch.rsqrt(ov[0::2]).to(torch.float32)
        counts = torch.tensor([2 ** (n + 1) for n in ns], dtype=torch.int64, device="cuda")
        return vec * torch.repeat_interleave(inv, counts)

    def encode_iterative(self, statevectors, bond_dimension: int, num_layers: int, sweeps_per_layer: int,
                         nqubits=None, schedule: str = "iter_dioall", precision: str = "fast") -> BatchResult:
        """Iterative schedules (arXiv:2209.00595, documented by the reference
        at qmprs/synthesis/mps_encoding/sequential.py:410-433): for k =
        1..num_layers, generate one analytic layer from the residual
        r = C^H |target> of the current circuit (the newest layer is applied
        first), then sweep `sweeps_per_layer` times
          "iter_dioall": all k layers against the target;
          "iter_dioi":   the newest layer alone against r (the older layers
                         stay fixed; its fidelity is the whole circuit's),
                         then r <- U^H r.
        Every state gets all num_layers layers (no early exit).
        ``sweep_fidelities`` holds the fidelity after every sweep,
        num_layers * sweeps_per_layer columns."""
        if schedule not in ("iter_dioall", "iter_dioi"):
            raise ValueError("schedule must be 'iter_dioall' or 'iter_dioi'.")
        dioi = schedule == "iter_dioi"
        if nqubits is None:
            p, sv = self.upload(statevectors, num_layers, bond_dimension, precision)
        else:
            p = self.plan(nqubits, num_layers, bond_dimension, precision)
            sv = statevectors if statevectors.is_cuda else statevectors.to("cuda", non_blocking=True)
        _, _, target = self.stage_mps(p, sv, bond_dimension)
        B, L, S = p.B, int(num_layers), int(sweeps_per_layer)
        gates = torch.zeros(p.gate_elems * 2, dtype=torch.float64, device="cuda")
        arity = torch.zeros(p.gate_elems // 16, dtype=torch.int8, device="cuda")
        nl = torch.zeros(B, dtype=torch.int32, device="cuda")
        # gate-store rows (16 complex each) of generated layer l, all states
        rows = [np.concatenate([p.gate_off[b] // 16 + l * n + np.arange(n) for b, n in enumerate(p.nqubits)])
                for l in range(L)]
        g_rows = gates.view(-1, 32)
        fids = []
        residual = target.clone()
        one = torch.ones(B, dtype=torch.int32, device="cuda")
        for k in range(L):
            g1, a1, _, _ = self.stage_layers(p, residual, 1, 1.0)
            if dioi and S > 0:
                # the newest layer alone, against the residual
                sf, _ = self.stage_sweeps(p, residual, g1, a1, one, S, 0.0)
                fids.append(sf[: B * S].view(B, S))
            src = torch.as_tensor(rows[0], device="cuda")
            dst = torch.as_tensor(rows[k], device="cuda")
            g_rows[dst] = g1.view(-1, 32)[src]
            arity[dst] = a1[src]
            nl.fill_(k + 1)
            if dioi:
                self.apply_layer(p, residual, gates, arity, k, True)   # r <- U_k^H r
                continue
            if S > 0:
                sf, _ = self.stage_sweeps(p, target, gates, arity, nl, S, 0.0)
                fids.append(sf[: B * S].view(B, S))
            residual = target.clone()
            for l in range(k + 1):       # C^H t: inverse of generated layer 0 (applied last) first
                self.apply_layer(p, residual, gates, arity, l, True)
        circ = self.stage_circuit(p, gates, arity, nl)
        ov = self.overlap(p, circ, sv)
        nn = self.overlap(p, sv, sv)
        torch.cuda.current_stream().synchronize()
        ovh = ov.cpu().numpy().view(np.complex128)
        nnh = nn.cpu().numpy().view(np.complex128).real
        sfh = torch.cat(fids, dim=1).cpu().numpy() if fids else np.zeros((B, 0))
        return BatchResult(
            nqubits=p.nqubits, gates=gates.cpu().numpy().view(np.complex128), arity=arity.cpu().numpy(),
            num_layers=nl.cpu().numpy(), layer_fidelities=np.zeros((B, L), np.complex128),
            sweep_fidelities=sfh, sweeps_done=np.full(B, L * S, np.int32), fidelity=np.abs(ovh) / np.sqrt(nnh),
            gate_off=p.gate_off, max_n=p.max_n, max_bond=int(bond_dimension))

    def _fallback(self, p: Plan, target, sv, analytic, gates, arity, nl, sf, sd, ov, nn, num_sweeps: int,
                  stop_fidelity: float):
        """States of a warm-started batch that end below stop_fidelity are
        swept from their analytic layers; each state keeps the better run."""
        fid = torch.sqrt(ov[0::2] ** 2 + ov[1::2] ** 2) / torch.sqrt(nn[0::2])
        if not bool((fid < stop_fidelity).any().item()):
            return gates, sf, sd, ov
        sf2, sd2 = self.stage_sweeps(p, target, analytic, arity, nl, num_sweeps, stop_fidelity, reuse="fb")
        ov2 = self.overlap(p, self.stage_circuit(p, analytic, arity, nl, reuse="fb"), sv, reuse="fb")
        fid2 = torch.sqrt(ov2[0::2] ** 2 + ov2[1::2] ** 2) / torch.sqrt(nn[0::2])
        take = (fid < stop_fidelity) & (fid2 > fid)                       # per state
        per_slot = torch.repeat_interleave(take, torch.as_tensor(
            [p.max_layers * n * 32 for n in p.nqubits], device=take.device))
        gates = torch.where(per_slot, analytic, gates)
        S = max(int(num_sweeps), 0)
        if S > 0:
            sf = torch.where(torch.repeat_interleave(take, S)[: sf.numel()], sf2, sf)
        sd = torch.where(take, sd2, sd)
        ov = torch.where(torch.repeat_interleave(take, 2), ov2, ov)
        return gates, sf, sd, ov

    @staticmethod
    def _sp(stream) -> ctypes.c_void_p:
        st = stream or torch.cuda.current_stream()
        return ctypes.c_void_p(st.cuda_stream)

    def _stage_input(self, p: Plan, host: torch.Tensor) -> torch.Tensor:
        """Copy a packed host buffer into the plan's own device input buffer
        (``qmprs_plan_upload``: one cudaMalloc per plan, reused) on the
        current stream and return a tensor view of it.  The current stream
        first waits for the previous call's last use of that buffer."""
        if host.dtype != p.vdtype or not host.is_contiguous():
            raise ValueError(f"packed statevectors must be a contiguous {p.vdtype} tensor")
        cur = torch.cuda.current_stream()
        ev = getattr(p, "input_free", None)
        if ev is not None:
            cur.wait_event(ev)
        dev = ctypes.c_void_p()
        self.hd.check(self.lib.qmprs_plan_upload(p.p, ctypes.c_void_p(host.data_ptr()),
                                                 host.numel() * host.element_size(),
                                                 ctypes.c_void_p(cur.cuda_stream), ctypes.byref(dev)))
        p.input_ptr = dev.value
        typestr = "<f8" if p.precision == "exact" else "<f4"
        return torch.as_tensor(_DeviceBuffer(dev.value, host.numel(), typestr), device="cuda")

    @staticmethod
    def _release_input(p: Plan, sv: torch.Tensor) -> None:
        """Mark the end of this call's use of the plan's input buffer."""
        if getattr(p, "input_ptr", None) == sv.data_ptr():
            p.input_free = torch.cuda.Event()
            p.input_free.record(torch.cuda.current_stream())

    # ---- whole path ------------------------------------------------------------
    def encode(self, statevectors, bond_dimension: int, num_layers: int = 1, num_sweeps: int = 0,
               fidelity_threshold: float = 1 - 1e-6, stop_fidelity: float = 0.0,
               keep_tensors: bool = False, nqubits=None, download: bool = True, warm_start=None,
               precision: str = "fast") -> BatchResult:
        """``prepare_state`` for a batch: (a) -> (b)+(c) -> (d) -> fidelity.

        ``statevectors`` is either a list of complex arrays, or (with
        ``nqubits``) one packed float32 tensor holding the complex64
        amplitudes of all states back to back, resident on the GPU or in
        (pinned) host memory.  Inputs need not be normalised: the reported
        fidelity is ``|<sv|C|0>| / ||sv||``.

        ``warm_start`` (a ``warmstart.WarmStartMLP``) replaces the analytic
        layers by the network's predictions before the sweeps; with
        ``stop_fidelity > 0`` every state that ends below it is swept again
        from its analytic layers (the plain method) and keeps the better of
        the two results.

        The stage outputs live in buffers kept on the plan (``Plan.buf``),
        so that repeated calls replay the library's stage graphs; with
        ``download=False`` the returned device tensors are those buffers and
        stay valid until the next ``encode`` on the same plan.

        ``precision="exact"`` runs the double-float mode
        (``QMPRS_PRECISION_EXACT``): a packed buffer is then float64 pairs
        (complex128), and the per-layer and per-sweep fidelities follow an
        FP64 run of the reference's algorithm.
        """
        if nqubits is None:
            p, sv = self.upload(statevectors, num_layers, bond_dimension, precision, reuse=True)
        else:
            p = self.plan(nqubits, num_layers, bond_dimension, precision)
            sv = statevectors
            if sv.numel() != 2 * p.vec_elems or sv.dtype != p.vdtype:
                raise ValueError("packed statevector buffer does not match the qubit counts and precision")
            if not sv.is_cuda:
                sv = self._stage_input(p, sv)
        tensors, bonds, target = self.stage_mps(p, sv, bond_dimension, reuse=True)
        gates, arity, nl, lf = self.stage_layers(p, target, num_layers, fidelity_threshold, reuse=True)
        analytic = None
        if warm_start is not None:
            from . import warmstart as _ws
            analytic = p.buf("analytic", gates.numel(), gates.dtype)
            analytic.copy_(gates)
            _ws.predict_layers(warm_start, gates, p.gate_off, p.nqubits, nl.cpu().numpy())
        sf, sd = self.stage_sweeps(p, target, gates, arity, nl, num_sweeps, stop_fidelity, reuse="main")
        circ = self.stage_circuit(p, gates, arity, nl, reuse="main")
        ov = self.overlap(p, circ, sv, reuse="ov")
        nn = self.overlap(p, sv, sv, reuse="nn")
        if analytic is not None and stop_fidelity > 0.0:
            gates, sf, sd, ov = self._fallback(p, target, sv, analytic, gates, arity, nl, sf, sd, ov, nn,
                                               num_sweeps, stop_fidelity)
        self._release_input(p, sv)
        B, S = p.B, max(int(num_sweeps), 0)
        if not download:
            return BatchResult(nqubits=p.nqubits, gates=gates, arity=arity, num_layers=nl, layer_fidelities=lf,
                               sweep_fidelities=sf, sweeps_done=sd, fidelity=torch.stack([ov, nn]),
                               gate_off=p.gate_off, max_n=p.max_n, max_bond=int(bond_dimension))
        torch.cuda.current_stream().synchronize()
        ovh = ov.cpu().numpy().view(np.complex128)
        nnh = nn.cpu().numpy().view(np.complex128).real
        res = BatchResult(
            nqubits=p.nqubits,
            gates=gates.cpu().numpy().view(np.complex128),
            arity=arity.cpu().numpy(),
            num_layers=nl.cpu().numpy(),
            layer_fidelities=lf.cpu().numpy().view(np.complex128).reshape(B, num_layers),
            sweep_fidelities=sf.cpu().numpy()[: B * S].reshape(B, S),
            sweeps_done=sd.cpu().numpy(),
            fidelity=np.abs(ovh) / np.sqrt(nnh),
            gate_off=p.gate_off,
            max_n=p.max_n,
            max_bond=int(bond_dimension),
        )
        if keep_tensors:
            res.tensors = tensors.cpu().numpy().view(np.complex128)
            res.tensor_off = p.tensor_off
            res.bonds = bonds.cpu().numpy()
        return res


_engine = None


def engine() -> Engine:
    global _engine
    if _engine is None:
        _engine = Engine()
    return _engine
