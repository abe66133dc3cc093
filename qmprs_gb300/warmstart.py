"""Learned warm start for the sequential encoder (no reference counterpart).

The reference initialises every unitary layer analytically (Ran's
construction, ``qmprs/primitives/mps.py:849-891``) and then sweeps.  Here a
small network predicts every gate of the layers from the gate's analytic
initial value, the analytic gates around it (two sites either side, the
same site in the neighbouring layers) and a position embedding.  The predicted matrices are projected to
unitaries (polar factor, null space completed towards the analytic gate) and
replace the analytic ones; all gates are replaced together because the
converged gates are one solution up to gauge, and mixing solutions breaks
the circuit.  The sweeps then start
from the predicted layers, and the exact overlap decides acceptance (a state
that misses the target fidelity continues with the plain method).

Network: 128 -> 256 -> 256 -> 256 -> 32, GELU, BF16 weights and
activations, FP32 accumulation, residual output (the prediction is the
block's analytic gate plus the network's correction, so an untrained network
reproduces the analytic layers), trained with Adam on one of two losses:

* the circuit fidelity |<t|C|0>|^2 / <t|t> of the predicted layers
  (``train_overlap``): every gate's environment at the projected circuit
  (``qmprs_layer_environments``, the sweep's own kernels without the update)
  is the derivative of the overlap with respect to that gate, and
  ``qmprs_mlp_overlap_grad`` carries it through the polar projection to the
  network output;
* the phase-invariant gate loss min_phi |Y - e^{i phi} U|_F^2 against the
  gates after the plain path's sweeps (``WarmStartMLP.train``), which learns
  the gate map but loses circuit fidelity: per-gate errors add up coherently
  over the circuit.

Every matmul runs on the tensor cores through ``qmprs_gemm_bf16``
(tcgen05.mma); losses, activation backward, bias gradients and the optimiser
are the library's own kernels.  PyTorch only allocates device memory and
gathers features.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N

DIMS = (256, 256, 256, 256, 32)
FEAT = 237            # used feature columns (the rest is zero padding)
MAX_LAYERS_EMB = 8    # one-hot layer embedding size


def _p(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _check(code: int, what: str) -> None:
    if code != N.OK:
        raise N.NativeError(code, f"{what} failed with status {code}")


def _pad128(b: int) -> int:
    return max(128, (b + 127) // 128 * 128)


# ---- features -------------------------------------------------------------------

def block_index(nqubits, nlayers):
    """(state, layer, site) of every gate of the generated layers: sites
    0..n-2 hold two-qubit gates, site n-1 the single-qubit gate (the layout
    of Ran's layers)."""
    rows = []
    for b, (n, L) in enumerate(zip(nqubits, nlayers)):
        for l in range(int(L)):
            for s in range(n):
                rows.append((b, l, s))
    return np.asarray(rows, dtype=np.int64).reshape(-1, 3)


def block_kind(nqubits, blocks: np.ndarray) -> np.ndarray:
    """Qubits of each block's gate (2, or 1 at the last site), int8."""
    nq = np.asarray(nqubits, np.int64)
    return np.where(blocks[:, 2] == nq[blocks[:, 0]] - 1, 1, 2).astype(np.int8)


def features(gates: torch.Tensor, gate_off, nqubits, nlayers, blocks: np.ndarray, device) -> torch.Tensor:
    """Feature rows (len(blocks) x 128, float32) on the device.

    gates: the plan's gate store as interleaved float64 (16 complex entries
    per (state, layer, site) slot); nlayers: generated layers per state.
    Columns (32 reals per gate, zero where the block does not exist): the
    block's gate; the two-qubit gates one and two sites to the left and to
    the right in the same layer; the gate of the same site in the previous
    and the next generated layer; then a one-hot layer index (8), the
    position s / (n - 2), n / 30, first / last two-qubit block flags and a
    single-qubit flag (the gate of site n - 1, 2 x 2 in the slot's first four
    entries).
    """
    g = gates.reshape(-1, 32).float()   # one row per slot
    off = torch.as_tensor(np.asarray(gate_off, np.int64) // 16, device=device)
    nq = torch.as_tensor(np.asarray(nqubits, np.int64), device=device)
    bl = torch.as_tensor(blocks, device=device)
    b, l, s = bl[:, 0], bl[:, 1], bl[:, 2]
    n = nq[b]
    nl = torch.as_tensor(np.asarray(nlayers, np.int64), device=device)[b]
    slot = off[b] + l * n + s
    zero = torch.zeros(1, 32, device=device)

    def pick(ok, sl):
        return torch.where(ok[:, None], g[torch.where(ok, sl, slot)], zero)

    x = torch.zeros(len(blocks), DIMS[0], device=device)
    x[:, 0:32] = g[slot]
    x[:, 32:64] = pick(s >= 1, slot - 1)
    x[:, 64:96] = pick(s + 1 <= n - 1, slot + 1)
    x[:, 96:128] = pick(s >= 2, slot - 2)
    x[:, 128:160] = pick(s + 2 <= n - 1, slot + 2)
    x[:, 160:192] = pick(l >= 1, slot - n)
    x[:, 192:224] = pick(l + 1 < nl, slot + n)
    x[torch.arange(len(blocks), device=device), 224 + l.clamp(max=MAX_LAYERS_EMB - 1)] = 1.0
    x[:, 232] = s.float() / (n - 2).clamp(min=1).float()
    x[:, 233] = n.float() / 30.0
    x[:, 234] = (s == 0).float()
    x[:, 235] = (s == n - 2).float()
    x[:, 236] = (s == n - 1).float()
    return x


def targets(gates: torch.Tensor, gate_off, nqubits, blocks: np.ndarray, device) -> torch.Tensor:
    """The blocks' gates as (len(blocks) x 32) float32 rows."""
    g = gates.reshape(-1, 32).float()
    off = torch.as_tensor(np.asarray(gate_off, np.int64) // 16, device=device)
    nq = torch.as_tensor(np.asarray(nqubits, np.int64), device=device)
    bl = torch.as_tensor(blocks, device=device)
    return g[off[bl[:, 0]] + bl[:, 1] * nq[bl[:, 0]] + bl[:, 2]]


# ---- network ----------------------------------------------------------------------

@dataclass
class _Buf:
    B: int
    X: torch.Tensor        # bf16 [B x 128]
    Xf: torch.Tensor       # fp32 [B x 128] (the residual: the block's own gate)
    XT: torch.Tensor       # bf16 [128 x B]
    Z: list                # fp32 pre-activations per layer
    H: list                # bf16 activations (hidden layers)
    HT: list               # bf16 transposed activations
    Y: torch.Tensor        # fp32 [B x 32]
    dY: torch.Tensor
    dYb: torch.Tensor
    dYT: torch.Tensor
    dH: torch.Tensor       # fp32 [B x 256]
    dZ: torch.Tensor
    dZb: torch.Tensor
    dZT: torch.Tensor
    loss: torch.Tensor
    part: torch.Tensor     # split-K partials


class WarmStartMLP:
    """The warm-start network; parameters live on the device."""

    def __init__(self, seed: int = 0, device: str = "cuda"):
        self.device = device
        self.lib = N.load()
        rng = np.random.default_rng(seed)
        self.W, self.b, self.mW, self.vW, self.mb, self.vb, self.Wb, self.WTb = [], [], [], [], [], [], [], []
        for i in range(len(DIMS) - 1):
            fan_in = DIMS[i] if i else FEAT
            w = (rng.standard_normal((DIMS[i + 1], DIMS[i])) * np.sqrt(2.0 / fan_in)).astype(np.float32)
            if i == len(DIMS) - 2:
                w[:] = 0.0   # an untrained network reproduces the analytic layers exactly
            self._add_layer(torch.as_tensor(w, device=device), torch.zeros(DIMS[i + 1], device=device))
        self.step_count = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=device)
        self._bufs = {}

    def _add_layer(self, w: torch.Tensor, b: torch.Tensor) -> None:
        self.W.append(w.contiguous())
        self.b.append(b.contiguous())
        self.mW.append(torch.zeros_like(w))
        self.vW.append(torch.zeros_like(w))
        self.mb.append(torch.zeros_like(b))
        self.vb.append(torch.zeros_like(b))
        self.Wb.append(w.to(torch.bfloat16).contiguous())
        self.WTb.append(w.t().contiguous().to(torch.bfloat16))

    # parameters as numpy (oracle checks, saving)
    def params(self):
        return [(w.cpu().numpy(), b.cpu().numpy()) for w, b in zip(self.W, self.b)]

    def load_params(self, params) -> None:
        self.W, self.b, self.mW, self.vW, self.mb, self.vb, self.Wb, self.WTb = [], [], [], [], [], [], [], []
        for w, b in params:
            self._add_layer(torch.as_tensor(np.asarray(w, np.float32), device=self.device),
                            torch.as_tensor(np.asarray(b, np.float32), device=self.device))

    def save(self, path: str) -> None:
        arrs = {}
        for i, (w, b) in enumerate(self.params()):
            arrs[f"W{i}"] = w
            arrs[f"b{i}"] = b
        np.savez_compressed(path, **arrs)

    @classmethod
    def load(cls, path: str, device: str = "cuda") -> "WarmStartMLP":
        z = np.load(path)
        m = cls(device=device)
        m.load_params([(z[f"W{i}"], z[f"b{i}"]) for i in range(len(DIMS) - 1)])
        return m

    def _buf(self, B: int) -> _Buf:
        if B in self._bufs:
            return self._bufs[B]
        d, bf, f = self.device, torch.bfloat16, torch.float32
        hid = DIMS[1:-1]
        buf = _Buf(
            B=B,
            X=torch.zeros(B, DIMS[0], dtype=bf, device=d),
            Xf=torch.zeros(B, DIMS[0], dtype=f, device=d),
            XT=torch.zeros(DIMS[0], B, dtype=bf, device=d),
            Z=[torch.zeros(B, k, dtype=f, device=d) for k in DIMS[1:]],
            H=[torch.zeros(B, k, dtype=bf, device=d) for k in hid],
            HT=[torch.zeros(k, B, dtype=bf, device=d) for k in hid],
            Y=torch.zeros(B, DIMS[-1], dtype=f, device=d),
            dY=torch.zeros(B, DIMS[-1], dtype=f, device=d),
            dYb=torch.zeros(B, DIMS[-1], dtype=bf, device=d),
            dYT=torch.zeros(DIMS[-1], B, dtype=bf, device=d),
            dH=torch.zeros(B, max(hid), dtype=f, device=d),
            dZ=torch.zeros(B, max(hid), dtype=f, device=d),
            dZb=torch.zeros(B, max(hid), dtype=bf, device=d),
            dZT=torch.zeros(max(hid), B, dtype=bf, device=d),
            loss=torch.zeros(B, dtype=f, device=d),
            # split-K partials: ceil(K / 512) blocks of M x N for K = B (the
            # backward GEMMs), as qmprs_gemm_bf16 requires
            part=torch.zeros(max(1, -(-B // 512)) * max(DIMS) * max(DIMS), dtype=f, device=d),
        )
        self._bufs[B] = buf
        return buf

    def _gemm(self, A, lda, Bm, ldb, M, Nn, K, bias=None, act=0, Cf=None, ldc=0, Cb=None, CbT=None, ldt=0,
              ksplit=0, part=None, resid=None, ldr=0, stream=None):
        code = self.lib.qmprs_gemm_bf16(_p(A), lda, _p(Bm), ldb, M, Nn, K, ksplit, _p(bias), _p(resid), ldr, act,
                                        _p(Cf), ldc, _p(Cb), _p(CbT), ldt, _p(part), _p(self.err), _sp(stream))
        _check(code, "qmprs_gemm_bf16")

    def forward(self, x: torch.Tensor, train: bool = False, stream=None) -> torch.Tensor:
        """x: (rows x 128) float32 features; returns (rows x 32) float32."""
        rows = x.shape[0]
        B = _pad128(rows)
        buf = self._buf(B)
        buf.Xf.zero_()
        buf.Xf[:rows] = x
        buf.X.copy_(buf.Xf)
        if train:
            buf.XT.copy_(buf.X.t())
        h = buf.X
        nl = len(DIMS) - 1
        for j in range(nl):
            last = j == nl - 1
            self._gemm(h, DIMS[j], self.Wb[j], DIMS[j], B, DIMS[j + 1], DIMS[j], bias=self.b[j],
                       act=0 if last else 1, Cf=buf.Z[j] if not last else buf.Y, ldc=DIMS[j + 1],
                       Cb=None if last else buf.H[j], CbT=(buf.HT[j] if (train and not last) else None), ldt=B,
                       resid=buf.Xf if last else None, ldr=DIMS[0], stream=stream)
            if not last:
                h = buf.H[j]
        return buf.Y[:rows]

    def backward(self, y_target: torch.Tensor, weight: torch.Tensor, stream=None):
        """Loss on the last forward (train=True) batch; returns (mean loss,
        gradients [(dW, db)] as device tensors)."""
        B = _pad128(y_target.shape[0])
        buf = self._buf(B)
        rows = y_target.shape[0]
        U = torch.zeros(B, 32, device=self.device)
        U[:rows] = y_target
        w = torch.zeros(B, device=self.device)
        w[:rows] = weight
        wsum = float(weight.sum().item())
        _check(self.lib.qmprs_mlp_loss(_p(buf.Y), _p(U), _p(w), B, 1.0 / wsum, _p(buf.loss), _p(buf.dY),
                                       _p(buf.dYb), _p(buf.dYT), B, _sp(stream)), "qmprs_mlp_loss")
        grads = self._backprop(buf, B, stream)
        loss = float((buf.loss[:rows].sum() / wsum).item())
        return loss, grads

    def backward_overlap(self, env: torch.Tensor, gates: torch.Tensor, slots: torch.Tensor, kind: torch.Tensor,
                         tinv: torch.Tensor, num_states: int, stream=None, grads: bool = True):
        """Circuit-fidelity loss on the last forward (train=True) batch, whose
        rows were projected into `gates` (qmprs_mlp_project) and whose
        environments at those gates are `env` (qmprs_layer_environments).
        The loss is the batch's mean infidelity 1 - |<t|C|0>|^2 / <t|t> over
        its `num_states` states; returns (per-row fidelity, gradients or
        None when grads is False)."""
        rows = int(slots.shape[0])
        B = _pad128(rows)
        buf = self._buf(B)
        _check(self.lib.qmprs_mlp_overlap_grad(_p(env), _p(gates), _p(slots), _p(kind), _p(tinv), rows, B,
                                               1.0 / float(num_states), _p(buf.loss), _p(buf.dY), _p(buf.dYb),
                                               _p(buf.dYT), B, _sp(stream)), "qmprs_mlp_overlap_grad")
        return buf.loss[:rows], (self._backprop(buf, B, stream) if grads else None)

    def _backprop(self, buf: _Buf, B: int, stream=None):
        """Parameter gradients from dY (and its bf16 copies) in `buf`."""
        nl = len(DIMS) - 1
        grads = [None] * nl
        ksplit = 512 if B > 512 else 0
        # output layer: dW^T = H^T dY  (out = 32 < 128 rows)
        hT = buf.HT[nl - 2]
        dWT = torch.empty(DIMS[nl - 1], DIMS[nl], device=self.device)
        self._gemm(hT, B, buf.dYT, B, DIMS[nl - 1], DIMS[nl], B, Cf=dWT, ldc=DIMS[nl], ksplit=ksplit, part=buf.part,
                   stream=stream)
        db = torch.empty(DIMS[nl], device=self.device)
        _check(self.lib.qmprs_mlp_col_sum(_p(buf.dY), B, DIMS[nl], _p(db), _sp(stream)), "col_sum")
        grads[nl - 1] = (dWT, db, True)
        d_bf, d_w = buf.dYb, DIMS[nl]
        for j in range(nl - 2, -1, -1):
            nout = DIMS[j + 1]
            # dH_j = dZ_{j+1} W_{j+1}
            self._gemm(d_bf, d_w, self.WTb[j + 1], d_w, B, nout, d_w, Cf=buf.dH, ldc=nout, stream=stream)
            _check(self.lib.qmprs_mlp_act_back(_p(buf.dH), _p(buf.Z[j]), B, nout, _p(buf.dZ), _p(buf.dZb),
                                               _p(buf.dZT), B, _sp(stream)), "act_back")
            inT = buf.XT if j == 0 else buf.HT[j - 1]
            dW = torch.empty(nout, DIMS[j], device=self.device)
            self._gemm(buf.dZT, B, inT, B, nout, DIMS[j], B, Cf=dW, ldc=DIMS[j], ksplit=ksplit, part=buf.part,
                       stream=stream)
            dbj = torch.empty(nout, device=self.device)
            _check(self.lib.qmprs_mlp_col_sum(_p(buf.dZ), B, nout, _p(dbj), _sp(stream)), "col_sum")
            grads[j] = (dW, dbj, False)
            # dZb holds dZ_j; the next iteration's first GEMM reads it before
            # act_back overwrites it (stream order)
            d_bf, d_w = buf.dZb, nout
        return grads

    def adam(self, grads, lr: float, b1=0.9, b2=0.999, eps=1e-8, wd=0.0, stream=None) -> None:
        self.step_count += 1
        t = self.step_count
        for j, (dW, db, tr) in enumerate(grads):
            rows, cols = self.W[j].shape
            _check(self.lib.qmprs_mlp_adam(_p(self.W[j]), _p(dW), 1 if tr else 0, _p(self.mW[j]), _p(self.vW[j]),
                                           rows, cols, lr, b1, b2, eps, t, wd, _p(self.Wb[j]), _p(self.WTb[j]),
                                           _sp(stream)), "adam")
            _check(self.lib.qmprs_mlp_adam(_p(self.b[j]), _p(db), 0, _p(self.mb[j]), _p(self.vb[j]), rows, 1, lr,
                                           b1, b2, eps, t, 0.0, None, None, _sp(stream)), "adam")

    def check_errors(self) -> None:
        if int(self.err.item()) != 0:
            raise N.NativeError(N.ERR_CUDA, "a tensor-core wait timed out in the warm-start network")

    def train(self, x: torch.Tensor, y: torch.Tensor, w: torch.Tensor | None = None, epochs: int = 10,
              batch: int = 4096, lr: float = 1e-3, seed: int = 0, log=None) -> list:
        """Minibatch Adam over (x, y); returns the per-epoch mean loss."""
        rows = x.shape[0]
        if w is None:
            w = torch.ones(rows, device=self.device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(rows, generator=g).to(self.device)
            tot, cnt = 0.0, 0
            for i in range(0, rows, batch):
                idx = perm[i:i + batch]
                self.forward(x[idx], train=True)
                loss, grads = self.backward(y[idx], w[idx])
                lr_t = lr * 0.5 * (1 + np.cos(np.pi * (ep * rows + i) / (epochs * rows)))
                self.adam(grads, lr_t)
                tot += loss * len(idx)
                cnt += len(idx)
            hist.append(tot / cnt)
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.5f}")
        self.check_errors()
        return hist


def slots_of(gate_off, nqubits, blocks: np.ndarray) -> np.ndarray:
    """Gate-store slot index (units of 16 complex entries) of every block."""
    off = np.asarray(gate_off, np.int64) // 16
    nq = np.asarray(nqubits, np.int64)
    b, l, s = blocks[:, 0], blocks[:, 1], blocks[:, 2]
    return off[b] + l * nq[b] + s


def predict_layers(model: WarmStartMLP, gates: torch.Tensor, gate_off, nqubits, nlayers, stream=None) -> int:
    """Replace the two-qubit gates of analytic layers by the network's
    predictions (polar-projected, null space towards the analytic gate), in
    place; every gate of the layers is predicted, so the layers stay one
    consistent solution.  Returns the number of gates predicted."""
    blocks = block_index(nqubits, nlayers)
    if len(blocks) == 0:
        return 0
    dev = gates.device
    x = features(gates, gate_off, nqubits, nlayers, blocks, dev)
    y = model.forward(x, stream=stream)
    slots = torch.as_tensor(slots_of(gate_off, nqubits, blocks), device=dev)
    kind = torch.as_tensor(block_kind(nqubits, blocks), device=dev)
    _check(model.lib.qmprs_mlp_project(_p(y), len(blocks), _p(slots), _p(kind), _p(gates), _sp(stream)),
           "qmprs_mlp_project")
    return len(blocks)


def _sp(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


# ---- training on the circuit overlap ------------------------------------------------

@dataclass
class OverlapBatch:
    """One plan's states, prepared for training on the circuit overlap: the
    targets, the analytic layers (features and fallback), the block rows."""
    plan: object
    target: torch.Tensor
    analytic: torch.Tensor      # the analytic gate store (float64 pairs)
    work: torch.Tensor          # gate store the predictions are projected into
    env: torch.Tensor           # environments at `work`
    arity: torch.Tensor
    nl: torch.Tensor
    x: torch.Tensor             # features (rows x 256 float32)
    slots: torch.Tensor         # int64 gate-store slot per row
    kind: torch.Tensor          # int8 qubits per row's gate
    state: torch.Tensor         # int64 state index per row
    tinv: torch.Tensor          # float32 1 / <t|t> per row
    num_states: int


def overlap_batch(eng, p, target: torch.Tensor, gates: torch.Tensor, arity: torch.Tensor,
                  nl: torch.Tensor) -> OverlapBatch:
    """Prepare a plan whose analytic layers are in `gates` (kept unchanged)."""
    dev = gates.device
    nlh = nl.cpu().numpy()
    blocks = block_index(p.nqubits, nlh)
    x = features(gates, p.gate_off, p.nqubits, nlh, blocks, dev)
    tn = eng.overlap(p, target, target)[0::2]
    st = torch.as_tensor(blocks[:, 0], device=dev)
    return OverlapBatch(
        plan=p, target=target, analytic=gates.clone(), work=gates.clone(), env=torch.empty_like(gates),
        arity=arity, nl=nl, x=x, slots=torch.as_tensor(slots_of(p.gate_off, p.nqubits, blocks), device=dev),
        kind=torch.as_tensor(block_kind(p.nqubits, blocks), device=dev), state=st,
        tinv=(1.0 / tn)[st].float().contiguous(), num_states=p.B)


def _state_mean(ob: OverlapBatch, rows: torch.Tensor) -> torch.Tensor:
    """Mean over each state's rows (float64, one entry per state)."""
    s = torch.zeros(ob.num_states, dtype=torch.float64, device=rows.device)
    c = torch.zeros_like(s)
    s.index_add_(0, ob.state, rows.double())
    c.index_add_(0, ob.state, torch.ones_like(rows, dtype=torch.float64))
    return s / c.clamp(min=1)


def overlap_step(eng, model: WarmStartMLP, ob: OverlapBatch, lr: float | None, stream=None) -> torch.Tensor:
    """One Adam step on the batch's mean infidelity 1 - |<t|C|0>|^2 / <t|t>
    of the predicted layers (no step when lr is None); returns each state's
    fidelity before the step."""
    rows = int(ob.slots.shape[0])
    y = model.forward(ob.x, train=lr is not None, stream=stream)
    ob.work.copy_(ob.analytic)   # null directions complete towards the analytic gate
    _check(model.lib.qmprs_mlp_project(_p(y), rows, _p(ob.slots), _p(ob.kind), _p(ob.work), _sp(stream)),
           "qmprs_mlp_project")
    eng.environments(ob.plan, ob.target, ob.work, ob.arity, ob.nl, env=ob.env, stream=stream)
    fid, grads = model.backward_overlap(ob.env, ob.work, ob.slots, ob.kind, ob.tinv, ob.num_states,
                                        stream=stream, grads=lr is not None)
    if lr is not None:
        model.adam(grads, lr, stream=stream)
    return _state_mean(ob, fid)


def train_overlap(eng, model: WarmStartMLP, batches: list, epochs: int, lr: float = 2e-4, log=None,
                  keep_best: bool = True) -> list:
    """Train on the circuit overlap: every epoch takes one step per batch
    (cosine-decayed learning rate).  Returns the mean fidelity of the
    predicted layers over all states per epoch (measured before each step of
    the epoch), then that of the final parameters.  With keep_best the
    parameters of the best entry are restored at the end (the first entry is
    the analytic layers' fidelity, so training never ends below it)."""
    hist, best_f, best_p = [], -1.0, None
    total = epochs * len(batches)
    for ep in range(epochs + 1):
        snap = model.params() if keep_best else None
        fs = []
        for i, ob in enumerate(batches):
            k = ep * len(batches) + i
            lr_k = None if ep == epochs else lr * 0.5 * (1 + np.cos(np.pi * k / total))
            fs.append(overlap_step(eng, model, ob, lr_k))
        hist.append(float(torch.cat(fs).mean().item()))
        if keep_best and hist[-1] > best_f:
            best_f, best_p = hist[-1], snap
        if log:
            log(f"epoch {ep}: mean fidelity of the predicted layers {hist[-1]:.5f}")
    if keep_best and best_p is not None and best_f > hist[-1]:
        model.load_params(best_p)
    model.check_errors()
    return hist
