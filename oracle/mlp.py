"""FP32/FP64 numpy oracle of the warm-start MLP (test infrastructure only).

The learned warm start has no reference counterpart; this module is the
checker the GPU kernels of ``qmprs_gb300/csrc/mlp.cu`` are held to:

* ``bf16``             round-to-nearest-even to bfloat16 (the GPU's operand
                       precision), kept in float32 storage;
* ``forward``          the network  h_{j} = GELU(h_{j-1} W_j^T + b_j)  for
                       the hidden layers and  y = h W^T + b (+ residual)
                       at the output,
                       with every matmul operand rounded to bf16 and the
                       products accumulated in float64;
* ``loss_and_grad``    the phase-invariant gate loss
                       min_phi |Y - e^{i phi} U|_F^2 = |Y|^2 + |U|^2 - 2|Tr(U^H Y)|
                       per sample (4 x 4 complex, row-major, interleaved)
                       and its gradient;
* ``backward``         parameter gradients of the weighted mean loss.
* ``overlap_grad``     the circuit-overlap loss: per gate row, the state's
                       fidelity |sum U*E|^2 tinv and the gradient of
                       -gscale times it with respect to the network output,
                       through the tangent map of the polar factor at U.

The GELU is the tanh form 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))).
"""

from __future__ import annotations

import numpy as np

C_GELU = np.sqrt(2.0 / np.pi)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C_GELU * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(C_GELU * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * C_GELU * (1.0 + 3.0 * 0.044715 * z * z)


def forward(params, x, residual=None):
    """params: list of (W [out x in], b [out]); returns (y, cache).  With
    ``residual`` (rows x out) the output is h W^T + b + residual."""
    hs = [x]
    zs = []
    h = x
    for j, (w, b) in enumerate(params):
        z = bf16(h).astype(np.float64) @ bf16(w).astype(np.float64).T + b
        if residual is not None and j == len(params) - 1:
            z = z + residual
        zs.append(z)
        h = gelu(z) if j < len(params) - 1 else z
        if j < len(params) - 1:
            hs.append(h)
    return h, (hs, zs)


def loss_and_grad(y, u, w):
    """Per-sample loss and d(sum_s w_s loss_s / sum w)/dy for y, u (B x 32)."""
    yc = y[:, 0::2] + 1j * y[:, 1::2]
    uc = u[:, 0::2] + 1j * u[:, 1::2]
    tr = np.sum(np.conj(uc) * yc, axis=1)
    at = np.abs(tr)
    loss = w * (np.sum(np.abs(yc) ** 2, axis=1) + np.sum(np.abs(uc) ** 2, axis=1) - 2 * at)
    ph = np.where(at > 0, tr / np.where(at > 0, at, 1), 1.0)
    g = 2 * (yc - ph[:, None] * uc) * (w / np.sum(w))[:, None]
    dy = np.empty_like(y)
    dy[:, 0::2] = g.real
    dy[:, 1::2] = g.imag
    return loss, dy


def backward(params, cache, dy):
    """Gradients [(dW, db)] of the loss whose output gradient is dy."""
    hs, zs = cache
    grads = [None] * len(params)
    d = dy
    for j in range(len(params) - 1, -1, -1):
        w, _ = params[j]
        if j < len(params) - 1:
            d = d * gelu_grad(zs[j])
        dw = bf16(d.astype(np.float32)).astype(np.float64).T @ bf16(hs[j].astype(np.float32)).astype(np.float64)
        db = d.sum(axis=0)
        grads[j] = (dw, db)
        if j > 0:
            d = bf16(d.astype(np.float32)).astype(np.float64) @ bf16(w).astype(np.float64)
    return grads


def init_params(dims, seed: int):
    """Scaled Gaussian weights (variance 2 / fan_in), zero biases, float32."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(len(dims) - 1):
        w = (rng.standard_normal((dims[i + 1], dims[i])) * np.sqrt(2.0 / dims[i])).astype(np.float32)
        out.append((w, np.zeros(dims[i + 1], np.float32)))
    return out


def polar_factor(y: np.ndarray) -> np.ndarray:
    """Unitary polar factor W V^H of y = W S V^H."""
    w, _, vh = np.linalg.svd(y)
    return w @ vh


def overlap_grad(env: np.ndarray, gates: np.ndarray, kind: np.ndarray, tinv: np.ndarray, gscale: float):
    """Circuit-overlap loss rows (the restatement of ``k_mlp_overlap_grad``).

    env, gates: (rows x 16) complex128 slots (m x m row-major in the first
    m*m entries, m = 2 for kind 1, else 4).  With f = sum_ac U[a,c] E[a,c]
    (the state's overlap <t|C|0>) the row's fidelity is F = |f|^2 tinv.  The
    gradient of -gscale F with respect to U, in the complex form
    d/dRe + i d/dIm, is G = -2 gscale tinv f conj(E); the polar factor's
    tangent map at a unitary U carries it to the network output as
    U skew(U^H G), skew(X) = (X - X^H) / 2.  Returns (F, dY) with dY
    (rows x 32) float64, interleaved re/im, zero beyond m*m entries.
    """
    rows = env.shape[0]
    fid = np.zeros(rows)
    dy = np.zeros((rows, 32))
    for r in range(rows):
        m = 2 if kind[r] == 1 else 4
        u = gates[r, : m * m].reshape(m, m)
        e = env[r, : m * m].reshape(m, m)
        f = np.sum(u * e)
        fid[r] = abs(f) ** 2 * tinv[r]
        g = -2.0 * gscale * tinv[r] * f * np.conj(e)
        x = u.conj().T @ g
        gy = u @ (0.5 * (x - x.conj().T))
        flat = gy.reshape(-1)
        dy[r, 0 : 2 * m * m : 2] = flat.real
        dy[r, 1 : 2 * m * m : 2] = flat.imag
    return fid, dy
