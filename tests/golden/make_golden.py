"""Generate the golden fixtures of tests/golden/ from the FP64 oracle.

The reference ships no golden vectors and cannot run here (quimb and
quick-core are absent), so the fixtures are produced by the oracle's dense
restatement in canonical conventions, whose agreement with the call-by-call
MPS restatement and with the reference's published behaviours is asserted in
tests/test_oracle.py.  Inputs are stored as complex64 (what the GPU reads);
the oracle runs on them upcast to complex128.

Run from the repository root:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dense as D  # noqa: E402
from oracle import states as S  # noqa: E402


def c64(v):
    v = np.asarray(v, dtype=np.complex64)
    return v


def up(v):
    v = v.astype(np.complex128)
    return v / np.linalg.norm(v)


def flat_gates(layers):
    gs = D.circuit_gates(layers)
    mats = np.zeros((len(gs), 16), dtype=np.complex128)
    meta = np.zeros((len(gs), 4), dtype=np.int64)
    for i, (li, bi, ti, q, g) in enumerate(gs):
        mats[i, : g.size] = g.reshape(-1)
        meta[i] = (li, bi, ti, q if g.shape[0] == 4 else -1 - q)
    return mats, meta


def ghz_like(n, pairs, plus):
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    t = psi.reshape([2] * n)
    for q in plus:
        t = np.moveaxis(np.tensordot(h, np.moveaxis(t, n - 1 - q, 0), axes=1), 0, n - 1 - q)
    for a, b in pairs:     # CX, control a, target b (little-endian labels)
        t = t.copy()
        ax_a, ax_b = n - 1 - a, n - 1 - b
        idx1 = [slice(None)] * n
        idx1[ax_a] = 1
        sub = t[tuple(idx1)]
        bx = ax_b - (1 if ax_b > ax_a else 0)
        t[tuple(idx1)] = np.flip(sub, axis=bx)
    return t.reshape(-1)


def main():
    out = {}
    # (a) statevector -> MPS, truncated and exact
    for name, n, chi, seed in [("sv_to_mps_n8_chi4", 8, 4, 1), ("sv_to_mps_n9_chi64", 9, 64, 2)]:
        sv = c64(S.uniform_complex(n, seed))
        ts = D.tt_svd_right(up(sv), n, chi)
        out[name] = dict(sv=sv, chi=chi, target=D.mps_to_dense(ts),
                         shapes=np.array([t.shape for t in ts]),
                         tensors=np.concatenate([t.reshape(-1) for t in ts]))
    # (b)+(c) layers
    sv = c64(S.uniform_complex(7, 3))
    t = D.mps_to_dense(D.tt_svd_right(up(sv), 7, 64))
    layers, fids = D.get_unitary_layers(t, 7, 3)
    mats, meta = flat_gates(layers)
    out["layers_n7_L3"] = dict(sv=sv, chi=64, L=3, layer_fid=np.array(fids), gates=mats, meta=meta)
    # (d) sweeps from those layers
    fs = []
    for _ in range(4):
        layers, f = D.sweep(t, 7, layers)
        fs.append(f)
    mats, meta = flat_gates(layers)
    out["sweeps_n7_L3_S4"] = dict(sv=sv, chi=64, L=3, S=4, sweep_fid=np.array(fs), gates=mats, meta=meta)
    # whole path, truncated target
    sv = c64(S.uniform_complex(8, 4))
    r = D.prepare_state(up(sv), 16, 4, 3)
    out["encode_n8_chi16_L4_S3"] = dict(sv=sv, chi=16, L=4, S=3, layer_fid=np.array(r.layer_fidelities),
                                        sweep_fid=np.array(r.sweep_fidelities), fidelity=r.fidelity)
    # partially entangled state (block structure)
    sv = c64(ghz_like(8, [(0, 3), (5, 7)], [0, 4, 5]))
    r = D.prepare_state(up(sv), 32, 1, 0)
    blocks = np.array([(s, e) for s, e, _ in r.layers[0]])
    out["partial_entanglement_n8"] = dict(sv=sv, chi=32, L=1, blocks=blocks, fidelity=r.fidelity,
                                          layer_fid=np.array(r.layer_fidelities))
    # uneven batch
    ns = [5, 9, 12]
    svs = [c64(S.random_mps(n, 4, 10 + n)) for n in ns]
    fids, lfs, sfs = [], [], []
    for sv in svs:
        r = D.prepare_state(up(sv), 16, 3, 2)
        fids.append(r.fidelity)
        lfs.append(np.abs(r.layer_fidelities[-1]))
        sfs.append(r.sweep_fidelities)
    out["batch_uneven"] = dict(ns=np.array(ns), sv=np.concatenate(svs), chi=16, L=3, S=2,
                               fidelity=np.array(fids), sweep_fid=np.array(sfs), last_layer_fid=np.array(lfs))
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print("wrote", name)


if __name__ == "__main__":
    main()
