"""FP64 oracle fixtures of the large configurations (per-layer and per-sweep
fidelities only; the inputs are regenerated from their seeds).

* ``c2_n20.npz``      20 qubits, re/im i.i.d. U[0,1) (``oracle.states.uniform_complex``,
                      seed 5), bond 256, 10 layers, 20 sweeps.
* ``c4_sample.npz``   8 states of the benchmark batch (512 random-MPS states,
                      qubits U{12..22}, bonds U{4,8,16,32}, ``bench.workload_spec``
                      seed 2024, drawn as ``oracle.states.random_mps_batch`` with
                      seed 2024), bond 64, 6 layers, 10 sweeps.
* ``c3_n24.npz``      24 qubits, 3-component Gaussian mixture with random
                      phases (``oracle.states.gaussian_mixture``, seed 3), bond
                      1024, 8 layers, 2 sweeps (the configuration's 10 sweeps
                      take hours in the dense FP64 oracle).

Minutes to about an hour of CPU time (numpy).  Run from the repository root:
    python tests/golden/make_large_golden.py [c2|c4|c3 ...]
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dense as D  # noqa: E402
from oracle import states as S  # noqa: E402

C4_SEED = 2024
# two states from each qubit band of the batch, the widest ones included
C4_PICK_N = (12, 14, 16, 17, 18, 19, 20, 22)


def c4_indices():
    import bench
    ns, bonds, _, _ = bench.workload_spec("batched", 512, C4_SEED)
    idx = []
    for n in C4_PICK_N:
        idx.append(next(i for i, m in enumerate(ns) if m == n))
    return ns, bonds, idx


def encode(sv, chi, L, S_):
    n = D.num_qubits(sv)
    ts = D.tt_svd_right(sv / np.linalg.norm(sv), n, chi)
    t = D.mps_to_dense(ts)
    layers, lf = D.get_unitary_layers(t, n, L)
    sf = []
    for _ in range(S_):
        layers, f = D.sweep(t, n, layers)
        sf.append(f)
    psi = D.circuit_state(layers, n)
    fid = abs(np.vdot(psi, sv)) / np.linalg.norm(sv)
    return np.array(lf), np.array(sf), np.array([x.shape[2] for x in ts[:-1]]), fid


def make_c2():
    n, seed, chi, L, S_ = 20, 5, 256, 10, 20
    lf, sf, bonds, fid = encode(S.uniform_complex(n, seed), chi, L, S_)
    np.savez(os.path.join(HERE, "c2_n20.npz"), n=n, seed=seed, chi=chi, L=L, S=S_, layer_fid=lf, sweep_fid=sf,
             bonds=bonds, fidelity=fid)


def make_c4():
    ns, bonds, idx = c4_indices()
    svs = S.random_mps_batch(ns, bonds, C4_SEED, idx)
    chi, L, S_ = 64, 6, 10
    lfs = np.zeros((len(idx), L), complex)
    sfs = np.zeros((len(idx), S_))
    nl = np.zeros(len(idx), np.int64)
    fids = np.zeros(len(idx))
    for k, sv in enumerate(svs):
        lf, sf, _, fid = encode(sv, chi, L, S_)
        lfs[k, : len(lf)] = lf
        nl[k] = len(lf)
        sfs[k] = sf
        fids[k] = fid
        print("c4", k, ns[idx[k]], flush=True)
    np.savez(os.path.join(HERE, "c4_sample.npz"), seed=C4_SEED, indices=np.array(idx),
             nqubits=np.array([ns[i] for i in idx]), bond=np.array([bonds[i] for i in idx]), chi=chi, L=L, S=S_,
             layer_fid=lfs, num_layers=nl, sweep_fid=sfs, fidelity=fids)


def make_c3():
    n, seed, chi, L, S_ = 24, 3, 1024, 8, 2
    lf, sf, bonds, fid = encode(S.gaussian_mixture(n, seed), chi, L, S_)
    np.savez(os.path.join(HERE, "c3_n24.npz"), n=n, seed=seed, chi=chi, L=L, S=S_, layer_fid=lf, sweep_fid=sf,
             bonds=bonds, fidelity=fid)


if __name__ == "__main__":
    which = sys.argv[1:] or ["c2", "c4", "c3"]
    for w in which:
        t0 = time.time()
        {"c2": make_c2, "c4": make_c4, "c3": make_c3}[w]()
        print(w, "done", time.time() - t0, flush=True)
