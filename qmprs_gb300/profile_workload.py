"""A fixed encode of a batched random-MPS workload, for profiler captures.

    python -m qmprs_gb300.profile_workload --states 32 --sweeps 2

runs statevector -> MPS -> layers -> sweeps once for ``--states`` random-MPS
statevectors (qubits uniform in {12..22}, bond uniform in {4, 8, 16, 32},
seeded), bond_dimension 64, 6 layers.  It is the command the committed
profiler summaries were taken with (after the same command had exited 0
without the profiler).
"""

from __future__ import annotations

import argparse

import numpy as np
import torch


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--states", type=int, default=32)
    ap.add_argument("--sweeps", type=int, default=2)
    ap.add_argument("--layers", type=int, default=6)
    ap.add_argument("--qubits", type=int, default=0, help="fixed qubit count (0: uniform 12..22)")
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args()
    from qmprs_gb300 import engine as E
    rng = np.random.default_rng(args.seed)
    if args.qubits:
        ns = [args.qubits] * args.states
    else:
        ns = [int(x) for x in rng.integers(12, 23, size=args.states)]
    bonds = [int(x) for x in rng.choice([4, 8, 16, 32], size=args.states)]
    eng = E.engine()
    sv = eng.random_mps_states(ns, bonds, seed=args.seed)
    res = eng.encode(sv, 64, num_layers=args.layers, num_sweeps=args.sweeps, nqubits=ns)
    torch.cuda.synchronize()
    print(f"states={len(ns)} amplitudes={sum(2 ** n for n in ns)} mean_fidelity={float(np.mean(res.fidelity)):.4f}")


if __name__ == "__main__":
    main()
