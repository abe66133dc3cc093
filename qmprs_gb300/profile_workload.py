"""A fixed encode of a batched random-MPS workload, for profiler captures.

    python -m qmprs_gb300.profile_workload --states 32 --sweeps 2

runs statevector -> MPS -> layers -> sweeps once for ``--states`` random-MPS
statevectors (qubits uniform in {12..22}, bond uniform in {4, 8, 16, 32},
seeded), bond_dimension 64, 6 layers.  ``--precision exact`` runs the
double-float mode (complex128 input); ``--host-input`` enters through
``Sequential.prepare_states`` from pinned host memory (the plan's upload
kernel) instead of a device buffer.  It is the command the committed
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
    ap.add_argument("--precision", default="fast", choices=["fast", "exact"])
    ap.add_argument("--host-input", action="store_true")
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
    if args.precision == "exact":
        sv = sv.view(torch.complex64).to(torch.complex128).view(torch.float64)
    if args.host_input:
        from qmprs_gb300.circuit import Circuit
        from qmprs_gb300.synthesis.mps_encoding import Sequential
        host = torch.empty(sv.numel(), dtype=sv.dtype, pin_memory=True)
        host.copy_(sv)
        _, res = Sequential(Circuit).prepare_states(host, 64, args.layers, args.sweeps, emit=False, nqubits=ns,
                                                    precision=args.precision)
    else:
        res = eng.encode(sv, 64, num_layers=args.layers, num_sweeps=args.sweeps, nqubits=ns,
                         precision=args.precision)
    torch.cuda.synchronize()
    print(f"states={len(ns)} amplitudes={sum(2 ** n for n in ns)} mean_fidelity={float(np.mean(res.fidelity)):.4f}")


if __name__ == "__main__":
    main()
