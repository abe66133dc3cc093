"""Run one of the named single-state configurations end to end.

    python -m qmprs_gb300.run_config --config n10_chi512      # 10 q, chi 512, L 15, S 50
    python -m qmprs_gb300.run_config --config n20_chi256      # 20 q, chi 256, L 10, S 20
    python -m qmprs_gb300.run_config --config n24_chi1024     # 24 q, chi 1024, L 8, S 10

Inputs (seeded synthetic data; the reference names no dataset):
  n10_chi512, n20_chi256  real and imaginary parts i.i.d. uniform[0, 1),
                          L2-normalised;
  n24_chi1024             a 3-component Gaussian mixture on the 2^24 grid
                          points (means uniform in [0, 1), widths uniform in
                          [0.02, 0.2], equal weights) with phases
                          exp(2 pi i u), u uniform[0, 1) per amplitude,
                          L2-normalised.
Prints one JSON line: per-stage times, bonds, the fidelity after every
layer and sweep, and the final |<target|C|0>|.  With --oracle (10 qubits)
the FP64 oracle runs the same encode and the per-sweep differences are
reported.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

CONFIGS = {
    "n10_chi512": dict(n=10, chi=512, layers=15, sweeps=50, family="uniform"),
    "n20_chi256": dict(n=20, chi=256, layers=10, sweeps=20, family="uniform"),
    "n24_chi1024": dict(n=24, chi=1024, layers=8, sweeps=10, family="gmm_phase"),
}


def make_state(n: int, family: str, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if family == "uniform":
        v = rng.uniform(0, 1, 2 ** n) + 1j * rng.uniform(0, 1, 2 ** n)
    else:
        x = (np.arange(2 ** n) + 0.5) / 2 ** n
        amp = np.zeros(2 ** n)
        for _ in range(3):
            mu, sig = rng.uniform(0, 1), rng.uniform(0.02, 0.2)
            amp += np.exp(-((x - mu) ** 2) / (2 * sig * sig))
        v = amp * np.exp(2j * np.pi * rng.uniform(0, 1, 2 ** n))
    return (v / np.linalg.norm(v)).astype(np.complex128)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", required=True, choices=sorted(CONFIGS))
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--sweeps", type=int, default=-1, help="override the configuration's sweeps")
    ap.add_argument("--oracle", action="store_true")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    if args.sweeps >= 0:
        cfg["sweeps"] = args.sweeps
    from qmprs_gb300 import engine as E
    sv = make_state(cfg["n"], cfg["family"], args.seed)
    eng = E.engine()
    p, svd = eng.upload([sv], cfg["layers"], cfg["chi"])
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    tensors, bonds, target = eng.stage_mps(p, svd, cfg["chi"])
    ev[1].record()
    gates, arity, nl, lf = eng.stage_layers(p, target, cfg["layers"], 1 - 1e-6)
    ev[2].record()
    sf, sd = eng.stage_sweeps(p, target, gates, arity, nl, cfg["sweeps"], 0.0)
    ev[3].record()
    circ = eng.stage_circuit(p, gates, arity, nl)
    ov = eng.overlap(p, circ, svd).cpu().numpy().view(np.complex128)
    tn = eng.overlap(p, target, target).cpu().numpy()[0]
    torch.cuda.synchronize()
    S = cfg["sweeps"]
    line = {
        "config": args.config, **cfg, "seed": args.seed,
        "stage_ms": {"mps_from_statevector": ev[0].elapsed_time(ev[1]),
                     "unitary_layers": ev[1].elapsed_time(ev[2]), "sweeps": ev[2].elapsed_time(ev[3])},
        "bonds": [int(x) for x in bonds.cpu().numpy()[: cfg["n"] + 1]],
        "target_norm2": float(tn),
        "num_layers": int(nl.cpu().numpy()[0]),
        "layer_fidelities": [float(abs(x)) for x in lf.cpu().numpy().view(np.complex128)[: int(nl[0])]],
        "sweep_fidelities": [float(x) for x in sf.cpu().numpy()[:S]],
        "fidelity": float(abs(ov[0])),
    }
    if args.oracle:
        from oracle import dense as D
        t0 = time.perf_counter()
        sv64 = sv.astype(np.complex64).astype(np.complex128)
        t = D.mps_to_dense(D.tt_svd_right(sv64 / np.linalg.norm(sv64), cfg["n"], cfg["chi"]))
        layers, fids = D.get_unitary_layers(t, cfg["n"], cfg["layers"])
        fs = []
        for _ in range(S):
            layers, f = D.sweep(t, cfg["n"], layers)
            fs.append(f)
        line["oracle_seconds"] = time.perf_counter() - t0
        line["oracle_sweep_fidelities"] = fs
        line["max_abs_sweep_difference"] = float(np.max(np.abs(np.asarray(fs) - line["sweep_fidelities"])))
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
