"""Run one of the named single-state configurations end to end.

    python -m qmprs_gb300.run_config --config n10_chi512      # 10 q, chi 512, L 15, S 50
    python -m qmprs_gb300.run_config --config n20_chi256      # 20 q, chi 256, L 10, S 20
    python -m qmprs_gb300.run_config --config n24_chi1024     # 24 q, chi 1024, L 8, S 10

Inputs (seeded synthetic data from ``qmprs_gb300.states``; the reference
names no dataset):
  n10_chi512, n20_chi256  real and imaginary parts i.i.d. uniform[0, 1),
                          L2-normalised (``uniform_complex``);
  n24_chi1024             a 3-component Gaussian mixture on the 2^24 grid
                          points (means uniform in [0, 1), widths uniform in
                          [0.02, 0.2], equal weights) with phases
                          exp(2 pi i u), u uniform[0, 1) per amplitude,
                          L2-normalised (``gaussian_mixture``).
``--precision fast|exact`` selects the library's arithmetic (complex64 or
double-float working states).  ``--reference FILE.npz`` compares with the
per-layer and per-sweep fidelities of an FP64 run of the same input stored
in FILE (``layer_fid``, ``sweep_fid``, ``fidelity`` and the configuration:
``n``, ``seed``, ``chi``, ``L``, ``S``), and reports the largest
differences as ``infidelity_vs_fp64``.

Prints one JSON line: per-stage times, bonds, the fidelity after every
layer and sweep, and the final |<sv|C|0>|.
"""

from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import states as ST

CONFIGS = {
    "n10_chi512": dict(n=10, chi=512, layers=15, sweeps=50, family="uniform"),
    "n20_chi256": dict(n=20, chi=256, layers=10, sweeps=20, family="uniform"),
    "n24_chi1024": dict(n=24, chi=1024, layers=8, sweeps=10, family="gmm_phase"),
}


def make_state(n: int, family: str, seed: int) -> np.ndarray:
    if family == "uniform":
        return ST.uniform_complex(n, seed)
    return ST.gaussian_mixture(n, seed)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", required=True, choices=sorted(CONFIGS))
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--sweeps", type=int, default=-1, help="override the configuration's sweeps")
    ap.add_argument("--precision", default="fast", choices=["fast", "exact"])
    ap.add_argument("--reference", default="", help="npz with the FP64 run's fidelities of the same input")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    if args.sweeps >= 0:
        cfg["sweeps"] = args.sweeps
    ref = None
    if args.reference:
        ref = np.load(args.reference)
        want = dict(n=cfg["n"], seed=args.seed, chi=cfg["chi"], L=cfg["layers"], S=cfg["sweeps"])
        have = {k: int(ref[k]) for k in want}
        if have != want:
            raise SystemExit(f"reference {args.reference} is for {have}, this run is {want}")
    from qmprs_gb300 import engine as E
    sv = make_state(cfg["n"], cfg["family"], args.seed)
    eng = E.engine()
    p, svd = eng.upload([sv], cfg["layers"], cfg["chi"], args.precision)
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
    L = int(nl.cpu().numpy()[0])
    lfh = lf.cpu().numpy().view(np.complex128)[:L]
    sfh = sf.cpu().numpy()[:S]
    line = {
        "config": args.config, **cfg, "seed": args.seed, "precision": args.precision,
        "stage_ms": {"mps_from_statevector": ev[0].elapsed_time(ev[1]),
                     "unitary_layers": ev[1].elapsed_time(ev[2]), "sweeps": ev[2].elapsed_time(ev[3])},
        "bonds": [int(x) for x in bonds.cpu().numpy()[: cfg["n"] + 1]],
        "target_norm2": float(tn),
        "num_layers": L,
        "layer_fidelities": [float(abs(x)) for x in lfh],
        "sweep_fidelities": [float(x) for x in sfh],
        "fidelity": float(abs(ov[0])),
    }
    if ref is not None:
        rl = np.asarray(ref["layer_fid"])
        m = min(len(rl), L)
        line["infidelity_vs_fp64"] = {
            "layers_compared": m, "num_layers_fp64": int(len(rl)),
            "max_layer": float(np.max(np.abs(lfh[:m] - rl[:m]))) if m else 0.0,
            "max_sweep": float(np.max(np.abs(sfh - np.asarray(ref["sweep_fid"])[:S]))) if S else 0.0,
            "final": float(abs(abs(ov[0]) - float(ref["fidelity"]))),
        }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
