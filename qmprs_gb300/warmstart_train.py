"""Train and evaluate the learned warm start.

    python -m qmprs_gb300.warmstart_train --train-states 2048 --out ws.npz

1. Training states: seeded states of a family (--family random_mps: random
   MPS with bond uniform in {8, 16, 32}; gmm: Gaussian mixtures on the
   amplitude grid), qubits uniform in --qmin..--qmax, go through the plain
   GPU path's analytic layers (--layers).
2. --objective overlap (the default): the network is trained on the circuit
   fidelity |<t|C|0>|^2 / <t|t> of its predicted layers.  Every step projects
   the predictions to unitaries, computes every gate's environment at that
   circuit (qmprs_layer_environments), turns them into the gradient
   (qmprs_mlp_overlap_grad) and back-propagates it through the library's
   tensor-core kernels.  --objective gates: the earlier per-gate loss against
   the gates after --sweeps sweeps of the plain path (one pair per block).
3. Evaluation on held-out states (--eval-qubits qubits): the plain path
   (analytic layers, then sweeps) against the warm start (predicted layers,
   then sweeps), fidelity |<target|C|0>| after every sweep, from the same
   targets.  Prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import engine as E
from . import warmstart as W


def _batches(ns, bonds, size):
    for i in range(0, len(ns), size):
        yield ns[i:i + size], bonds[i:i + size]


def gmm_states(ns, seed: int, components: int = 3) -> torch.Tensor:
    """Packed complex64 (interleaved float32) states: on the grid
    x_j = (j + 1/2) / 2^n, a mixture of `components` Gaussians with means
    U[0, 1), widths U[0.02, 0.2], equal weights and a random phase per
    component; normalised."""
    rng = np.random.default_rng(seed)
    parts = []
    for n in ns:
        x = (torch.arange(2 ** n, device="cuda", dtype=torch.float64) + 0.5) / 2 ** n
        psi = torch.zeros(2 ** n, dtype=torch.complex128, device="cuda")
        for _ in range(components):
            mu, sig, ph = rng.uniform(0, 1), rng.uniform(0.02, 0.2), rng.uniform(0, 2 * np.pi)
            psi += torch.exp(-((x - mu) ** 2) / (2 * sig * sig)) * complex(np.cos(ph), np.sin(ph))
        psi /= torch.linalg.vector_norm(psi)
        parts.append(torch.view_as_real(psi.to(torch.complex64)).reshape(-1))
    return torch.cat(parts)


def states(eng, family, nb, bb, seed):
    if family == "gmm":
        return gmm_states(nb, seed)
    return eng.random_mps_states(nb, bb, seed=seed)


def make_pairs(eng, ns, bonds, layers, sweeps, chi, seed, batch=256, log=print, family="random_mps"):
    """Features (analytic layers) and targets (the gates after `sweeps`
    sweeps of the plain path) of every two-qubit block of the given states."""
    xs, ys = [], []
    t0 = time.perf_counter()
    for k, (nb, bb) in enumerate(_batches(ns, bonds, batch)):
        sv = states(eng, family, nb, bb, seed + k)
        p = eng.plan(nb, layers, chi)
        _, _, target = eng.stage_mps(p, sv, chi)
        gates, arity, nl, _ = eng.stage_layers(p, target, layers, 1 - 1e-6)
        analytic = gates.clone()
        eng.stage_sweeps(p, target, gates, arity, nl, sweeps, 0.0)
        nlh = nl.cpu().numpy()
        blocks = W.block_index(nb, nlh)
        xs.append(W.features(analytic, p.gate_off, nb, nlh, blocks, "cuda"))
        ys.append(W.targets(gates, p.gate_off, nb, blocks, "cuda"))
        del sv, target
    torch.cuda.synchronize()
    log(f"pairs: {sum(len(x) for x in xs)} blocks from {len(ns)} states in {time.perf_counter() - t0:.1f} s")
    return torch.cat(xs), torch.cat(ys)


def overlap_batches(eng, ns, bonds, layers, chi, seed, batch=256, log=print, family="random_mps"):
    """Training batches for the circuit-overlap objective: targets and
    analytic layers of the given states, one plan per `batch` states."""
    out = []
    t0 = time.perf_counter()
    for k, (nb, bb) in enumerate(_batches(ns, bonds, batch)):
        sv = states(eng, family, nb, bb, seed + k)
        p = eng.plan(nb, layers, chi)
        _, _, target = eng.stage_mps(p, sv, chi)
        gates, arity, nl, _ = eng.stage_layers(p, target, layers, 1 - 1e-6)
        out.append(W.overlap_batch(eng, p, target, gates, arity, nl))
        del sv
    torch.cuda.synchronize()
    log(f"overlap batches: {sum(int(b.slots.shape[0]) for b in out)} gates of {len(ns)} states "
        f"in {time.perf_counter() - t0:.1f} s")
    return out


def evaluate(eng, model, ns, bonds, layers, sweeps, chi, seed, batch=256, family="random_mps"):
    """Per-sweep fidelities (B x sweeps) of the plain and the warm-started path."""
    plain, warm, init_p, init_w = [], [], [], []
    for k, (nb, bb) in enumerate(_batches(ns, bonds, batch)):
        sv = states(eng, family, nb, bb, seed + k)
        p = eng.plan(nb, layers, chi)
        _, _, target = eng.stage_mps(p, sv, chi)
        gates, arity, nl, _ = eng.stage_layers(p, target, layers, 1 - 1e-6)
        nlh = nl.cpu().numpy()
        g_w = gates.clone()
        W.predict_layers(model, g_w, p.gate_off, nb, nlh)
        tn = eng.overlap(p, target, target).cpu().numpy()[0::2]
        for g, out, init in ((gates, plain, init_p), (g_w, warm, init_w)):
            circ = eng.stage_circuit(p, g, arity, nl)
            ov = eng.overlap(p, circ, target).cpu().numpy().view(np.complex128)
            init.append(np.abs(ov) / np.sqrt(tn))
            sf, _ = eng.stage_sweeps(p, target, g, arity, nl, sweeps, 0.0)
            out.append(sf.cpu().numpy()[: len(nb) * sweeps].reshape(len(nb), sweeps))
        del sv, target
    return np.concatenate(init_p), np.concatenate(plain), np.concatenate(init_w), np.concatenate(warm)


def sweeps_to(curves, thr):
    """First sweep (1-based) whose fidelity reaches thr, inf if none."""
    hit = curves >= thr
    return np.where(hit.any(axis=1), hit.argmax(axis=1) + 1, np.inf)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-states", type=int, default=2048)
    ap.add_argument("--qmin", type=int, default=16)
    ap.add_argument("--qmax", type=int, default=20)
    ap.add_argument("--layers", type=int, default=8)
    ap.add_argument("--sweeps", type=int, default=10)
    ap.add_argument("--chi", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=None, help="default 2e-4 (overlap), 1e-3 (gates)")
    ap.add_argument("--eval-states", type=int, default=256)
    ap.add_argument("--eval-qubits", type=int, default=20)
    ap.add_argument("--eval-sweeps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default="")
    ap.add_argument("--family", default="random_mps", choices=["random_mps", "gmm"])
    ap.add_argument("--objective", default="overlap", choices=["overlap", "gates"])
    ap.add_argument("--state-batch", type=int, default=256, help="states per plan (overlap objective)")
    args = ap.parse_args()
    if args.lr is None:
        args.lr = 2e-4 if args.objective == "overlap" else 1e-3
    eng = E.engine()
    rng = np.random.default_rng(args.seed)
    ns = [int(x) for x in rng.integers(args.qmin, args.qmax + 1, size=args.train_states)]
    bonds = [int(x) for x in rng.choice([8, 16, 32], size=args.train_states)]
    model = W.WarmStartMLP(seed=args.seed)
    if args.objective == "overlap":
        batches = overlap_batches(eng, ns, bonds, args.layers, args.chi, seed=args.seed * 1000,
                                  batch=args.state_batch, family=args.family)
        pairs = sum(int(b.slots.shape[0]) for b in batches)
        t0 = time.perf_counter()
        hist = W.train_overlap(eng, model, batches, epochs=args.epochs, lr=args.lr, log=print)
        del batches
    else:
        x, y = make_pairs(eng, ns, bonds, args.layers, args.sweeps, args.chi, seed=args.seed * 1000,
                          family=args.family)
        pairs = int(x.shape[0])
        t0 = time.perf_counter()
        hist = model.train(x, y, epochs=args.epochs, batch=args.batch, lr=args.lr, log=print)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    if args.out:
        model.save(args.out)
    ens = [args.eval_qubits] * args.eval_states
    ebonds = [int(b) for b in np.random.default_rng(args.seed + 1).choice([8, 16, 32], size=args.eval_states)]
    ip, fp, iw, fw = evaluate(eng, model, ens, ebonds, args.layers, args.eval_sweeps, args.chi,
                              seed=args.seed * 1000 + 777777, family=args.family)
    thr = float(np.median(fp[:, -1]))
    line = {
        "family": args.family, "objective": args.objective, "target_sweeps": args.sweeps,
        "pairs": pairs, "train_states": args.train_states, "epochs": args.epochs, "lr": args.lr,
        "train_seconds": train_s, "history_first": hist[0], "history_last": hist[-1],
        "history_best": max(hist) if args.objective == "overlap" else min(hist),
        "eval_states": args.eval_states, "eval_qubits": args.eval_qubits, "layers": args.layers,
        "init_fidelity_plain": float(ip.mean()), "init_fidelity_warm": float(iw.mean()),
        "fidelity_per_sweep_plain": [float(v) for v in fp.mean(axis=0)],
        "fidelity_per_sweep_warm": [float(v) for v in fw.mean(axis=0)],
        "reached_0.98_plain": int((fp.max(axis=1) >= 0.98).sum()),
        "reached_0.98_warm": int((fw.max(axis=1) >= 0.98).sum()),
        "threshold_median_plain_final": thr,
        "mean_sweeps_to_threshold_plain": float(np.mean(np.minimum(sweeps_to(fp, thr), args.eval_sweeps + 1))),
        "mean_sweeps_to_threshold_warm": float(np.mean(np.minimum(sweeps_to(fw, thr), args.eval_sweeps + 1))),
        "warm_better_final_fraction": float(np.mean(fw[:, -1] > fp[:, -1])),
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
