"""A fixed warm-start network workload, for profiler captures.

    python -m qmprs_gb300.profile_mlp --rows 65536 --steps 3

runs `--steps` training steps (forward, loss, backward, Adam) of the
warm-start network on seeded random features and targets, then one forward
pass; every matmul is ``qmprs_gemm_bf16`` (tcgen05).  It is the command the
committed profiler summaries of the network kernels were taken with.
"""

from __future__ import annotations

import argparse
import time

import numpy as np
import torch


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()
    from qmprs_gb300 import warmstart as W
    rng = np.random.default_rng(args.seed)
    x = torch.as_tensor(rng.standard_normal((args.rows, W.DIMS[0])).astype(np.float32) * 0.5, device="cuda")
    y = torch.as_tensor(rng.standard_normal((args.rows, 32)).astype(np.float32) * 0.3, device="cuda")
    w = torch.ones(args.rows, device="cuda")
    model = W.WarmStartMLP(seed=args.seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        model.forward(x, train=True)
        loss, grads = model.backward(y, w)
        model.adam(grads, 1e-3)
    out = model.forward(x)
    torch.cuda.synchronize()
    model.check_errors()
    dt = time.perf_counter() - t0
    print(f"rows={args.rows} steps={args.steps} loss={loss:.5f} out_norm={float(out.norm()):.4f} wall={dt:.3f}s")


if __name__ == "__main__":
    main()
