"""Benchmark of the GB300 MPS-encoding path (one JSON line on rank 0).

Workload (default ``batched``): the batched uneven-size configuration —
512 statevectors, qubit counts uniform in {12..22}, each the contraction of
a random MPS (i.i.d. complex Gaussian tensors, bond uniform in
{4, 8, 16, 32}, left-canonicalised, normalised); encoded with
bond_dimension=64, num_layers=6, num_sweeps=10, sweeps stopping per state at
fidelity 0.98.  Seeded synthetic data (the reference has no dataset).

A step is one pass of the whole path (statevector -> MPS -> layers ->
sweeps -> circuit state -> fidelity) over the batch.

* ``value``  states/s with the inputs resident in HBM (CUDA events on the
  launching stream, barrier + synchronize on both sides, max over ranks).
* ``e2e``    the same through the public batched API
  (``Sequential.prepare_states``) from pinned HOST buffers, with the
  host->device input copy and the device->host result copy timed.
* ``roofline``  the grouped sweep pass (k_group_pass): algorithmic bytes
  (32 B per amplitude of every state the pass touches: read and write psi
  and t; 16 B for a state's first group, which only reads) over its
  event-timed launches in a profiled pass of the same batch, against the
  measured HBM copy bandwidth.
* ``cpu_baseline``  the FP64 oracle's call-by-call restatement of the
  reference (``oracle.mpsops``, literal conventions, one state per process,
  OPENBLAS_NUM_THREADS=1) on a bounded stratified sample; the per-state
  time is extrapolated to the workload's qubit mix with a 2^n cost model.

``--impl reference`` times that CPU path alone on all host cores and prints
its own line (the reference itself cannot be installed here: quimb and
quick-core are absent).  ``--gpus N`` under torchrun runs N independent
replicas (the path does not shard within a state).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "states/sec to fidelity≥0.98: learned warm-start+batched vs plain sweep, 1 GB300"
UNIT = "states/s"
# DRAM bytes (read + write) per algorithmic byte of a k_group_pass launch,
# from an ncu capture of `python -m qmprs_gb300.profile_workload --states 32
# --sweeps 1` (a group-1 launch: dram__bytes_read.sum + dram__bytes_write.sum
# = 371.3 + 311.4 MB against 32 B x 23,195,648 amplitudes); a full-size
# launch is scaled by its algorithmic bytes.
PASS_DRAM_PER_ALG_BYTE = (371.333120e6 + 311.374848e6) / (32.0 * 23195648)


def workload_spec(name: str, states: int, seed: int):
    rng = np.random.default_rng(seed)
    if name == "batched":
        ns = [int(x) for x in rng.integers(12, 23, size=states)]
        bonds = [int(x) for x in rng.choice([4, 8, 16, 32], size=states)]
        cfg = dict(bond_dimension=64, num_layers=6, num_sweeps=10, stop_fidelity=0.98)
        desc = (f"{states} random-MPS states, qubits U{{12..22}}, bond U{{4,8,16,32}}; "
                "chi=64, L=6, S=10, stop at 0.98")
    elif name == "n20":
        ns = [20] * states
        bonds = [int(x) for x in rng.choice([8, 16, 32], size=states)]
        cfg = dict(bond_dimension=64, num_layers=8, num_sweeps=10, stop_fidelity=0.98)
        desc = f"{states} 20-qubit random-MPS states, bond U{{8,16,32}}; chi=64, L=8, S=10, stop at 0.98"
    else:
        raise SystemExit(f"unknown workload {name}")
    return ns, bonds, cfg, desc


# ---------------------------------------------------------------------------
# clocks sampling during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference, one state/process
# ---------------------------------------------------------------------------
def _cpu_one(args):
    n, bond, seed, cfg = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from oracle import mpsops as M
    from oracle import states as S
    sv = S.random_mps(n, bond, seed)
    t0 = time.perf_counter()
    M.prepare_state(sv, cfg["bond_dimension"], cfg["num_layers"], cfg["num_sweeps"], conv="literal")
    return n, time.perf_counter() - t0


def cpu_baseline(ns_mix, cfg, workers: int, sample_ns=(12, 12, 13, 13, 14), seed=7):
    """Time the oracle path on a stratified sample; extrapolate to the mix.

    Returns (states/s on `workers` cores, details)."""
    import multiprocessing as mp
    rng = np.random.default_rng(seed)
    jobs = [(int(n), int(rng.choice([4, 8, 16, 32])), 1000 + i, cfg) for i, n in enumerate(sample_ns)]
    env_before = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(min(workers, len(jobs))) as pool:
        res = pool.map(_cpu_one, jobs)
    wall = time.perf_counter() - t0
    if env_before is None:
        os.environ.pop("OPENBLAS_NUM_THREADS", None)
    else:
        os.environ["OPENBLAS_NUM_THREADS"] = env_before
    # cost model t(n) = a * 2^n fitted on the sample
    a = float(np.mean([t / 2.0 ** n for n, t in res]))
    mean_t = float(np.mean([a * 2.0 ** n for n in ns_mix]))
    sps = workers / mean_t
    detail = {"per_state_s": {str(n): round(t, 3) for n, t in res}, "fit_s_per_amplitude": a,
              "mean_state_s_on_mix": mean_t, "sample_wall_s": wall}
    return sps, detail


# ---------------------------------------------------------------------------
def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_reference(args, rank, world):
    if rank != 0:
        return
    ns, bonds, cfg, desc = workload_spec(args.workload, args.states, args.seed)
    cores = len(os.sched_getaffinity(0))
    vals = []
    detail = None
    for it in range(args.warmup + args.steps):
        sps, detail = cpu_baseline(ns, cfg, cores, sample_ns=tuple([12] * cores))
        if it >= args.warmup:
            vals.append(sps)
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": desc, **cfg, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} 12-qubit states of the workload per step, one per core, "
                                   "oracle restatement (quimb/quick absent); per-state time extrapolated "
                                   "to the qubit mix with t(n) ~ 2^n",
                         "detail": detail},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def replica_spec(workload: str, states: int, seed: int, rank: int):
    """The batch of one replica: every rank encodes its own seeded batch of
    the same configuration (the path does not shard within a state)."""
    return workload_spec(workload, states, seed + rank)


def max_over_ranks(vals, world: int, device: str):
    """Element-wise maximum over the ranks (a no-op for one rank)."""
    import torch
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist
    from qmprs_gb300 import engine as E
    from qmprs_gb300.synthesis.mps_encoding import Sequential
    from qmprs_gb300.circuit import Circuit

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    ns, bonds, cfg, desc = replica_spec(args.workload, args.states, args.seed, rank)
    eng = E.engine()
    sv_dev = eng.random_mps_states(ns, bonds, seed=args.seed + 17 * rank)
    host = torch.empty(sv_dev.numel(), dtype=torch.float32, pin_memory=True)
    host.copy_(sv_dev)
    torch.cuda.synchronize()
    B = len(ns)
    in_bytes = int(sv_dev.numel() * 4)

    def barrier():
        if world > 1:
            dist.barrier()

    def step_device():
        return eng.encode(sv_dev, nqubits=ns, download=False, **cfg)

    def step_e2e():
        seq = Sequential(Circuit)
        _, res = seq.prepare_states(host, nqubits=ns, emit=False, **cfg)
        return res

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    # ---- value: device-resident inputs
    launches0 = eng.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    last = None
    for _ in range(args.steps):
        last = step_device()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    launches = (eng.launch_count() - launches0) // args.steps
    ov, nn = last.fidelity[0].cpu().numpy().view(np.complex128), last.fidelity[1].cpu().numpy().view(np.complex128)
    fid = np.abs(ov) / np.sqrt(nn.real)
    sd = last.sweeps_done.cpu().numpy()
    reached = int(np.sum(fid >= 0.98))
    # ---- e2e: public API from host buffers
    step_e2e()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    res = None
    for _ in range(args.steps):
        res = step_e2e()
    torch.cuda.synchronize()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    out_bytes = int(res.gates.nbytes + res.arity.nbytes + res.num_layers.nbytes + res.layer_fidelities.nbytes
                    + res.sweep_fidelities.nbytes + res.sweeps_done.nbytes + res.fidelity.nbytes)
    # ---- roofline: profiled pass of the same batch (per-stage events, then
    # per-kernel events of the sweep stage)
    p = eng.plan(ns, cfg["num_layers"], cfg["bond_dimension"])
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    ev[0].record(stream)
    tensors, bondsd, target = eng.stage_mps(p, sv_dev, cfg["bond_dimension"])
    ev[1].record(stream)
    gates, arity, nl, lf = eng.stage_layers(p, target, cfg["num_layers"], 1 - 1e-6)
    ev[2].record(stream)
    eng.set_profiling(p, True)
    eng.stage_sweeps(p, target, gates, arity, nl, cfg["num_sweeps"], cfg["stop_fidelity"])
    ev[3].record(stream)
    circ = eng.stage_circuit(p, gates, arity, nl)
    eng.overlap(p, circ, sv_dev)
    ev[4].record(stream)
    torch.cuda.synchronize()
    stage_ms = {"mps_from_statevector": ev[0].elapsed_time(ev[1]), "unitary_layers": ev[1].elapsed_time(ev[2]),
                "sweeps_profiled": ev[2].elapsed_time(ev[3]), "circuit_and_fidelity": ev[3].elapsed_time(ev[4])}
    prof = {k: eng.profile(p, k) for k in (0, 1, 2, 3)}
    eng.set_profiling(p, False)
    peak, peak_kind = peaks()
    n_env, ms_env, by_env = prof[0]
    achieved = (by_env / n_env) / (ms_env / n_env * 1e-3) / 1e9 if n_env and ms_env > 0 else 0.0

    # ---- max over ranks
    ms, e2e_ms = max_over_ranks([ms, e2e_ms], world, "cuda")
    if rank != 0:
        return
    cores = len(os.sched_getaffinity(0))
    cpu_v, cpu_detail = cpu_baseline(ns, cfg, cores)
    vec_gb = sum(2 ** n for n in ns) * 8 / 1e9
    line = {
        "metric": METRIC,
        "value": B * world / (ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64 (fp32 state, fp64 reductions/polar/eig)",
        "data": "synthetic",
        "config": {"workload": desc, "states_per_gpu": B, **cfg,
                   "l2": f"inputs larger than L2 ({vec_gb:.1f} GB of statevectors per copy)",
                   "reached_0.98": reached, "mean_fidelity": float(np.mean(fid)),
                   "mean_sweeps_run": float(np.mean(sd))},
        "roofline": {"bound": "hbm", "kernel": "k_group_pass", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": PASS_DRAM_PER_ALG_BYTE * (by_env / max(n_env, 1)),
                     "traffic_note": "DRAM bytes per launch, scaled by algorithmic bytes from a 32-state ncu capture",
                     "launches": n_env, "avg_launch_us": ms_env / max(n_env, 1) * 1e3,
                     "bytes_per_launch": by_env / max(n_env, 1),
                     "sweep_kernel_ms": {"group_pass": prof[0][1], "group_polar": prof[3][1],
                                         "rebuild": prof[2][1]}},
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "5 states of the workload family with 12-14 qubits, one per core, "
                                   "oracle restatement of the reference (literal conventions); per-state "
                                   "time extrapolated to the qubit mix with t(n) ~ 2^n",
                         "detail": cpu_detail},
        "e2e": {"value": B * world / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": in_bytes,
                "d2h_bytes_per_step": out_bytes, "ms_per_step": e2e_ms},
        "stage_ms": stage_ms,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched")
    ap.add_argument("--states", type=int, default=512)
    ap.add_argument("--seed", type=int, default=2024)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
