"""CUDA-graph replay of the layer and sweep stages (qmprs_plan_set_graphs)
against the launch-by-launch path: bit-identical gates and fidelities.

The batch mixes states that leave the layer stage early (a two-block
product state disentangles in one layer) or stop sweeping at the stop
fidelity with states that run every layer and sweep, so the replayed graph,
which enqueues every layer and sweep and leaves finished states to the
kernels' active flags, is compared with the path that stops at the first
layer or sweep after which no state is left."""

import numpy as np
import pytest

from oracle import states as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(cuda_lib):
    from qmprs_gb300 import engine
    return engine.engine()


def _batch():
    from tests.test_oracle import _ghz_like
    return [S.random_mps(9, 2, 3), S.uniform_complex(11, 4), _ghz_like(8, [(0, 2), (5, 7)], [0, 5]),
            S.random_mps(12, 4, 5)]


def _fields(r):
    return [r.gates, r.arity, r.num_layers, r.layer_fidelities, r.sweep_fidelities, r.sweeps_done, r.fidelity]


@pytest.mark.parametrize("precision", ["fast", "exact"])
@pytest.mark.parametrize("stop", [0.0, 0.9])
def test_graph_replay_is_bit_identical(eng, precision, stop):
    svs = _batch()
    kw = dict(num_layers=5, num_sweeps=6, stop_fidelity=stop, precision=precision)
    ns = [int(np.log2(len(v))) for v in svs]
    p = eng.plan(ns, 5, 16, precision)
    eng.set_graphs(p, False)
    ref = eng.encode(svs, 16, **kw)
    eng.set_graphs(p, True)
    _, before = eng.graph_stats(p)
    runs = [eng.encode(svs, 16, **kw) for _ in range(4)]      # direct, capture, replay, replay
    cached, after = eng.graph_stats(p)
    # the layer stage replays a graph from the third call on; the sweep
    # stage of states this small is one launch (every sweep in one kernel)
    assert cached >= 1 and after - before >= 3, (cached, before, after)
    for r in runs:
        for a, b in zip(_fields(r), _fields(ref)):
            assert np.array_equal(a, b)
    assert int(ref.num_layers[2]) < 5                         # the product state left the layer stage early


def test_autotuned_grid_changes_no_result(eng):
    """The sweep's autotuner (qmprs_plan_set_autotune) times candidate grids
    of the tile passes on the first sweeps (here 384 chunks: 384, 384 and
    304 blocks); its choice changes no bit of the result, and it is cached
    on the handle for later plans of the same batch signature."""
    import torch
    from qmprs_gb300 import engine as E
    ns = [21] * 12
    svs = [S.random_mps(21, 4, 40 + i) for i in range(12)]
    kw = dict(num_layers=2, num_sweeps=4)
    p = eng.plan(ns, 2, 16)
    eng.set_autotune(p, False)
    eng.set_graphs(p, False)
    ref = eng.encode(svs, 16, **kw)
    assert eng.tuning(p) == (384, False)
    eng.set_autotune(p, True)
    runs = [eng.encode(svs, 16, **kw) for _ in range(2)]
    grid, tuned = eng.tuning(p)
    assert tuned and grid in (384, 304)
    for r in runs:
        for a, b in zip(_fields(r), _fields(ref)):
            assert np.array_equal(a, b)
    q = E.Plan(eng.hd, ns, 2, 16)                  # a second plan of the same signature
    assert eng.tuning(q) == (384, False)
    packed = np.concatenate([v.astype(np.complex64) for v in svs])
    sv = torch.from_numpy(packed.view(np.float32).copy()).cuda()
    _, _, target = eng.stage_mps(q, sv, 16)
    gates, arity, nl, _ = eng.stage_layers(q, target, 2, 1 - 1e-6)
    eng.stage_sweeps(q, target, gates, arity, nl, 1, 0.0)
    assert eng.tuning(q) == (grid, True)
