"""Launch shapes and their autotuners (wedg_set_launch_shape, wedg_autotune, wedg_batch_autotune;
no counterpart in the reference): the threads per block of k_prep and of the mass solves (and,
in a batch, persistent grids) change only how elements are spread over blocks, never an
element's arithmetic, so every shape must give the same states bit for bit; the tuners leave the
states they are given unchanged and keep a valid shape."""
import numpy as np
import pytest

import edg_westervelt_gb300 as W
from test_gpu_batch import INSTANCES

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128), (32, 32), (64, 96), (96, 64)]


def _state(q, N, kw, dev, steps=40):
    """The instance after `steps` RK4 steps from the zero state (so that v, and with it the
    Chebyshev step counts, vary over the elements)."""
    import torch
    pre, _ = W.precompute(q, N, **kw)
    nu, nv = pre["qu1"], pre["qv1"]
    u = torch.zeros(N * N * nu * nu, dtype=torch.float64, device=dev)
    v = torch.zeros(N * N * nv * nv, dtype=torch.float64, device=dev)
    dt = (1.0 / N) / (10 * q * q)
    t0 = 0.0 if kw.get("mode", "mms") == "mms" else 0.013
    ws = W.Workspace(pre, N)
    ws.rk4_steps(u, v, t0, dt, steps)
    return pre, N, u, v, t0 + steps * dt, dt


@pytest.mark.parametrize("index", range(len(INSTANCES)))
def test_launch_shapes_give_identical_states(index):
    import torch
    dev = torch.device("cuda:0")
    q, N, kw = INSTANCES[index]
    pre, N, u0, v0, t0, dt = _state(q, N, kw, dev)
    assert float(v0.abs().max()) > 0
    out = []
    for p, m in SHAPES:
        ws = W.Workspace(pre, N)
        ws.set_launch_shape(p, m)
        assert ws.launch_shape == (p, m)
        u, v = u0.clone(), v0.clone()
        ws.rk4_steps(u, v, t0, dt, 25)
        out.append((u.cpu().numpy(), v.cpu().numpy()))
    for u, v in out[1:]:
        assert np.array_equal(u, out[0][0]) and np.array_equal(v, out[0][1])


def test_launch_shape_refuses_other_sizes():
    pre, _ = W.precompute(2, 4)
    ws = W.Workspace(pre, 4)
    for p, m in ((16, 128), (128, 256), (100, 64), (0, 32)):
        with pytest.raises(Exception):
            ws.set_launch_shape(p, m)
    assert ws.launch_shape == (128, 128)


def test_autotune_keeps_a_valid_shape_and_the_state():
    import torch
    dev = torch.device("cuda:0")
    q, N, kw = INSTANCES[2]
    pre, N, u0, v0, t0, dt = _state(q, 24, kw, dev)
    ws = W.Workspace(pre, N)
    u, v = u0.clone(), v0.clone()
    ms = ws.autotune(u, v, t0, dt, steps=3)
    assert ms > 0
    p, m = ws.launch_shape
    assert p in (32, 64, 128) and m in (32, 64, 128)
    assert torch.equal(u, u0) and torch.equal(v, v0)
    # the tuned workspace gives the untuned one's states
    ref = W.Workspace(pre, N)
    ur, vr = u0.clone(), v0.clone()
    ref.rk4_steps(ur, vr, t0, dt, 10)
    ws.rk4_steps(u, v, t0, dt, 10)
    assert torch.equal(u, ur) and torch.equal(v, vr)


def test_batch_autotune_then_batch_matches_single_instances():
    import torch
    dev = torch.device("cuda:0")
    inst = [_state(q, N, kw, dev) for q, N, kw in INSTANCES]
    batch = W.Batch([W.Workspace(pre, N) for pre, N, *_ in inst])
    us = [x[2].clone() for x in inst]
    vs = [x[3].clone() for x in inst]
    t0s = [x[4] for x in inst]
    dts = [x[5] for x in inst]
    ms = batch.autotune(us, vs, t0s, dts, steps=2)
    assert ms > 0
    for s in batch.shapes():
        assert s["prep_threads"] in (32, 64, 128) and s["mass_threads"] in (32, 64, 128) and s["persist"] in (-1, 0, 1, 2)
    for x, u, v in zip(inst, us, vs):
        assert torch.equal(u, x[2]) and torch.equal(v, x[3])
    batch.rk4_steps(us, vs, t0s, dts, 30)
    for (pre, N, u0, v0, t0, dt), u, v in zip(inst, us, vs):
        ws = W.Workspace(pre, N)
        ur, vr = u0.clone(), v0.clone()
        ws.rk4_steps(ur, vr, t0, dt, 30)
        assert torch.equal(u, ur) and torch.equal(v, vr)
