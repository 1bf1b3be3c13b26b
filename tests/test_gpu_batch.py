"""The batched form (wedg_batch_*): instances of different N, degrees, fluxes, boundary kinds,
coefficients and mass solvers advanced together by one replayed CUDA graph per step, every stage
kernel launched once per bucket of instances with the same kernels. An element's arithmetic is
the one of a single-instance launch and the time factors are those of the single-instance
calls, so every instance must match its own Workspace.rk4_steps run bit for bit; the factor
tables are refilled every WEDG_BATCH_CHUNK = 256 steps, so a run of 600 steps crosses two
refills. Buckets of many instances of different N (more than the 32 one launch takes) and every
launch shape give the same states. Errors stay with their instance."""
import numpy as np
import pytest

import edg_westervelt_gb300 as W

pytestmark = pytest.mark.gpu

INSTANCES = [
    (3, 6, dict(flux="upwind", mixed=True)),                                              # mms, paper coefficients
    (2, 9, dict(flux="central", mixed=False, mode="initial_value",
                boundary=dict(bot="dirichlet", top="absorbing", lft="absorbing_2beta", rgt="wall"))),
    (6, 5, dict(flux="alternating", mixed=False, mode="source", kappa=0.5,
                coefficients=W.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0),
                boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))),
    (4, 7, dict(flux="upwind", mixed=True, mode="source", mass_solver="cg",
                coefficients=W.constant_coefficients(c=1.3, alpha=1e-4, beta=2.0))),
    (5, 4, dict(flux="central", mixed=True, mode="mms", phase=(0.4, 0.3))),
]


def _setup():
    """The instances from the zero state, as the reference's solve starts every mode; t0 = 0 for
    the manufactured-solution instances, 0.013 for the others."""
    out = []
    for q, N, kw in INSTANCES:
        pre, _ = W.precompute(q, N, **kw)
        nu, nv = pre["qu1"], pre["qv1"]
        u = np.zeros(N * N * nu * nu)
        v = np.zeros(N * N * nv * nv)
        dt = (1.0 / N) / (10 * q * q)
        t0 = 0.0 if kw.get("mode", "mms") == "mms" else 0.013
        out.append((pre, N, u, v, dt, t0))
    return out


def test_batch_matches_single_instances():
    """602 steps: two table chunks of 256 and a third of 90, run as graphs of four steps and, for
    the last two, of one step; then 3 more steps (graphs of one step)."""
    import torch
    dev = torch.device("cuda:0")
    inst = _setup()
    nsteps = 602
    ref = []
    for pre, N, u, v, dt, t0 in inst:
        ws = W.Workspace(pre, N)
        du = torch.from_numpy(u.copy()).to(dev)
        dv = torch.from_numpy(v.copy()).to(dev)
        assert ws.rk4_steps(du, dv, t0, dt, nsteps) == nsteps
        ref.append((du.cpu().numpy(), dv.cpu().numpy()))
        assert np.max(np.abs(ref[-1][0])) > 0
    wss = [W.Workspace(pre, N) for pre, N, *_ in inst]
    batch = W.Batch(wss)
    us = [torch.from_numpy(x[2].copy()).to(dev) for x in inst]
    vs = [torch.from_numpy(x[3].copy()).to(dev) for x in inst]
    done, fin, st = batch.rk4_steps(us, vs, [x[5] for x in inst], [x[4] for x in inst], nsteps)
    assert done == [nsteps] * len(inst) and all(fin) and st == [0] * len(inst)
    for (ru, rv), u, v in zip(ref, us, vs):
        assert np.array_equal(ru, u.cpu().numpy()) and np.array_equal(rv, v.cpu().numpy())
    # a second call continues from the new states with the same (cached) graph
    done, _, _ = batch.rk4_steps(us, vs, [x[5] + nsteps * x[4] for x in inst], [x[4] for x in inst], 3)
    assert done == [3] * len(inst)


def test_batch_errors_stay_with_their_instance():
    """One instance violates 1 - 2βv > 0 at a boundary point: it reports the reference's error,
    the others complete."""
    import torch
    dev = torch.device("cuda:0")
    inst = _setup()
    wss = [W.Workspace(pre, N) for pre, N, *_ in inst]
    batch = W.Batch(wss)
    us = [torch.from_numpy(x[2].copy()).to(dev) for x in inst]
    vs = [torch.from_numpy(x[3].copy()).to(dev) for x in inst]
    vs[2][0] = 10.0                                  # the q = 6, β = 8 source instance: v far beyond 1/(2β)
    with pytest.raises(W.ErrorException):
        batch.rk4_steps(us, vs, [x[5] for x in inst], [x[4] for x in inst], 4)
    done = [w.stats()["steps_done"] for w in wss]
    assert done[2] == 0 and all(d == 4 for i, d in enumerate(done) if i != 2)


def _many(seed=12):
    """44 seeded instances, q_v = q_u - 1, N from 2 to 9, random fluxes and boundary kinds, in three
    buckets: 6 manufactured-solution instances of q_u = 3 (paper coefficients: the general
    kernels), 34 initial-value or source instances of q_u = 3 and 4 of q_u = 2 (constant
    coefficients)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(44):
        q = 2 if i >= 40 else 3
        N = int(rng.integers(2, 10))
        mode = "mms" if i < 6 else str(rng.choice(["initial_value", "source"]))
        kinds = [str(k) for k in rng.choice(["absorbing_2beta", "absorbing", "dirichlet", "wall"], 4)]
        kw = dict(flux=str(rng.choice(["upwind", "central", "alternating"])), mixed=True, mode=mode, kappa=0.5,
                  boundary=dict(bot=kinds[0], top=kinds[1], lft=kinds[2], rgt=kinds[3]))
        if mode != "mms":
            # β small enough that 1 - 2βv stays positive under the initial data Φ (|v| grows to ~15)
            kw["coefficients"] = W.constant_coefficients(c=float(rng.uniform(0.6, 1.5)),
                                                         alpha=float(10 ** rng.uniform(-5, -3)),
                                                         beta=0.3 * float(rng.uniform(0.0, 0.05)))
        pre, _ = W.precompute(q, N, **kw)
        out.append((pre, N, q, 0.0 if mode == "mms" else 0.013))
    return out


def test_buckets_of_many_instances_and_every_shape():
    """44 instances in three buckets (one of 34 instances, so its stages take two launches), each advanced 40 steps by the batch under several launch shapes (threads per block
    of k_prep and of the mass solve, persistent grids): the states equal each instance's own run
    bit for bit."""
    import torch
    dev = torch.device("cuda:0")
    inst = _many()
    nsteps = 40
    ref, us0, vs0, dts = [], [], [], []
    for pre, N, q, t0 in inst:
        nu, nv = pre["qu1"], pre["qv1"]
        dt = (1.0 / N) / (10 * q * q)
        u = torch.zeros(N * N * nu * nu, dtype=torch.float64, device=dev)
        v = torch.zeros(N * N * nv * nv, dtype=torch.float64, device=dev)
        us0.append(u.clone())
        vs0.append(v.clone())
        dts.append(dt)
        assert W.Workspace(pre, N).rk4_steps(u, v, t0, dt, nsteps) == nsteps
        ref.append((u.cpu().numpy(), v.cpu().numpy()))
    batch = W.Batch([W.Workspace(pre, N) for pre, N, *_ in inst])
    shapes = batch.shapes()
    assert sum(s["instances"] for s in shapes) == len(inst) and max(s["instances"] for s in shapes) > 32
    t0s = [x[3] for x in inst]
    for prep, mass, persist in ((128, 128, 0), (32, 64, 0), (64, 32, 1), (128, 96, 2), (64, 64, -1)):
        for k in range(len(shapes)):
            batch.set_shape(k, prep, mass, persist)
        us = [u.clone() for u in us0]
        vs = [v.clone() for v in vs0]
        done, fin, st = batch.rk4_steps(us, vs, t0s, dts, nsteps)
        assert done == [nsteps] * len(inst) and all(fin)
        for (ru, rv), u, v in zip(ref, us, vs):
            assert np.array_equal(ru, u.cpu().numpy()) and np.array_equal(rv, v.cpu().numpy()), (prep, mass, persist)
