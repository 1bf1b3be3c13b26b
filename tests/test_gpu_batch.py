"""The batched form (wedg_batch_*): instances of different N, degrees, fluxes, boundary kinds,
coefficients and mass solvers advanced together by one replayed CUDA graph per step. The
kernels and time factors are those of the single-instance calls, so every instance must
match its own Workspace.rk4_steps run bit for bit; the factor tables are refilled every
WEDG_BATCH_CHUNK = 256 steps, so a run of 600 steps crosses two refills. Errors stay with
their instance."""
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
    import torch
    dev = torch.device("cuda:0")
    inst = _setup()
    nsteps = 600
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
