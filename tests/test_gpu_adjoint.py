"""The discrete adjoint (no counterpart in the reference): wedg_rhs_adjoint against central
finite differences of the forward right-hand side (wedg_rhs) -- the dot-product test
⟨λ, (F(x + εw) - F(x - εw)) / 2ε⟩ = ⟨Jᵀλ, w⟩ on seeded x, w, λ -- over both pairings, every
boundary kind (the absorbing families are nonlinear through √(1 - kβv)), the three fluxes,
one-sided faces with jumping coefficients, both mass solvers and the constant-coefficient and
general kernels."""
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from oracle import coefficients as oc
from test_oracle import quadrant_coefficients

pytestmark = pytest.mark.gpu


def _dot(a, b):
    return float(np.sum(a[0] * b[0]) + np.sum(a[1] * b[1]))


def _check(pre, N, t, rng, amp_v=0.004, eps=1e-6, fast_path=True):
    nu, nv = pre["qu1"], pre["qv1"]
    ws = W.Workspace(pre, N, fast_path=fast_path)
    x = (np.asfortranarray(0.3 * rng.standard_normal((N, N, nu, nu))),
         np.asfortranarray(amp_v * rng.standard_normal((N, N, nv, nv))))
    w = (np.asfortranarray(rng.standard_normal((N, N, nu, nu))),
         np.asfortranarray(amp_v * rng.standard_normal((N, N, nv, nv))))
    lam = (np.asfortranarray(rng.standard_normal((N, N, nu, nu))),
           np.asfortranarray(rng.standard_normal((N, N, nv, nv))))
    fp = [y.copy() for y in ws.rhs(x[0] + eps * w[0], x[1] + eps * w[1], t)]
    fm = [y.copy() for y in ws.rhs(x[0] - eps * w[0], x[1] - eps * w[1], t)]
    jvp = ((fp[0] - fm[0]) / (2 * eps), (fp[1] - fm[1]) / (2 * eps))
    g = ws.rhs_adjoint(x[0], x[1], t, lam[0], lam[1])
    a, b = _dot(lam, jvp), _dot(g, w)
    scale = abs(_dot(lam, (np.abs(jvp[0]), np.abs(jvp[1])))) + 1e-300
    return abs(a - b) / max(abs(a), 1e-12 * scale)


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_rhs_adjoint_dot_product(gpu, solver):
    rng = np.random.default_rng(41)
    worst = 0.0
    for q, N, mixed, flux, boundary, mode in (
            (1, 3, True, "upwind", "absorbing_2beta", "mms"),
            (2, 4, False, "central", "absorbing", "source"),
            (3, 4, True, "alternating", "dirichlet", "initial_value"),
            (4, 3, False, "upwind", "wall", "source"),
            (3, 5, True, "upwind", dict(bot="absorbing_2beta", top="wall", lft="dirichlet", rgt="absorbing"), "mms")):
        co = oc.constant_coefficients(c=1.2, alpha=1e-3, beta=4.0) if mode != "mms" else None
        kw = dict(mixed=mixed, flux=flux, boundary=boundary, mode=mode, mass_solver=solver, kappa=0.6, sigma=0.3,
                  sigma_dirichlet=0.5, phase=(0.4, 0.3))
        if co is not None:
            kw["coefficients"] = W.constant_coefficients(c=1.2, alpha=1e-3, beta=4.0)
        pre, _ = W.precompute(q, N, **kw)
        for fast in (True, False):
            worst = max(worst, _check(pre, N, 0.037, rng, fast_path=fast))
    assert worst < 1e-6, worst


def test_rhs_adjoint_one_sided_faces(gpu):
    """Jumping coefficients: the one-sided face kernel (src/rhs.jl:660-700) and its jump terms."""
    rng = np.random.default_rng(42)
    co = quadrant_coefficients(0.5, 0.5, smooth=False)
    worst = 0.0
    for q, N in ((2, 4), (4, 4)):
        pre, _ = W.precompute(q, N, mode="source", coefficients=co, flux_params=dict(theta=0.3, tau=0.7, lambda_u=0.4,
                                                                                        lambda_v=0.9),
                              boundary="absorbing_2beta")
        assert pre["one_sided"]
        worst = max(worst, _check(pre, N, 0.2, rng))
    assert worst < 1e-6, worst


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_rk4_adjoint_against_finite_differences(gpu, solver):
    """The reverse RK4 with checkpoints: the gradient of J = λ·y(T) with respect to the initial
    state against central differences of forward runs (wedg_rk4_steps) along seeded directions;
    37 steps with a checkpoint every 8, so the last segment is partial."""
    rng = np.random.default_rng(43)
    for q, N, kw in ((3, 4, dict(mode="source", flux="upwind", boundary="absorbing_2beta",
                                 coefficients=W.constant_coefficients(c=1.1, alpha=1e-3, beta=3.0))),
                     (2, 5, dict(mode="mms", flux="alternating", mixed=False,
                                 boundary=dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"),
                                 kappa=0.5))):
        pre, _ = W.precompute(q, N, mass_solver=solver, **kw)
        nu, nv = pre["qu1"], pre["qv1"]
        ws = W.Workspace(pre, N)
        dt = (1.0 / N) / (10 * q * q)
        nsteps, t0 = 37, 0.02
        def smooth(n, amp):                      # modal coefficients decaying with the degree
            d = 1.0 / (1.0 + np.add.outer(np.arange(n), np.arange(n))) ** 2
            return np.asfortranarray(amp * rng.standard_normal((N, N, n, n)) * d)
        y0 = (smooth(nu, 0.01), smooth(nv, 0.001))
        lam = (np.asfortranarray(rng.standard_normal((N, N, nu, nu))),
               np.asfortranarray(rng.standard_normal((N, N, nv, nv))))

        def J(u, v):
            u, v = u.copy(order="F"), v.copy(order="F")
            assert ws.rk4_steps(u, v, t0, dt, nsteps) == nsteps
            return float(np.sum(lam[0] * u) + np.sum(lam[1] * v))
        gu, gv = ws.rk4_adjoint(y0[0], y0[1], t0, dt, nsteps, lam[0], lam[1], every=8)
        for _ in range(3):
            w = (smooth(nu, 1.0), smooth(nv, 0.1))
            eps = 1e-5
            fd = (J(y0[0] + eps * w[0], y0[1] + eps * w[1]) - J(y0[0] - eps * w[0], y0[1] - eps * w[1])) / (2 * eps)
            ad = float(np.sum(gu * w[0]) + np.sum(gv * w[1]))
            assert abs(fd - ad) <= 1e-6 * abs(fd), (q, N, fd, ad)


MISFIT_CASES = {
    # jumping cells: one-sided faces; every physical side absorbing_2beta
    "one_sided": (2, dict(flux="upwind", mixed=False, boundary="absorbing_2beta")),
    # every boundary kind, the alternating flux with its penalties, one-sided faces
    "kinds": (2, dict(flux="alternating", mixed=False, kappa=0.6, sigma=0.3,
                      boundary=dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"))),
    # one cell: constant coefficients, continuous faces; central flux
    "continuous": (1, dict(flux="central", mixed=False, boundary=dict(bot="absorbing_2beta", top="wall",
                                                                        lft="absorbing", rgt="absorbing_2beta"))),
}


@pytest.mark.parametrize("case", sorted(MISFIT_CASES))
def test_misfit_gradient_against_finite_differences(gpu, case):
    """The gradient of a receiver misfit with respect to c², α, β constant on m × m cells (the
    parameter fields of the adjoint form) against central differences of the misfit along seeded
    directions, one parameter field at a time: forward runs with perturbed cell values."""
    m, kw = MISFIT_CASES[case]
    rng = np.random.default_rng(44)
    q, N, T = 2, 8, 0.06
    c2 = rng.uniform(0.8, 1.5, (m, m))
    al = 10 ** rng.uniform(-4, -3, (m, m))
    be = rng.uniform(0.5, 3.0, (m, m))
    g = (np.arange(4) + 0.5) / 4
    receivers = [(x, y) for y in g for x in g]
    u_obs = 1e-4 * rng.standard_normal(len(receivers))
    src = W.GaussianSource(x0=(0.4, 0.55), r0=0.15, omega=12 * math.pi, Ts=0.5)
    kw = dict(kw, source=src)
    if m == 1:
        pre, _ = W.precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(c2, al, be), **kw)
        assert not pre["one_sided"]
    J0, grad = W.misfit_gradient(q, N, T, c2, al, be, receivers, u_obs, every=7, **kw)
    assert J0 > 0
    base = {"c2": c2, "alpha": al, "beta": be}
    for name in ("c2", "alpha", "beta"):
        d = {k: (rng.standard_normal((m, m)) * base[k] if k == name else np.zeros((m, m))) for k in base}
        # α enters the misfit weakly (α ~ 1e-4): a larger relative step keeps the difference of the
        # misfits well above their rounding
        eps = 1e-4 if name == "alpha" else 1e-6
        Jp = W.misfit_gradient(q, N, T, c2 + eps * d["c2"], al + eps * d["alpha"], be + eps * d["beta"],
                               receivers, u_obs, every=7, **kw)[0]
        Jm = W.misfit_gradient(q, N, T, c2 - eps * d["c2"], al - eps * d["alpha"], be - eps * d["beta"],
                               receivers, u_obs, every=7, **kw)[0]
        fd = (Jp - Jm) / (2 * eps)
        ad = float(np.sum(grad[name] * d[name]))
        assert abs(fd - ad) <= 1e-5 * abs(fd), (case, name, fd, ad)


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_reverse_sweep_kept_stage_data(gpu, solver):
    """The reverse sweep that keeps each segment stage's forward data (wedg_set_adjoint_memory
    large enough) against the one that evaluates every stage's forward RHS again (memory 0):
    the same gradients up to rounding, with fewer kernel launches; a ragged last segment."""
    rng = np.random.default_rng(45)
    q, N, nsteps, every = 3, 6, 11, 4
    c2 = rng.uniform(0.8, 1.5, (2, 2))
    al = 10 ** rng.uniform(-4, -3, (2, 2))
    be = rng.uniform(0.5, 3.0, (2, 2))
    src = W.GaussianSource(x0=(0.4, 0.55), r0=0.15, omega=12 * math.pi, Ts=0.5)
    pre, _ = W.precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(c2, al, be), flux="central",
                          mixed=True, source=src, mass_solver=solver, kappa=0.5,
                          boundary=dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"))
    ws = W.Workspace(pre, N)
    nu, nv = pre["qu1"], pre["qv1"]
    u0 = np.zeros((N, N, nu, nu), order="F")
    v0 = np.zeros((N, N, nv, nv), order="F")
    dt = (1.0 / N) / (10 * q * q)
    ws.rk4_adjoint_forward(u0, v0, 0.0, dt, nsteps, every=every)
    lam_u = np.asfortranarray(rng.standard_normal((N, N, nu, nu)))
    lam_v = np.asfortranarray(rng.standard_normal((N, N, nv, nv)))
    out, launches = {}, {}
    for mem in (0, 1 << 40):
        ws.set_adjoint_memory(mem)
        out[mem] = ws.rk4_adjoint_reverse(lam_u, lam_v, params=True)
        launches[mem] = ws.stats()["kernel_launches"]
    ws.set_adjoint_memory(-1)
    auto = ws.rk4_adjoint_reverse(lam_u, lam_v, params=True)
    for a, b, c in zip(out[0], out[1 << 40], auto):
        scale = np.abs(a).max()
        assert scale > 0
        assert np.abs(a - b).max() <= 1e-10 * scale
        assert np.array_equal(b, c)
    assert launches[1 << 40] < launches[0]


def test_misfit_gradient_against_oracle_differences(gpu):
    """The GPU adjoint's misfit gradient against central differences of the misfit computed
    by the oracle (the C restatement of the reference's RHS and RK4, run on the CPU): the
    gradient is anchored on the reference's algorithm, not only on the GPU forward."""
    from oracle.precompute import precompute as oracle_precompute
    from oracle.rhs import OracleWorkspace
    from edg_westervelt_gb300.solver import _locate, _vrow
    rng = np.random.default_rng(46)
    q, N, T = 2, 8, 0.06
    c2 = rng.uniform(0.8, 1.5, (2, 2))
    al = 10 ** rng.uniform(-4, -3, (2, 2))
    be = rng.uniform(0.5, 3.0, (2, 2))
    g = (np.arange(4) + 0.5) / 4
    receivers = [(x, y) for y in g for x in g]
    u_obs = 1e-4 * rng.standard_normal(len(receivers))
    src = dict(x0=(0.4, 0.55), r0=0.15, omega=12 * math.pi, Ts=0.5)
    kw = dict(flux="upwind", mixed=False, boundary="absorbing_2beta")
    J0, grad = W.misfit_gradient(q, N, T, c2, al, be, receivers, u_obs, every=7, source=W.GaussianSource(**src),
                                 **kw)

    def J_oracle(c2_, al_, be_):
        pre, _ = oracle_precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(c2_, al_, be_),
                                   source=oc.GaussianSource(**src), **kw)
        nu, nv = pre["qu1"], pre["qv1"]
        dt = (1.0 / N) / (10 * q * q)
        nsteps = int(round(T / dt))
        dt = T / nsteps
        u = np.zeros((N, N, nu, nu), order="F")
        v = np.zeros((N, N, nv, nv), order="F")
        OracleWorkspace(pre).rk4_steps(u, v, 0.0, dt, nsteps)
        J = 0.0
        for (xr, yr), obs in zip(receivers, u_obs):
            kr, xi = _locate(xr, N)
            jr, eta = _locate(yr, N)
            J += 0.5 * (float(_vrow(eta, nu) @ u[jr - 1, kr - 1] @ _vrow(xi, nu)) - obs) ** 2
        return J

    assert abs(J_oracle(c2, al, be) - J0) <= 1e-10 * J0
    base = {"c2": c2, "alpha": al, "beta": be}
    for name in ("c2", "alpha", "beta"):
        d = {k: (rng.standard_normal((2, 2)) * base[k] if k == name else np.zeros((2, 2))) for k in base}
        eps = 1e-4 if name == "alpha" else 1e-6
        fd = (J_oracle(c2 + eps * d["c2"], al + eps * d["alpha"], be + eps * d["beta"]) -
              J_oracle(c2 - eps * d["c2"], al - eps * d["alpha"], be - eps * d["beta"])) / (2 * eps)
        ad = float(np.sum(grad[name] * d[name]))
        assert abs(fd - ad) <= 1e-5 * abs(fd), (name, fd, ad)


def test_misfit_gradient_n128_q4_twenty_directions(gpu):
    """The adjoint form at the shape of its workload: N = 128, q_u = q_v = 4, c², α, β constant on
    16 × 16 cells (c ~ U[0.8, 1.25], α log-uniform on [1e-6, 1e-5], β ~ U[0, 4]), a 32 × 32 receiver
    grid whose observations come from the forward solver on the fields perturbed by ±10 %,
    absorbing_2beta sides, upwind flux, a Gaussian source strong and fast enough that 1 - 2βv_h
    comes down to about 0.7 within T = 0.02 (410 RK4 steps, checkpoints every 32). The gradient with
    respect to all 768 cell values at once is checked against central differences of the misfit
    (step 1e-6 relative to each cell value) along 20 seeded random directions, to 1e-6 relative."""
    from edg_westervelt_gb300.solver import _locate, _vrow
    rng = np.random.default_rng(51)
    q, N, m, T = 4, 128, 16, 0.02
    c2 = rng.uniform(0.8, 1.25, (m, m)) ** 2
    al = 10.0 ** rng.uniform(-6, -5, (m, m))
    be = rng.uniform(0.0, 4.0, (m, m))
    g = (np.arange(32) + 0.5) / 32
    receivers = [(x, y) for y in g for x in g]
    src = W.GaussianSource(x0=(0.45, 0.5), r0=0.08, omega=16 * math.pi, Ts=0.04, amplitude=6.0)
    kw = dict(flux="upwind", mixed=False, boundary="absorbing_2beta", source=src)
    pert = lambda a: a * (1.0 + 0.1 * rng.uniform(-1, 1, a.shape))   # noqa: E731
    pre, _ = W.precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(pert(c2), pert(al), pert(be)),
                          **kw)
    dt = (1.0 / N) / (10 * q * q)
    nsteps = int(round(T / dt))
    ws = W.Workspace(pre, N)
    u = np.zeros((N, N, 5, 5), order="F")
    v = np.zeros((N, N, 5, 5), order="F")
    assert ws.rk4_steps(u, v, 0.0, T / nsteps, nsteps) == nsteps
    u_obs = []
    for xr, yr in receivers:
        kr, xi = _locate(xr, N)
        jr, eta = _locate(yr, N)
        u_obs.append(float(_vrow(eta, 5) @ u[jr - 1, kr - 1] @ _vrow(xi, 5)))
    del ws
    J0, grad = W.misfit_gradient(q, N, T, c2, al, be, receivers, u_obs, every=32, **kw)
    assert J0 > 0
    eps = 1e-6
    worst = 0.0
    for _ in range(20):
        d = {k: rng.standard_normal((m, m)) * x for k, x in (("c2", c2), ("alpha", al), ("beta", be))}
        Jp = W.misfit(q, N, T, c2 + eps * d["c2"], al + eps * d["alpha"], be + eps * d["beta"], receivers, u_obs, **kw)
        Jm = W.misfit(q, N, T, c2 - eps * d["c2"], al - eps * d["alpha"], be - eps * d["beta"], receivers, u_obs, **kw)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float(np.sum(grad[k] * d[k])) for k in d)
        worst = max(worst, abs(fd - ad) / abs(fd))
    assert worst <= 1e-6, worst


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_group_gradients_match_single_calls(gpu, solver):
    """misfit_gradients for four seeded parameter fields at once (the forward runs and reverse
    sweeps of the four workspaces as multi-instance launches) against misfit_gradient for each
    field alone: the same misfits and gradients. Also with an allowance too small to keep the
    stage data, where the reverse sweeps run one after the other."""
    rng = np.random.default_rng(47)
    q, N, T, m = 3, 8, 0.05, 2
    g = (np.arange(4) + 0.5) / 4
    receivers = [(x, y) for y in g for x in g]
    src = W.GaussianSource(x0=(0.4, 0.55), r0=0.15, omega=12 * math.pi, Ts=0.5)
    kw = dict(flux="alternating", mixed=True, kappa=0.5, source=src, mass_solver=solver,
              boundary=dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"))
    fields = [(rng.uniform(0.8, 1.5, (m, m)), 10 ** rng.uniform(-4, -3, (m, m)), rng.uniform(0.5, 3.0, (m, m)))
              for _ in range(4)]
    u_obs = [1e-4 * rng.standard_normal(len(receivers)) for _ in fields]
    single = [W.misfit_gradient(q, N, T, *f, receivers, o, every=5, **kw) for f, o in zip(fields, u_obs)]
    group = W.misfit_gradients(q, N, T, fields, receivers, u_obs, every=5, **kw)
    for (J1, g1), (J2, g2) in zip(single, group):
        assert J1 == J2
        for k in g1:
            assert np.max(np.abs(g1[k] - g2[k])) <= 1e-13 * np.max(np.abs(g1[k])), k
    # the reverse sweeps one after the other: every workspace's allowance below one segment's data
    from edg_westervelt_gb300.solver import _misfit_problem, _misfit_value
    probs = [_misfit_problem(q, N, T, *f, 10, kw) for f in fields]
    wss = [p[1] for p in probs]
    for w in wss:
        w.set_adjoint_memory(1)
    nu, nv = probs[0][0]["qu1"], probs[0][0]["qv1"]
    z = [np.zeros((N, N, nu, nu), order="F") for _ in wss]
    zv = [np.zeros((N, N, nv, nv), order="F") for _ in wss]
    uT, vT = W.rk4_adjoint_forward_many(wss, z, zv, 0.0, probs[0][2], probs[0][3], every=5)
    lams = [_misfit_value(uT[i], N, receivers, u_obs[i])[1] for i in range(len(wss))]
    out = W.rk4_adjoint_reverse_many(wss, lams, [np.zeros_like(x) for x in vT], params=True)
    for (J1, g1), o in zip(single, out):
        gc2 = o[2].reshape(m, N // m, m, N // m).sum(axis=(1, 3))
        assert np.max(np.abs(gc2 - g1["c2"])) <= 1e-10 * np.max(np.abs(g1["c2"]))
