"""Whole-run properties of the reference's own test suite, through ``solve`` on the GPU.

These need no second implementation: they are the reference's integration tests
(test/runtests.jl), run here through the product's ``solve`` (the time loop, the
source-mode diagnostics and the error norms on the GPU).
- boundary spellings give bit-identical runs (test/runtests.jl:243-264);
- after the source stops, the energy is conserved by walls with κ = 0 and Dirichlet sides
  with σ_D = 0 under the central flux, and dissipated otherwise (test/runtests.jl:386-406);
- every boundary kind converges at the reference's orders on meshes 6 → 12
  (test/runtests.jl:408-413), and so does a jump of β alone (:824-835);
- with c, α, β jumping on mesh lines and absorbing sides the energy decays after the source
  stops (test/runtests.jl:838-848);
- the interface terms of an initial profile u₀ (test/runtests.jl:760-784);
- the semi-discrete energy identity with jumping coefficients (test/runtests.jl:734-761);
- the convergence of a two-layer standing mode across a jump of c (test/runtests.jl:816-823).
"""
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W

pytestmark = pytest.mark.gpu

MIXED = dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing")


def test_boundary_spellings_bitwise(gpu):
    e = W.solve(2, 4, 0.05)
    assert e == W.solve(2, 4, 0.05, boundary="absorbing_2beta")
    assert e == W.solve(2, 4, 0.05, boundary=dict(rgt="absorbing_2beta", lft="absorbing_2beta",
                                                  top="absorbing_2beta", bot="absorbing_2beta"),
                        kappa=0.7, phase=(0.0, 0.0))
    assert W.solve(2, 4, 0.05, boundary="absorbing") == W.solve(
        2, 4, 0.05, boundary=dict(rgt="absorbing", lft="absorbing", top="absorbing", bot="absorbing"))
    d4 = dict(bot="dirichlet", top="dirichlet", lft="dirichlet", rgt="dirichlet")
    assert W.solve(2, 4, 0.05, boundary="dirichlet", sigma=0.3) == W.solve(2, 4, 0.05, boundary=d4,
                                                                           sigma_dirichlet=0.3)


def _energy_after(**kw):
    src = W.GaussianSource(x0=(0.3, 0.6), r0=0.1, omega=8 * math.pi, Ts=0.25)
    co = W.constant_coefficients(c=1.0, alpha=0.0, beta=0.0)
    H = W.solve(3, 8, 0.75, mode="source", coefficients=co, source=src, record_every=5, **kw)
    return H["energy"][H["t"] > 0.25]


@pytest.mark.parametrize("kw", [dict(boundary="wall", flux="central"), dict(boundary="dirichlet", flux="central"),
                                dict(boundary=dict(bot="dirichlet", top="wall", lft="wall", rgt="dirichlet"),
                                     flux="central")])
def test_energy_conserved_after_the_source(gpu, kw):
    E = _energy_after(**kw)
    assert len(E) > 10
    assert np.max(np.abs(E - E[0])) / E[0] < 1e-6


@pytest.mark.parametrize("kw", [dict(boundary="wall", kappa=0.5, flux="central"),
                                dict(boundary="dirichlet", sigma_dirichlet=1.0, flux="central"),
                                dict(boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))])
def test_energy_dissipated_after_the_source(gpu, kw):
    E = _energy_after(**kw)
    assert len(E) > 10
    assert np.max(np.diff(E)) <= 1e-10 * E[0]
    assert E[-1] / E[0] < 0.95


@pytest.mark.parametrize("boundary", ["absorbing_2beta", "dirichlet", "wall", "mixed"])
def test_convergence_per_boundary_kind(gpu, boundary):
    bd = MIXED if boundary == "mixed" else boundary
    kw = dict(boundary=bd, sigma_dirichlet=1.0, kappa=1.0, phase=(0.4, 0.3))
    e1 = W.solve(2, 6, 0.1, **kw)
    e2 = W.solve(2, 12, 0.1, **kw)
    assert math.log2(e1["erru"] / e2["erru"]) > 2.5
    assert math.log2(e1["errE"] / e2["errE"]) > 1.5


@pytest.mark.parametrize("flux", ["upwind", "central"])
def test_energy_decay_with_jumping_coefficients(gpu, flux):
    """test/runtests.jl:838-848: c, α, β jumping on x = ½ and y = ½ (one-sided faces), absorbing
    sides; after the source stops the energy does not increase and falls below 95 %."""
    from test_oracle import quadrant_coefficients
    co = quadrant_coefficients(0.5, 0.5, alpha=(1e-5, 4e-6, 2e-5, 1e-6), beta=(1e-4, 3e-4, 0.0, 2e-4))
    src = W.GaussianSource(x0=(0.45, 0.55), r0=0.08, amplitude=50.0, omega=8 * math.pi, Ts=0.25)
    H = W.solve(3, 8, 0.75, mode="source", coefficients=co, flux=flux, source=src, record_every=5)
    E = H["energy"][H["t"] > 0.25]
    assert len(E) > 10
    assert np.max(np.diff(E)) <= 1e-10 * E[0]
    assert E[-1] / E[0] < 0.95


def test_convergence_with_a_jump_of_beta_alone(gpu):
    """test/runtests.jl:824-835: a jump of β alone keeps the continuous face kernel and the
    manufactured solution; the orders on meshes 6 → 12 with mixed sides."""
    from test_oracle import quadrant_coefficients
    cb = quadrant_coefficients(0.5, 0.5, c=(1.0, 1.0, 1.0, 1.0), alpha=(1e-3, 1e-3, 1e-3, 1e-3))
    assert not W.precompute(2, 6, coefficients=cb)[0]["one_sided"]
    kw = dict(coefficients=cb, boundary=MIXED, kappa=0.5, sigma_dirichlet=1.0, phase=(0.4, 0.3))
    e1 = W.solve(2, 6, 0.1, **kw)
    e2 = W.solve(2, 12, 0.1, **kw)
    assert math.log2(e1["erru"] / e2["erru"]) > 2.5
    assert math.log2(e1["errE"] / e2["errE"]) > 1.5


class _Lin:
    """test/runtests.jl:33-38: u₀ = a|x - ½| + b x + y/2 (d = 0) and its derivatives ∂_x (d = 1),
    ∂_y (d = 2), ∂_xx = ∂_yy = 0 (d = 3)."""

    def __init__(self, a, b, d):
        self.a, self.b, self.d = a, b, d

    def __call__(self, x, y):
        if self.d == 0:
            return self.a * abs(x - 0.5) + self.b * x + 0.5 * y
        if self.d == 1:
            return (-self.a if x < 0.5 else self.a) + self.b
        return 0.5 if self.d == 2 else 0.0


def _lin_profile(a, b):
    return dict(u0=_Lin(a, b, 0), u0_x=_Lin(a, b, 1), u0_y=_Lin(a, b, 2), u0_xx=_Lin(a, b, 3), u0_yy=_Lin(a, b, 3))


def _project_u(f, pre, N):
    """test/runtests.jl:111-118: the L² projection of f on the u basis of every element."""
    P = pre["P_u"]
    z, w = W.GaussQCofs(pre["qu1"])
    h, n = 1.0 / N, P.shape[1]
    U = np.zeros((N, N, n, n), order="F")
    for k in range(N):
        for j in range(N):
            xs, ys = (k + 0.5) * h + h * z / 2, (j + 0.5) * h + h * z / 2
            M = np.array([[f(x, y) for x in xs] for y in ys])
            U[j, k] = P.T @ (w[:, None] * M * w[None, :]) @ P
    return U


def test_interface_terms_of_the_initial_profile(gpu):
    """test/runtests.jl:760-784: with u = ũ + u₀, the :initial_value RHS at (ũ, v) = (0, 0) equals
    the plain RHS at (u, v) = (u₀, 0) when u₀ lies in U_h: c jumping at x = ½ where ∂_n u₀ ≠ 0, and
    u₀ = |x - ½| + y/2 for a constant c. The jump terms of u₀ enter the one-sided faces (here
    projected on the face modes, the coefficients being one value along every face)."""
    from test_host import Step
    z0 = lambda x, y: 0.0   # noqa: E731
    N, h = 8, 1.0 / 8
    for c1, c2, ip in ((1.0, 0.5, _lin_profile(0.0, 1.0)), (0.8, 0.8, _lin_profile(1.0, 0.0))):
        coef = W.Coefficients(Step(1, 0.5, c1, c2), z0, z0, Step(1, 0.5, 1e-3 * c1 ** 2, 1e-3 * c2 ** 2), z0, z0, z0)
        for flux in ("upwind", "central", "alternating"):
            for q in (1, 3):
                kw = dict(coefficients=coef, boundary="wall", flux=flux)
                pI, _ = W.precompute(q, N, mode="initial_value", initial_profile=ip, **kw)
                pS, _ = W.precompute(q, N, mode="source", source=W.GaussianSource(amplitude=0.0), **kw)
                assert pI["one_sided"]
                zu, zv = np.zeros((N, N, pI["qu1"], pI["qu1"]), order="F"), np.zeros((N, N, pI["qv1"], pI["qv1"]), order="F")
                rI = tuple(x.copy() for x in W.Workspace(pI, N).rhs(zu, zv, 0.3))
                rS = W.Workspace(pS, N).rhs(_project_u(ip["u0"], pS, N), zv, 0.3)
                assert np.max(np.abs(rI[1] - rS[1])) <= 1e-11 * np.max(np.abs(rS[1])), (c1, flux, q)
                assert np.max(np.abs(rI[0] - rS[0])) <= 1e-11, (c1, flux, q)


def energy_terms(u, v, ut, vt, pre, coef, N):
    """test/runtests.jl:64-103: the terms of the semi-discrete energy identity (eq. (2.10) of the
    paper with the code's penalty weight) for a state (u, v) and its RHS (ut, vt), four walls with
    κ = 0 and no source, with the scheme's quadrature rules:
        dE/dt = Σ∫ c²∇u_h·∇u̇_h + Σ∫ (1 - 2βv_h) v_h v̇_h = -Σ∫ α|∇v_h|² - D_I,
        D_I = Σ_F ∫_F (½(c²₁ + c²₂)λ_u + ½(α₁ + α₂)λ_v) [[v_h]]² + τ ([[c²∇u_h]] + [[α∇v_h]])².
    Piecewise-constant coefficients: an element's one-sided values are those at its centre."""
    h, nu, nv, qh = 1.0 / N, pre["qu1"], pre["qv1"], pre["q_high"]
    z, w = W.GaussQCofs(nu)
    zh, wh = W.GaussQCofs(qh)
    Wq, Wh = np.outer(w, w), np.outer(wh, wh)
    Pu, Su, Pv, Sv, Ph = pre["P_u"], pre["S_u"], pre["P_v"], pre["S_v"], pre["P_h_v"]
    crd = lambda i, r: (i + 0.5) * h + h * np.asarray(r) / 2   # noqa: E731
    ev = np.vectorize(lambda f, x, y: f(x, y), excluded={0})
    T1 = T2 = Dv = scale = 0.0
    for k in range(N):
        for j in range(N):
            X, Y = np.meshgrid(crd(k, z), crd(j, z))              # X[r, s] = x_s, Y[r, s] = y_r
            Xh, Yh = np.meshgrid(crd(k, zh), crd(j, zh))
            U, Ud, V, Vd = u[j, k], ut[j, k], v[j, k], vt[j, k]
            c2 = ev(coef.c, X, Y) ** 2
            al = ev(coef.alpha, X, Y)
            bh = ev(coef.beta, Xh, Yh)
            vq = Ph @ V @ Ph.T
            t1 = Wq * c2 * ((Pu @ U @ Su.T) * (Pu @ Ud @ Su.T) + (Su @ U @ Pu.T) * (Su @ Ud @ Pu.T))
            t2 = (h * h / 4) * Wh * (1 - 2 * bh * vq) * vq * (Ph @ Vd @ Ph.T)
            T1 += t1.sum()
            T2 += t2.sum()
            scale += np.abs(t1).sum() + np.abs(t2).sum()
            Dv += (Wq * al * ((Pv @ V @ Sv.T) ** 2 + (Sv @ V @ Pv.T) ** 2)).sum()
    one = np.array([1.0])
    E = lambda n, x: np.array([W.JacobiP(one * x, 0, 0, d)[0] for d in range(n)])        # noqa: E731
    E1 = lambda n, x: np.array([W.GradJacobiP(one * x, 0, 0, d)[0] for d in range(n)])   # noqa: E731
    DI, wf = 0.0, (h / 2) * w
    for k in range(N):
        for j in range(N):
            for hz in (True, False):
                j2, k2 = (j + 1, k) if hz else (j, k + 1)        # element 2 above or to the right
                if j2 >= N or k2 >= N:
                    continue
                tr = (lambda Z, P, e: P @ (Z.T @ e)) if hz else (lambda Z, P, e: P @ (Z @ e))
                U1, V1, U2, V2 = u[j, k], v[j, k], u[j2, k2], v[j2, k2]
                jv = tr(V1, Pv, E(nv, 1.0)) - tr(V2, Pv, E(nv, -1.0))
                du1, du2 = (2 / h) * tr(U1, Pu, E1(nu, 1.0)), (2 / h) * tr(U2, Pu, E1(nu, -1.0))
                dv1, dv2 = (2 / h) * tr(V1, Pv, E1(nv, 1.0)), (2 / h) * tr(V2, Pv, E1(nv, -1.0))
                x1, y1, x2, y2 = crd(k, 0.0), crd(j, 0.0), crd(k2, 0.0), crd(j2, 0.0)
                a1, a2 = coef.c(x1, y1) ** 2, coef.c(x2, y2) ** 2
                b1, b2 = coef.alpha(x1, y1), coef.alpha(x2, y2)
                J = a1 * du1 - a2 * du2 + b1 * dv1 - b2 * dv2
                pen = 0.5 * (a1 + a2) * pre["lambda_u"] + 0.5 * (b1 + b2) * pre["lambda_v"]
                DI += (wf * (pen * jv ** 2 + pre["tau"] * J ** 2)).sum()
    return dict(dEdt=T1 + T2, Dv=Dv, DI=DI, scale=scale + Dv + DI)


ENERGY_FLUXES = (dict(theta=0.5, tau=0.0, lambda_u=0.0, lambda_v=0.0),      # central
                 dict(theta=1.0, tau=0.0, lambda_u=0.0, lambda_v=0.0),      # alternating
                 dict(theta=0.3, tau=0.0, lambda_u=0.0, lambda_v=0.0),
                 dict(theta=1.0, tau=1.0, lambda_u=1.0, lambda_v=1.0),      # upwind
                 dict(theta=0.5, tau=1.0, lambda_u=0.0, lambda_v=0.0),
                 dict(theta=0.3, tau=0.7, lambda_u=0.4, lambda_v=0.9))


def test_energy_identity_with_jumping_coefficients(gpu):
    """test/runtests.jl:734-761: for random states, c, α, β jumping on x = ½ and y = ½ (one-sided
    faces), four walls with κ = 0 and no source, the GPU RHS satisfies dE/dt = -Σ∫α|∇v_h|² - D_I to
    1e-12 of the terms' size (D_I = 0 for the fluxes without dissipation), so dE/dt ≤ 0; q = 1..4,
    both pairings, six flux parameter sets."""
    from test_oracle import quadrant_coefficients
    co = quadrant_coefficients(0.5, 0.5, beta=(0.0, 0.3, 0.1, 0.2))
    N, worst, rise = 4, 0.0, -math.inf
    for q in (1, 2, 3, 4):
        for mixed in (True, False):
            for fp in ENERGY_FLUXES:
                pre, _ = W.precompute(q, N, flux_params=fp, mixed=mixed, mode="source", boundary="wall", kappa=0.0,
                                      coefficients=co, source=W.GaussianSource(amplitude=0.0))
                rng = np.random.default_rng(10 * q + mixed)
                u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                ut, vt = (x.copy() for x in W.Workspace(pre, N).rhs(u, v, 0.3))
                et = energy_terms(u, v, ut, vt, pre, co, N)
                if fp["tau"] == 0 and fp["lambda_u"] == 0 and fp["lambda_v"] == 0:
                    assert et["DI"] == 0
                worst = max(worst, abs(et["dEdt"] + et["Dv"] + et["DI"]) / et["scale"])
                rise = max(rise, et["dEdt"] / et["scale"])
    assert worst < 1e-12, worst
    assert rise < 1e-12, rise


def two_layer_error(solve, Coefficients, q, N, T, flux, direction):
    """test/runtests.jl:125-152: the energy-norm error at T of the exact standing mode of a two-layer
    medium (c = 1 below s = ½, c = ½ above, s = x or y, four walls), started from its profile
    in :initial_value mode; `solve` and `Coefficients` are those of the package under test."""
    om, A = 2 * math.atan(math.sqrt(2.0)), -math.sqrt(3.0)
    phi = lambda s: np.where(s < 0.5, np.cos(om * s), A * np.cos(2 * om * (1 - s)))                    # noqa: E731
    dphi = lambda s: np.where(s < 0.5, -om * np.sin(om * s), 2 * om * A * np.sin(2 * om * (1 - s)))    # noqa: E731
    d2phi = lambda s: np.where(s < 0.5, -om ** 2 * np.cos(om * s), -(2 * om) ** 2 * A * np.cos(2 * om * (1 - s)))  # noqa: E731
    cs = lambda s: 1.0 if s < 0.5 else 0.5   # noqa: E731
    z0 = lambda x, y: 0.0   # noqa: E731
    f = lambda g: (lambda x, y: float(g(np.float64(x if direction == "x" else y))))   # noqa: E731
    co = Coefficients(lambda x, y: cs(x if direction == "x" else y), z0, z0, z0, z0, z0, z0)
    ip = dict(u0=f(phi), u0_x=f(dphi) if direction == "x" else z0, u0_y=z0 if direction == "x" else f(dphi),
              u0_xx=f(d2phi) if direction == "x" else z0, u0_yy=z0 if direction == "x" else f(d2phi))
    st = solve(q, N, T, mode="initial_value", initial_profile=ip, coefficients=co, boundary="wall", flux=flux,
               return_state=True)
    fu, fv = math.cos(om * T) - 1.0, -om * math.sin(om * T)      # ũ = u - Φ and v at T, times Φ
    h = st["h"]
    z, _ = W.GaussQCofs(q + 1)
    e = 0.0
    for j in range(N):
        for k in range(N):
            if direction == "x":
                S = np.tile(((k + 0.5) * h + h * z / 2)[None, :], (q + 1, 1))
            else:
                S = np.tile(((j + 0.5) * h + h * z / 2)[:, None], (1, q + 1))
            U, V = st["u"][j, k], st["v"][j, k]
            ux = (2 / h) * (st["P_u"] @ U @ st["S_u"].T)
            uy = (2 / h) * (st["S_u"] @ U @ st["P_u"].T)
            g = fu * dphi(S)
            gx, gy = (g, np.zeros_like(S)) if direction == "x" else (np.zeros_like(S), g)
            e += np.sum(st["W2d"] * (0.5 * st["err_c2"][j, k] * ((gx - ux) ** 2 + (gy - uy) ** 2)
                                     + 0.5 * (fv * phi(S) - st["P_v"] @ V @ st["P_v"].T) ** 2))
    return h / 2 * math.sqrt(e)


def test_convergence_at_a_coefficient_jump(gpu):
    """test/runtests.jl:816-823: the two-layer standing mode converges at about q_u in the energy
    norm for the upwind flux and about 1 for the central flux (q_u = 2, meshes 8 → 16), and the
    interface along y gives the same error as along x."""
    e8 = two_layer_error(W.solve, W.Coefficients, 2, 8, 0.5, "upwind", "x")
    e16 = two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "upwind", "x")
    assert math.log2(e8 / e16) > 1.8
    assert two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "upwind", "y") == pytest.approx(e16, rel=1e-10)
    c8 = two_layer_error(W.solve, W.Coefficients, 2, 8, 0.5, "central", "x")
    c16 = two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "central", "x")
    assert math.log2(c8 / c16) > 0.9
