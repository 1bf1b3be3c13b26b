"""Helpers of the reference's property tests (test/runtests.jl), restated for this repository's
tests: the initial profile u₀ = a|x - ½| + b x + y/2 and the L² projection on the element bases,
the terms of the semi-discrete energy identity, and the energy-norm error of the two-layer
standing mode. They take the package under test (the product or the oracle) as arguments where
they run it, so that the CPU suite pins them on the oracle and the GPU suite applies them to the
product.
"""
import math

import numpy as np

import edg_westervelt_gb300 as W


class Lin:
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


def lin_profile(a, b):
    return dict(u0=Lin(a, b, 0), u0_x=Lin(a, b, 1), u0_y=Lin(a, b, 2), u0_xx=Lin(a, b, 3), u0_yy=Lin(a, b, 3))


def project_u(f, pre, N):
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
