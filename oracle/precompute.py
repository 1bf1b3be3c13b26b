"""``precompute`` of WesterveltEDG.jl, restated for the oracle.

Test infrastructure only. Follows ``src/solver.jl:341-770``: the element
operators, face coefficients and data arrays read by the right-hand side,
with the reference's array names, shapes and (column-major) memory layouts.
Indices are 0-based here; the shapes are the Julia ones, so that
``pre["Cw"][r, e, s]`` is Julia's ``pre.Cw[r+1, e+1, s+1]`` and the memory
order is identical (arrays are Fortran-ordered).
"""
import math

import numpy as np

from .coefficients import (Coefficients, GaussianSource, boundary_sides,
                           flux_parameters, paper_coefficients)
from .quadrature import gauss_q_cofs, grad_jacobi_p, jacobi_p

FACE_SHIFT = 2.0 ** -40   # src/solver.jl:361
JUMP_TOL = 1e-8           # src/solver.jl:362


def _zeros(*shape):
    return np.zeros(shape, dtype=np.float64, order="F")


def _ev(f, X, Y):
    """f at the points (X, Y): vectorised when f accepts arrays, else point by point."""
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    try:
        with np.errstate(all="ignore"):
            r = f(X, Y)
        r = np.asarray(r, dtype=np.float64)
        if r.shape == X.shape:
            return r
        if r.shape == ():
            return np.full(X.shape, float(r))
    except (TypeError, ValueError):
        pass
    out = np.empty(X.shape)
    for idx in np.ndindex(X.shape):
        out[idx] = f(float(X[idx]), float(Y[idx]))
    return out


def side_values(bot, top, lft, rgt, f, xloc, yloc, N, h):
    """One-sided face values of f (src/solver.jl:371-408).

    bot[j, k, i] is the value at point i of the bottom side of element (j, k)
    seen from inside it; likewise top, lft, rgt. Pass None to skip a pair.
    """
    nq = xloc.shape[1]
    d = FACE_SHIFT
    hz = bot is not None
    vt = lft is not None
    if hz:
        # face rows jf = 0..N at y = jf*h, columns k; point i along x
        X = np.empty((nq, N + 1, N))
        Yf = np.empty((nq, N + 1, N))
        for k in range(N):
            for jf in range(N + 1):
                X[:, jf, k] = xloc[k, :]
                Yf[:, jf, k] = jf * h
        H0 = _ev(f, X, Yf)
        HM = H0.copy()
        HP = H0.copy()
        HM[:, 1:, :] = _ev(f, X[:, 1:, :], Yf[:, 1:, :] - d)
        HP[:, :N, :] = _ev(f, X[:, :N, :], Yf[:, :N, :] + d)
    if vt:
        Xf = np.empty((nq, N, N + 1))
        Y = np.empty((nq, N, N + 1))
        for j in range(N):
            for kf in range(N + 1):
                Xf[:, j, kf] = kf * h
                Y[:, j, kf] = yloc[j, :]
        V0 = _ev(f, Xf, Y)
        VM = V0.copy()
        VP = V0.copy()
        VM[:, :, 1:] = _ev(f, Xf[:, :, 1:] - d, Y[:, :, 1:])
        VP[:, :, :N] = _ev(f, Xf[:, :, :N] + d, Y[:, :, :N])

    def amax(A):
        A = A[np.isfinite(A)]
        return float(np.max(np.abs(A))) if A.size else 0.0

    sh = max(amax(HM[:, 1:, :]), amax(HP[:, :N, :])) if hz else 0.0
    sv = max(amax(VM[:, :, 1:]), amax(VP[:, :, :N])) if vt else 0.0
    s = JUMP_TOL * max(sh, sv)

    def sides(f0, fm, fp):
        # (f0, f0) where f0 is finite and both shifted values are near it, else (fm, fp)
        with np.errstate(invalid="ignore"):
            near_m = np.abs(fm - f0) <= JUMP_TOL * np.maximum(np.abs(fm), np.abs(f0)) + s
            near_p = np.abs(fp - f0) <= JUMP_TOL * np.maximum(np.abs(fp), np.abs(f0)) + s
        keep = np.isfinite(f0) & near_m & near_p
        return np.where(keep, f0, fm), np.where(keep, f0, fp)

    if hz:
        fm, fp = sides(H0, HM, HP)
        for jf in range(N + 1):
            if jf >= 1:
                top[jf - 1, :, :] = fm[:, jf, :].T
            if jf <= N - 1:
                bot[jf, :, :] = fp[:, jf, :].T
    if vt:
        fm, fp = sides(V0, VM, VP)
        for kf in range(N + 1):
            if kf >= 1:
                rgt[:, kf - 1, :] = fm[:, :, kf].T
            if kf <= N - 1:
                lft[:, kf, :] = fp[:, :, kf].T


def precompute(q, N, mixed=True, flux="upwind", flux_params=None, sigma=0.0,
               boundary="absorbing_2beta", sigma_dirichlet=None, kappa=0.0,
               phase=(0.0, 0.0), coefficients=None, mode="mms", kx=1, ky=1,
               source=None, mass_solver="chebyshev", initial_profile=None):
    """src/solver.jl:428-694. Returns (pre, geo) as dicts."""
    if sigma_dirichlet is None:
        sigma_dirichlet = sigma
    if coefficients is None:
        coefficients = paper_coefficients()
    if source is None:
        source = GaussianSource()
    if mass_solver not in ("cg", "chebyshev"):
        raise ValueError(f"unknown mass_solver {mass_solver} (expected :cg or :chebyshev)")
    if initial_profile is not None and mode != "initial_value":
        raise ValueError("initial_profile is only available in :initial_value mode")
    if mode not in ("mms", "initial_value", "source"):
        raise ValueError(f"unknown mode {mode} (expected :mms, :initial_value or :source)")
    q_u = q
    q_v = q_u - 1 if mixed else q_u
    qu1 = q_u + 1
    qv1 = q_v + 1
    h = 1.0 / N
    omega = 2 * math.pi * math.sqrt(kx ** 2 + ky ** 2)
    fp = flux_parameters(flux) if flux_params is None else {
        k: float(flux_params[k]) for k in ("theta", "tau", "lambda_u", "lambda_v")}
    bc = boundary_sides(boundary, sigma, sigma_dirichlet, kappa)
    legacy = boundary in ("absorbing", "dirichlet")
    gamma_abc = bc["bot"]["gamma_abc"] if legacy else math.nan
    px, py = phase
    C = coefficients
    pi = math.pi

    z, w = gauss_q_cofs(qu1)
    W2d = np.asfortranarray(np.outer(w, w))
    P_u = _zeros(qu1, qu1)
    S_u = _zeros(qu1, qu1)
    Ebl_u = _zeros(1, qu1)
    Ebr_u = _zeros(1, qu1)
    E1bl_u = _zeros(1, qu1)
    E1br_u = _zeros(1, qu1)
    for d in range(qu1):
        P_u[:, d] = jacobi_p(z, 0, 0, d)
        S_u[:, d] = grad_jacobi_p(z, 0, 0, d)
        Ebl_u[0, d] = jacobi_p(-1.0, 0, 0, d)
        Ebr_u[0, d] = jacobi_p(1.0, 0, 0, d)
        E1bl_u[0, d] = grad_jacobi_p(-1.0, 0, 0, d)
        E1br_u[0, d] = grad_jacobi_p(1.0, 0, 0, d)
    P_v = np.asfortranarray(P_u[:, :qv1])
    Ebl_v = np.asfortranarray(Ebl_u[:, :qv1])
    Ebr_v = np.asfortranarray(Ebr_u[:, :qv1])
    E1bl_v = np.asfortranarray(E1bl_u[:, :qv1])
    E1br_v = np.asfortranarray(E1br_u[:, :qv1])

    q_high = max(int(math.ceil(3 * q_v / 2) + 1), q_u + 1)
    z_h, w_h = gauss_q_cofs(q_high)
    W2d_h = np.asfortranarray(np.outer(w_h, w_h))
    P_h_v = _zeros(q_high, qv1)
    for d in range(qv1):
        P_h_v[:, d] = jacobi_p(z_h, 0, 0, d)
    Phi2d_h_v = np.asfortranarray(np.kron(P_h_v, P_h_v))
    Phi_xi_u = np.kron(P_u, S_u)
    Phi_eta_u = np.kron(S_u, P_u)
    S_v = np.asfortranarray(S_u[:, :qv1])

    xloc = _zeros(N, qu1)
    xloc_h = _zeros(N, q_high)
    for i in range(N):
        xloc[i, :] = (i * h + (i + 1) * h + h * z) / 2
        xloc_h[i, :] = (i * h + (i + 1) * h + h * z_h) / 2
    yloc = xloc.copy(order="F")
    yloc_h = xloc_h.copy(order="F")

    # volume data and the packed inverse of the pinned c²-stiffness (solver.jl:513-536)
    E = N * N
    Cw = _zeros(qu1, E, qu1)
    Aw = _zeros(qu1, E, qu1)
    nu2 = qu1 * qu1
    Ainv_u = _zeros(nu2 * (nu2 + 1) // 2, E)
    # all element points at once: XQ[j, k, r, s] = x_s of column k, YQ = y_r of row j
    XQ = np.broadcast_to(xloc[None, :, None, :], (N, N, qu1, qu1))
    YQ = np.broadcast_to(yloc[:, None, :, None], (N, N, qu1, qu1))
    cQ = _ev(C.c, XQ, YQ)
    aQ = _ev(C.alpha, XQ, YQ)
    iu, ju = np.triu_indices(nu2)      # (row ii <= column jj)
    tri_rows = ju * (ju + 1) // 2 + iu
    for k in range(N):
        for j in range(N):
            e = j + k * N
            Cw[:, e, :] = cQ[j, k] ** 2 * W2d
            Aw[:, e, :] = aQ[j, k] * W2d
    # M_e = Φ_ξ' diag(c²W) Φ_ξ + Φ_η' diag(c²W) Φ_η, (1,1) += 1; inverse via Cholesky, element by element
    # (elements stacked in chunks for numpy)
    for e0 in range(0, E, 1024):
        es = range(e0, min(E, e0 + 1024))
        cw = np.stack([Cw[:, e, :].reshape(-1, order="F") for e in es])
        M = (np.einsum("pi,ep,pj->eij", Phi_xi_u, cw, Phi_xi_u, optimize=True)
             + np.einsum("pi,ep,pj->eij", Phi_eta_u, cw, Phi_eta_u, optimize=True))
        M[:, 0, 0] += 1.0
        L = np.linalg.cholesky(M)
        Li = np.linalg.inv(L)
        Aj = np.einsum("eki,ekj->eij", Li, Li, optimize=True)
        Ainv_u[np.ix_(tri_rows, np.arange(e0, e0 + len(es)))] = Aj[:, iu, ju].T

    # one-sided face values of c, alpha, beta (solver.jl:541-552)
    faces = {}
    for name in ("bot", "top", "lft", "rgt"):
        faces[name] = {key: _zeros(N, N, qu1) for key in ("c2", "af", "cf", "bf")}
    for fun, key in ((C.c, "cf"), (C.alpha, "af"), (C.beta, "bf")):
        side_values(faces["bot"][key], faces["top"][key], faces["lft"][key], faces["rgt"][key],
                    fun, xloc, yloc, N, h)
    for name in ("bot", "top", "lft", "rgt"):
        faces[name]["c2"][...] = faces[name]["cf"] ** 2

    # ∂_e u0 seen from inside the elements (solver.jl:558-568)
    g0 = {s: _zeros(N, N, qu1) for s in ("bot", "top", "lft", "rgt")}
    if mode != "source":
        if initial_profile is None:
            def u0_x(x, y):
                return -2 * pi * kx * np.sin(2 * pi * kx * x + px) * np.sin(2 * pi * ky * y + py)

            def u0_y(x, y):
                return 2 * pi * ky * np.cos(2 * pi * kx * x + px) * np.cos(2 * pi * ky * y + py)
        else:
            u0_x = initial_profile["u0_x"]
            u0_y = initial_profile["u0_y"]
        side_values(g0["bot"], g0["top"], None, None, u0_y, xloc, yloc, N, h)
        side_values(None, None, g0["lft"], g0["rgt"], u0_x, xloc, yloc, N, h)

    # manufactured-solution data at the high-order points (solver.jl:570-602)
    XH = np.broadcast_to(xloc_h[None, :, None, :], (N, N, q_high, q_high))
    YH = np.broadcast_to(yloc_h[:, None, :, None], (N, N, q_high, q_high))
    if initial_profile is None:
        sp = np.cos(2 * pi * kx * XH + px) * np.sin(2 * pi * ky * YH + py)
        sp_x = -2 * pi * kx * np.sin(2 * pi * kx * XH + px) * np.sin(2 * pi * ky * YH + py)
        sp_y = 2 * pi * ky * np.cos(2 * pi * kx * XH + px) * np.cos(2 * pi * ky * YH + py)
        sp_xx = -(2 * pi * kx) ** 2 * sp
        sp_yy = -(2 * pi * ky) ** 2 * sp
    else:
        ip = initial_profile
        sp = _ev(ip["u0"], XH, YH)
        sp_x = _ev(ip["u0_x"], XH, YH)
        sp_y = _ev(ip["u0_y"], XH, YH)
        sp_xx = _ev(ip["u0_xx"], XH, YH)
        sp_yy = _ev(ip["u0_yy"], XH, YH)
    cf = _ev(C.c, XH, YH)
    c2 = cf ** 2
    cx = _ev(C.c_x, XH, YH)
    cy = _ev(C.c_y, XH, YH)
    c2x = 2 * cf * cx
    c2y = 2 * cf * cy
    af = _ev(C.alpha, XH, YH)
    ax = _ev(C.alpha_x, XH, YH)
    ay = _ev(C.alpha_y, XH, YH)
    mms_SP = np.asfortranarray(sp)
    mms_Cdiv = np.asfortranarray(c2x * sp_x + c2y * sp_y + c2 * (sp_xx + sp_yy))
    mms_Ddiv = np.asfortranarray(ax * sp_x + ay * sp_y + af * (sp_xx + sp_yy))
    mms_BF = np.asfortranarray(_ev(C.beta, XH, YH))

    # Φ and ∇Φ on the physical boundary (solver.jl:604-635)
    bc_bot_sp = _zeros(N, qu1)
    bc_bot_spy = _zeros(N, qu1)
    bc_top_sp = _zeros(N, qu1)
    bc_top_spy = _zeros(N, qu1)
    bc_lft_sp = _zeros(N, qu1)
    bc_lft_spx = _zeros(N, qu1)
    bc_rgt_sp = _zeros(N, qu1)
    bc_rgt_spx = _zeros(N, qu1)
    for k in range(N):
        xq = xloc[k, :]
        bc_bot_sp[k, :] = np.cos(2 * pi * kx * xq + px) * math.sin(2 * pi * ky * 0 + py)
        bc_bot_spy[k, :] = 2 * pi * ky * np.cos(2 * pi * kx * xq + px) * math.cos(2 * pi * ky * 0 + py)
        bc_top_sp[k, :] = np.cos(2 * pi * kx * xq + px) * math.sin(2 * pi * ky * 1 + py)
        bc_top_spy[k, :] = 2 * pi * ky * np.cos(2 * pi * kx * xq + px) * math.cos(2 * pi * ky * 1 + py)
    for j in range(N):
        yq = yloc[j, :]
        bc_lft_sp[j, :] = math.cos(2 * pi * kx * 0 + px) * np.sin(2 * pi * ky * yq + py)
        bc_lft_spx[j, :] = -2 * pi * kx * math.sin(2 * pi * kx * 0 + px) * np.sin(2 * pi * ky * yq + py)
        bc_rgt_sp[j, :] = math.cos(2 * pi * kx * 1 + px) * np.sin(2 * pi * ky * yq + py)
        bc_rgt_spx[j, :] = -2 * pi * kx * math.sin(2 * pi * kx * 1 + px) * np.sin(2 * pi * ky * yq + py)
    if initial_profile is not None:
        ip = initial_profile
        for k in range(N):
            xq = xloc[k, :]
            zq = np.zeros_like(xq)
            bc_bot_sp[k, :] = _ev(ip["u0"], xq, zq)
            bc_bot_spy[k, :] = _ev(ip["u0_y"], xq, zq)
            bc_top_sp[k, :] = _ev(ip["u0"], xq, zq + 1.0)
            bc_top_spy[k, :] = _ev(ip["u0_y"], xq, zq + 1.0)
        for j in range(N):
            yq = yloc[j, :]
            zq = np.zeros_like(yq)
            bc_lft_sp[j, :] = _ev(ip["u0"], zq, yq)
            bc_lft_spx[j, :] = _ev(ip["u0_x"], zq, yq)
            bc_rgt_sp[j, :] = _ev(ip["u0"], zq + 1.0, yq)
            bc_rgt_spx[j, :] = _ev(ip["u0_x"], zq + 1.0, yq)

    # c² and β at the standard points (solver.jl:637-645)
    err_c2 = np.asfortranarray(cQ ** 2)
    err_beta = np.asfortranarray(_ev(C.beta, XQ, YQ))

    src_on = mode == "source"
    src_proj = _zeros(N, N, qv1, qv1)
    if src_on:
        for A in (mms_SP, mms_Cdiv, mms_Ddiv, bc_bot_sp, bc_bot_spy, bc_top_sp, bc_top_spy,
                  bc_lft_sp, bc_lft_spx, bc_rgt_sp, bc_rgt_spx):
            A.fill(0.0)
        g = source.amplitude * np.exp(-((XH - source.x0[0]) ** 2 + (YH - source.x0[1]) ** 2) / source.r0 ** 2)
        for k in range(N):
            for j in range(N):
                src_proj[j, k] = P_h_v.T @ (W2d_h * g[j, k]) @ P_h_v

    pre = dict(
        N=N, qu1=qu1, qv1=qv1, q_high=q_high, omega=omega, w=w,
        P_u=P_u, P_v=P_v, S_u=S_u, S_v=S_v,
        Ebl_u=Ebl_u, Ebr_u=Ebr_u, E1bl_u=E1bl_u, E1br_u=E1br_u,
        Ebl_v=Ebl_v, Ebr_v=Ebr_v, E1bl_v=E1bl_v, E1br_v=E1br_v,
        W2d_h=W2d_h, P_h_v=P_h_v, Phi2d_h_v=Phi2d_h_v,
        Cw=Cw, Aw=Aw, Ainv_u=Ainv_u,
        mms_SP=mms_SP, mms_Cdiv=mms_Cdiv, mms_Ddiv=mms_Ddiv, mms_BF=mms_BF,
        bc_bot_sp=bc_bot_sp, bc_bot_spy=bc_bot_spy, bc_top_sp=bc_top_sp, bc_top_spy=bc_top_spy,
        bc_lft_sp=bc_lft_sp, bc_lft_spx=bc_lft_spx, bc_rgt_sp=bc_rgt_sp, bc_rgt_spx=bc_rgt_spx,
        theta=fp["theta"], tau=fp["tau"], lambda_u=fp["lambda_u"], lambda_v=fp["lambda_v"],
        gamma_abc=gamma_abc, eta_abc=math.sqrt(1.0 - gamma_abc ** 2) if legacy else math.nan,
        sigma=bc["bot"]["sigma"] if legacy else math.nan,
        bc=bc, src_on=src_on, src_proj=src_proj, source=source,
        mms_on=mode == "mms", mass_solver=mass_solver,
    )
    for name in ("bot", "top", "lft", "rgt"):
        for key in ("c2", "af", "cf", "bf"):
            pre[f"{name}_{key}"] = faces[name][key]
        pre[f"{name}_g0"] = g0[name]
    pre.update(_rhs_data(pre, N))
    geo = dict(S_u=S_u, W2d=W2d, xloc=xloc, yloc=yloc, err_c2=err_c2, err_beta=err_beta)
    return pre, geo


def src_time(pre, t):
    """src/solver.jl:662: sin(ωt) sin²(πt/Ts) for t < Ts in :source mode, else 0."""
    s = pre["source"]
    if pre["src_on"] and t < s.Ts:
        return math.sin(s.omega * t) * math.sin(math.pi * t / s.Ts) ** 2
    return 0.0


def _rhs_data(pre, N):
    """Face arrays by face, jumps, projections, transposes (src/solver.jl:716-770)."""
    nq = pre["qu1"]
    qh = pre["q_high"]
    E = N * N

    def hface(bot, top):
        A = _zeros(nq, N + 1, N)
        for k in range(N):
            for j in range(N):
                A[:, j, k] = bot[j, k, :]
            A[:, N, k] = top[N - 1, k, :]
        return A

    def vface(lft, rgt):
        A = _zeros(nq, N, N + 1)
        for k in range(N):
            for j in range(N):
                A[:, j, k] = lft[j, k, :]
        for j in range(N):
            A[:, j, N] = rgt[j, N - 1, :]
        return A

    def hfaceM(bot, top):
        A = _zeros(nq, N + 1, N)
        for k in range(N):
            A[:, 0, k] = bot[0, k, :]
            for j in range(N):
                A[:, j + 1, k] = top[j, k, :]
        return A

    def vfaceM(lft, rgt):
        A = _zeros(nq, N, N + 1)
        for j in range(N):
            A[:, j, 0] = lft[j, 0, :]
        for k in range(N):
            for j in range(N):
                A[:, j, k + 1] = rgt[j, k, :]
        return A

    Ph = pre["P_h_v"]
    Wh = pre["W2d_h"]

    def proj(X):
        nv = pre["qv1"]
        Pi = _zeros(nv, nv, N, N)
        for k in range(N):
            for j in range(N):
                Pi[:, :, j, k] = Ph.T @ (Wh * X[j, k]) @ Ph
        return Pi

    def elast(X):
        return np.asfortranarray(np.transpose(X, (2, 3, 0, 1)))

    p = pre
    hc2 = hface(p["bot_c2"], p["top_c2"])
    hc2m = hfaceM(p["bot_c2"], p["top_c2"])
    haf = hface(p["bot_af"], p["top_af"])
    hafm = hfaceM(p["bot_af"], p["top_af"])
    vc2 = vface(p["lft_c2"], p["rgt_c2"])
    vc2m = vfaceM(p["lft_c2"], p["rgt_c2"])
    vaf = vface(p["lft_af"], p["rgt_af"])
    vafm = vfaceM(p["lft_af"], p["rgt_af"])
    hg0 = hface(p["bot_g0"], p["top_g0"])
    hg0m = hfaceM(p["bot_g0"], p["top_g0"])
    vg0 = vface(p["lft_g0"], p["rgt_g0"])
    vg0m = vfaceM(p["lft_g0"], p["rgt_g0"])

    def differ(a, b):
        # Julia's != on arrays: elementwise ==, NaN never equal
        return not np.array_equal(a, b)

    jumps = differ(hc2m, hc2) or differ(hafm, haf) or differ(vc2m, vc2) or differ(vafm, vaf)
    if p["mms_on"] and jumps:
        raise ValueError("mode = :mms needs c and α continuous across the element faces; "
                         "use :initial_value or :source for coefficients that jump")
    hJC = np.asfortranarray(hc2m * hg0m - hc2 * hg0)
    vJC = np.asfortranarray(vc2m * vg0m - vc2 * vg0)
    hJC[:, 0, :] = 0.0
    hJC[:, N, :] = 0.0
    vJC[:, :, 0] = 0.0
    vJC[:, :, N] = 0.0
    one_sided = jumps or bool(np.any(hJC != 0)) or bool(np.any(vJC != 0))
    beta_hE = elast(p["mms_BF"])
    return dict(
        hc2=hc2, haf=haf, hcf=hface(p["bot_cf"], p["top_cf"]), hbf=hface(p["bot_bf"], p["top_bf"]),
        vc2=vc2, vaf=vaf, vcf=vface(p["lft_cf"], p["rgt_cf"]), vbf=vface(p["lft_bf"], p["rgt_bf"]),
        hc2m=hc2m, hafm=hafm, vc2m=vc2m, vafm=vafm, hJC=hJC, vJC=vJC, one_sided=one_sided,
        bcB_sp=np.asfortranarray(p["bc_bot_sp"].T), bcB_spy=np.asfortranarray(p["bc_bot_spy"].T),
        bcT_sp=np.asfortranarray(p["bc_top_sp"].T), bcT_spy=np.asfortranarray(p["bc_top_spy"].T),
        bcL_sp=np.asfortranarray(p["bc_lft_sp"].T), bcL_spx=np.asfortranarray(p["bc_lft_spx"].T),
        bcR_sp=np.asfortranarray(p["bc_rgt_sp"].T), bcR_spx=np.asfortranarray(p["bc_rgt_spx"].T),
        PiSP=proj(p["mms_SP"]), PiBSP2=proj(p["mms_BF"] * p["mms_SP"] ** 2),
        PiCdiv=proj(p["mms_Cdiv"]), PiDdiv=proj(p["mms_Ddiv"]),
        src_projE=elast(p["src_proj"]), beta_hE=beta_hE,
        beta_hq=np.asfortranarray(np.transpose(beta_hE.reshape(qh, qh, E, order="F"), (0, 2, 1))),
        W_hq=np.asfortranarray(p["W2d_h"].reshape(qh, 1, qh, order="F")),
        P_h_vT=np.asfortranarray(p["P_h_v"].T), mass_tol=1e-14,
    )
