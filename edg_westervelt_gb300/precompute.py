"""``precompute`` of WesterveltEDG.jl: the host data the GPU workspace reads.

Mirrors src/solver.jl:341-770 (``precompute``, ``_side_values!``,
``_rhs_data``) and returns the reference's ``pre`` and ``geo`` as dicts with
its array names, shapes and column-major memory layouts (numpy arrays in
Fortran order, indices 0-based), so that ``pre["Cw"][r, e, s]`` is Julia's
``pre.Cw[r+1, e+1, s+1]`` at the same memory offset. The work is vectorised
over the mesh; the inverse pinned stiffness ``Ainv_u`` is computed once per
distinct element matrix (all elements share one for constant coefficients).
With ``inverses="device"`` (the default) and more than 64 distinct element
matrices, ``Ainv_u`` is left to the GPU workspace (``pre["Ainv_u"]`` is None and
wedg_create computes the inverses on the device from ``Cw``).
"""
import math

import numpy as np

from .coefficients import (GaussianSource, _Cells, _Const, _sym, boundary_sides, flux_parameters,
                           paper_coefficients)
from .errors import ArgumentErrorException
from .quadrature import GaussQCofs, GradJacobiP, JacobiP

FACE_SHIFT = 2.0 ** -40   # src/solver.jl:361
JUMP_TOL = 1e-8           # src/solver.jl:362


def _F(a):
    return np.asfortranarray(a, dtype=np.float64)


def evaluate(f, X, Y):
    """f at the points (X, Y): one vectorised call when f accepts arrays, else point by point."""
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    try:
        with np.errstate(all="ignore"):
            r = np.asarray(f(X, Y), dtype=np.float64)
        if r.shape == X.shape:
            return r
        if r.shape == ():
            return np.full(X.shape, float(r))
    except (TypeError, ValueError):
        pass
    fv = np.frompyfunc(lambda a, b: float(f(float(a), float(b))), 2, 1)
    return fv(X, Y).astype(np.float64)


def _sides(H0, HM, HP, s):
    """Values seen from the "-" and "+" side of every face point (src/solver.jl:389-392)."""
    with np.errstate(invalid="ignore"):
        near_m = np.abs(HM - H0) <= JUMP_TOL * np.maximum(np.abs(HM), np.abs(H0)) + s
        near_p = np.abs(HP - H0) <= JUMP_TOL * np.maximum(np.abs(HP), np.abs(H0)) + s
    use0 = np.isfinite(H0) & near_m & near_p
    return np.where(use0, H0, HM), np.where(use0, H0, HP)


def _amax(A):
    """max |A| over the finite entries of A (0 if none)."""
    if A.size == 0:
        return 0.0
    m = float(np.max(np.abs(A)))
    if math.isfinite(m):
        return m
    A = A[np.isfinite(A)]
    return float(np.max(np.abs(A))) if A.size else 0.0


def side_values(f, xloc, yloc, N, h, horizontal=True, vertical=True):
    """One-sided values of f on the sides of every element (src/solver.jl:371-408).

    Returns dict side -> (N, N, nq) arrays for the requested families; a side
    value is f(x_f ± δe) where f jumps across the face, f(x_f) where it is
    continuous to the tolerance (bitwise the plain point value then).
    """
    nq = xloc.shape[1]
    d = FACE_SHIFT
    out = {}
    if horizontal:
        X = np.broadcast_to(xloc.T[:, None, :], (nq, N + 1, N))            # [i, jf, k] = xloc[k, i]
        Yf = np.broadcast_to((np.arange(N + 1) * h)[None, :, None], (nq, N + 1, N))
        H0 = evaluate(f, X, Yf)
        HM = H0.copy()
        HP = H0.copy()
        HM[:, 1:, :] = evaluate(f, X[:, 1:, :], Yf[:, 1:, :] - d)
        HP[:, :N, :] = evaluate(f, X[:, :N, :], Yf[:, :N, :] + d)
    if vertical:
        Xf = np.broadcast_to((np.arange(N + 1) * h)[None, None, :], (nq, N, N + 1))
        Y = np.broadcast_to(yloc.T[:, :, None], (nq, N, N + 1))             # [i, j, kf] = yloc[j, i]
        V0 = evaluate(f, Xf, Y)
        VM = V0.copy()
        VP = V0.copy()
        VM[:, :, 1:] = evaluate(f, Xf[:, :, 1:] - d, Y[:, :, 1:])
        VP[:, :, :N] = evaluate(f, Xf[:, :, :N] + d, Y[:, :, :N])
    sh = max(_amax(HM[:, 1:, :]), _amax(HP[:, :N, :])) if horizontal else 0.0
    sv = max(_amax(VM[:, :, 1:]), _amax(VP[:, :, :N])) if vertical else 0.0
    s = JUMP_TOL * max(sh, sv)
    if horizontal:
        fm, fp = _sides(H0, HM, HP, s)
        out["top"] = _F(np.transpose(fm[:, 1:, :], (1, 2, 0)))
        out["bot"] = _F(np.transpose(fp[:, :N, :], (1, 2, 0)))
    if vertical:
        fm, fp = _sides(V0, VM, VP, s)
        out["rgt"] = _F(np.transpose(fm[:, :, 1:], (1, 2, 0)))
        out["lft"] = _F(np.transpose(fp[:, :, :N], (1, 2, 0)))
    return out


def _packed_inverses(Cw_blocks, Phi_xi, Phi_eta, chunk=2048):
    """Packed upper triangles (by columns) of inv(pinned c²-stiffness) for element blocks
    Cw_blocks (n, nq*nq) in column-major point order (src/solver.jl:528-535)."""
    n2 = Phi_xi.shape[1]
    iu, ju = np.triu_indices(n2)
    order = np.argsort(ju * (ju + 1) // 2 + iu)
    iu, ju = iu[order], ju[order]
    out = np.empty((Cw_blocks.shape[0], n2 * (n2 + 1) // 2))
    for c0 in range(0, Cw_blocks.shape[0], chunk):
        cw = Cw_blocks[c0:c0 + chunk]
        M = (np.einsum("pi,ep,pj->eij", Phi_xi, cw, Phi_xi, optimize=True)
             + np.einsum("pi,ep,pj->eij", Phi_eta, cw, Phi_eta, optimize=True))
        M[:, 0, 0] += 1.0
        L = np.linalg.cholesky(M)
        Li = np.linalg.inv(L)
        A = np.einsum("eki,ekj->eij", Li, Li)
        out[c0:c0 + chunk] = A[:, iu, ju]
    return out


def _distinct_rows(a, limit=None):
    """The distinct rows of a (E, n) array and each row's index among them, as
    np.unique(a, axis=0, return_inverse=True) gives them up to their order, without sorting
    the rows: all rows equal (constant coefficients) is checked directly, otherwise the rows
    are grouped by a projection key (a 1D sort) and the groups are checked to hold equal rows,
    with the row sort as the fallback when a key is shared by different rows. With `limit`,
    (None, None) when there are more distinct rows than that."""
    if a.shape[0] == 0 or np.array_equal(a, np.broadcast_to(a[0], a.shape)):
        return a[:1], np.zeros(a.shape[0], dtype=np.int64)
    key = a @ np.random.default_rng(0).uniform(1.0, 2.0, a.shape[1])
    ukey, first, inv = np.unique(key, return_index=True, return_inverse=True)
    if limit is not None and ukey.shape[0] > limit:
        return None, None                    # at least as many distinct rows as distinct keys
    uniq = a[first]
    if not np.array_equal(uniq[inv], a):
        uniq, inv = np.unique(a, axis=0, return_inverse=True)
        if limit is not None and uniq.shape[0] > limit:
            return None, None
    return uniq, inv.reshape(-1)


def precompute(q, N, *, mixed=True, flux="upwind", flux_params=None, sigma=0.0, boundary="absorbing_2beta",
               sigma_dirichlet=None, kappa=0.0, phase=(0.0, 0.0), coefficients=None, mode="mms", kx=1, ky=1,
               source=None, mass_solver="chebyshev", initial_profile=None, inverses="device", target="host"):
    """Element operators, face coefficients and data arrays of the RHS (``pre``) and the
    quadrature geometry for errors and diagnostics (``geo``); src/solver.jl:428-694.

    Keywords as the reference's ``precompute`` (symbols as strings, e.g. flux="upwind").
    target="device": the large arrays are left to the GPU workspace, which forms them from the
    coefficient functions' values at the point grids (precompute_points, wedg_create_points).
    """
    if target == "device":
        return precompute_points(q, N, mixed=mixed, flux=flux, flux_params=flux_params, sigma=sigma,
                                 boundary=boundary, sigma_dirichlet=sigma_dirichlet, kappa=kappa, phase=phase,
                                 coefficients=coefficients, mode=mode, kx=kx, ky=ky, source=source,
                                 mass_solver=mass_solver, initial_profile=initial_profile)
    if target != "host":
        raise ArgumentErrorException(f"target must be \"host\" or \"device\", not {target!r}")
    mode = _sym(mode)
    mass_solver = _sym(mass_solver)
    flux = _sym(flux)
    if sigma_dirichlet is None:
        sigma_dirichlet = sigma
    coefficients = paper_coefficients() if coefficients is None else coefficients
    source = GaussianSource() if source is None else source
    if mass_solver not in ("cg", "chebyshev"):
        raise ArgumentErrorException(f"unknown mass_solver {mass_solver} (expected :cg or :chebyshev)")
    if initial_profile is not None and mode != "initial_value":
        raise ArgumentErrorException("initial_profile is only available in :initial_value mode")
    if mode not in ("mms", "initial_value", "source"):
        raise ArgumentErrorException(f"unknown mode {mode} (expected :mms, :initial_value or :source)")
    q_u = int(q)
    q_v = q_u - 1 if mixed else q_u
    qu1, qv1 = q_u + 1, q_v + 1
    h = 1.0 / N
    omega = 2 * math.pi * math.sqrt(kx ** 2 + ky ** 2)
    fp = flux_parameters(flux) if flux_params is None else {
        k: float(flux_params[k]) for k in ("theta", "tau", "lambda_u", "lambda_v")}
    bc = boundary_sides(boundary, sigma, sigma_dirichlet, kappa)
    legacy = isinstance(boundary, str) and _sym(boundary) in ("absorbing", "dirichlet")
    gamma_abc = bc["bot"]["gamma_abc"] if legacy else math.nan
    px, py = phase
    C = coefficients
    pi = math.pi
    E = N * N

    # ---- 1D bases at the (q_u+1)-point rule (solver.jl:462-480)
    z, w = GaussQCofs(qu1)
    W2d = _F(np.outer(w, w))
    d_idx = range(qu1)
    P_u = _F(np.stack([JacobiP(z, 0, 0, d) for d in d_idx], axis=1))
    S_u = _F(np.stack([GradJacobiP(z, 0, 0, d) for d in d_idx], axis=1))
    Ebl_u = _F([[JacobiP(-1.0, 0, 0, d) for d in d_idx]])
    Ebr_u = _F([[JacobiP(1.0, 0, 0, d) for d in d_idx]])
    E1bl_u = _F([[GradJacobiP(-1.0, 0, 0, d) for d in d_idx]])
    E1br_u = _F([[GradJacobiP(1.0, 0, 0, d) for d in d_idx]])
    P_v, S_v = _F(P_u[:, :qv1]), _F(S_u[:, :qv1])
    Ebl_v, Ebr_v = _F(Ebl_u[:, :qv1]), _F(Ebr_u[:, :qv1])
    E1bl_v, E1br_v = _F(E1bl_u[:, :qv1]), _F(E1br_u[:, :qv1])

    # ---- high-order rule of the source and the nonlinear mass (solver.jl:482-490)
    q_high = max(int(math.ceil(3 * q_v / 2) + 1), q_u + 1)
    z_h, w_h = GaussQCofs(q_high)
    W2d_h = _F(np.outer(w_h, w_h))
    P_h_v = _F(np.stack([JacobiP(z_h, 0, 0, d) for d in range(qv1)], axis=1))
    Phi2d_h_v = _F(np.kron(P_h_v, P_h_v))
    Phi_xi_u, Phi_eta_u = np.kron(P_u, S_u), np.kron(S_u, P_u)

    cells = np.arange(N)
    xloc = _F((cells[:, None] * h + (cells[:, None] + 1) * h + h * z[None, :]) / 2)
    xloc_h = _F((cells[:, None] * h + (cells[:, None] + 1) * h + h * z_h[None, :]) / 2)
    yloc, yloc_h = xloc.copy(order="F"), xloc_h.copy(order="F")

    # ---- volume data: c²W, αW (point, element, point) and Ainv_u (solver.jl:509-536)
    XQ = np.broadcast_to(xloc[None, :, None, :], (N, N, qu1, qu1))    # [j, k, r, s] = x_s of column k
    YQ = np.broadcast_to(yloc[:, None, :, None], (N, N, qu1, qu1))    # = y_r of row j
    cQ = evaluate(C.c, XQ, YQ)
    aQ = evaluate(C.alpha, XQ, YQ)
    cw4 = cQ ** 2 * W2d                                                 # [j, k, r, s]
    aw4 = aQ * W2d
    # element-major (e = j + N k): [e, r, s]
    cw_e = np.transpose(cw4, (1, 0, 2, 3)).reshape(E, qu1, qu1)
    aw_e = np.transpose(aw4, (1, 0, 2, 3)).reshape(E, qu1, qu1)
    Cw = _F(np.transpose(cw_e, (1, 0, 2)))
    Aw = _F(np.transpose(aw_e, (1, 0, 2)))
    cw_cols = np.transpose(cw_e, (0, 2, 1)).reshape(E, qu1 * qu1)      # vec in column-major (r fastest)
    if inverses not in ("device", "host"):
        raise ArgumentErrorException(f"inverses must be \"device\" or \"host\", not {inverses!r}")
    uniq, inv = _distinct_rows(cw_cols, limit=64 if inverses == "device" else None)
    if inverses == "device" and uniq is None:
        Ainv_u = None                         # computed by the GPU workspace from Cw
    else:
        packed = _packed_inverses(uniq, Phi_xi_u, Phi_eta_u)
        if packed.shape[0] == 1 and E > 1:
            # one matrix for all elements (constant coefficients): a read-only broadcast view
            Ainv_u = np.broadcast_to(packed[0][:, None], (packed.shape[1], E))
        else:
            Ainv_u = _F(packed[inv.reshape(-1)].T)

    # ---- one-sided face values of c, α, β (solver.jl:538-552)
    faces = {s: {} for s in ("bot", "top", "lft", "rgt")}
    for fun, key in ((C.c, "cf"), (C.alpha, "af"), (C.beta, "bf")):
        for s, arr in side_values(fun, xloc, yloc, N, h).items():
            faces[s][key] = arr
    for s in faces:
        faces[s]["c2"] = _F(faces[s]["cf"] ** 2)

    # ---- ∂_e u0 on the sides seen from inside (solver.jl:554-568)
    g0 = {s: np.zeros((N, N, qu1), order="F") for s in ("bot", "top", "lft", "rgt")}
    if mode != "source":
        if initial_profile is None:
            def u0_x(x, y):
                return -2 * pi * kx * np.sin(2 * pi * kx * x + px) * np.sin(2 * pi * ky * y + py)

            def u0_y(x, y):
                return 2 * pi * ky * np.cos(2 * pi * kx * x + px) * np.cos(2 * pi * ky * y + py)
        else:
            u0_x, u0_y = initial_profile["u0_x"], initial_profile["u0_y"]
        g0.update(side_values(u0_y, xloc, yloc, N, h, vertical=False))
        g0.update(side_values(u0_x, xloc, yloc, N, h, horizontal=False))

    # ---- manufactured-solution data at the high-order points (solver.jl:570-602)
    XH = np.broadcast_to(xloc_h[None, :, None, :], (N, N, q_high, q_high))
    YH = np.broadcast_to(yloc_h[:, None, :, None], (N, N, q_high, q_high))
    src_on = mode == "source"
    if src_on:
        pass                                  # source mode: no manufactured-solution data
    elif initial_profile is None:
        sp = np.cos(2 * pi * kx * XH + px) * np.sin(2 * pi * ky * YH + py)
        sp_x = -2 * pi * kx * np.sin(2 * pi * kx * XH + px) * np.sin(2 * pi * ky * YH + py)
        sp_y = 2 * pi * ky * np.cos(2 * pi * kx * XH + px) * np.cos(2 * pi * ky * YH + py)
        sp_xx = -(2 * pi * kx) ** 2 * sp
        sp_yy = -(2 * pi * ky) ** 2 * sp
    else:
        ip = initial_profile
        sp, sp_x, sp_y = (evaluate(ip[n], XH, YH) for n in ("u0", "u0_x", "u0_y"))
        sp_xx, sp_yy = evaluate(ip["u0_xx"], XH, YH), evaluate(ip["u0_yy"], XH, YH)
    mms_BF = _F(evaluate(C.beta, XH, YH))
    if src_on:
        mms_SP = mms_Cdiv = mms_Ddiv = np.zeros((N, N, q_high, q_high), order="F")
    else:
        cf = evaluate(C.c, XH, YH)
        c2 = cf ** 2
        c2x, c2y = 2 * cf * evaluate(C.c_x, XH, YH), 2 * cf * evaluate(C.c_y, XH, YH)
        af = evaluate(C.alpha, XH, YH)
        ax, ay = evaluate(C.alpha_x, XH, YH), evaluate(C.alpha_y, XH, YH)
        mms_SP = _F(sp)
        mms_Cdiv = _F(c2x * sp_x + c2y * sp_y + c2 * (sp_xx + sp_yy))
        mms_Ddiv = _F(ax * sp_x + ay * sp_y + af * (sp_xx + sp_yy))

    # ---- Φ and ∇Φ on the physical boundary (solver.jl:604-635), as (N, nq)
    bcd = {}
    zx = np.zeros_like(xloc)
    if src_on:
        for n in ("bc_bot_sp", "bc_bot_spy", "bc_top_sp", "bc_top_spy",
                  "bc_lft_sp", "bc_lft_spx", "bc_rgt_sp", "bc_rgt_spx"):
            bcd[n] = np.zeros((N, qu1), order="F")
    elif initial_profile is None:
        cx = np.cos(2 * pi * kx * xloc + px)
        sy = np.sin(2 * pi * ky * yloc + py)
        bcd["bc_bot_sp"] = _F(cx * math.sin(2 * pi * ky * 0 + py))
        bcd["bc_bot_spy"] = _F(2 * pi * ky * cx * math.cos(2 * pi * ky * 0 + py))
        bcd["bc_top_sp"] = _F(cx * math.sin(2 * pi * ky * 1 + py))
        bcd["bc_top_spy"] = _F(2 * pi * ky * cx * math.cos(2 * pi * ky * 1 + py))
        bcd["bc_lft_sp"] = _F(math.cos(2 * pi * kx * 0 + px) * sy)
        bcd["bc_lft_spx"] = _F(-2 * pi * kx * math.sin(2 * pi * kx * 0 + px) * sy)
        bcd["bc_rgt_sp"] = _F(math.cos(2 * pi * kx * 1 + px) * sy)
        bcd["bc_rgt_spx"] = _F(-2 * pi * kx * math.sin(2 * pi * kx * 1 + px) * sy)
    else:
        ip = initial_profile
        bcd["bc_bot_sp"] = _F(evaluate(ip["u0"], xloc, zx))
        bcd["bc_bot_spy"] = _F(evaluate(ip["u0_y"], xloc, zx))
        bcd["bc_top_sp"] = _F(evaluate(ip["u0"], xloc, zx + 1.0))
        bcd["bc_top_spy"] = _F(evaluate(ip["u0_y"], xloc, zx + 1.0))
        bcd["bc_lft_sp"] = _F(evaluate(ip["u0"], zx, yloc))
        bcd["bc_lft_spx"] = _F(evaluate(ip["u0_x"], zx, yloc))
        bcd["bc_rgt_sp"] = _F(evaluate(ip["u0"], zx + 1.0, yloc))
        bcd["bc_rgt_spx"] = _F(evaluate(ip["u0_x"], zx + 1.0, yloc))

    err_c2 = _F(cQ ** 2)
    err_beta = _F(evaluate(C.beta, XQ, YQ))

    # ---- source projection (solver.jl:647-662)
    src_proj = np.zeros((N, N, qv1, qv1), order="F")
    if src_on:
        g = source.amplitude * np.exp(-((XH - source.x0[0]) ** 2 + (YH - source.x0[1]) ** 2) / source.r0 ** 2)
        src_proj = _F(np.einsum("ra,jkrs,sb->jkab", P_h_v, W2d_h * g, P_h_v, optimize=True))

    pre = dict(
        N=N, qu1=qu1, qv1=qv1, q_high=q_high, omega=omega, w=w,
        P_u=P_u, P_v=P_v, S_u=S_u, S_v=S_v,
        Ebl_u=Ebl_u, Ebr_u=Ebr_u, E1bl_u=E1bl_u, E1br_u=E1br_u,
        Ebl_v=Ebl_v, Ebr_v=Ebr_v, E1bl_v=E1bl_v, E1br_v=E1br_v,
        W2d_h=W2d_h, P_h_v=P_h_v, Phi2d_h_v=Phi2d_h_v,
        Cw=Cw, Aw=Aw, Ainv_u=Ainv_u,
        mms_SP=mms_SP, mms_Cdiv=mms_Cdiv, mms_Ddiv=mms_Ddiv, mms_BF=mms_BF,
        theta=fp["theta"], tau=fp["tau"], lambda_u=fp["lambda_u"], lambda_v=fp["lambda_v"],
        gamma_abc=gamma_abc, eta_abc=math.sqrt(1.0 - gamma_abc ** 2) if legacy else math.nan,
        sigma=bc["bot"]["sigma"] if legacy else math.nan,
        bc=bc, src_on=src_on, src_proj=src_proj, source=source,
        mms_on=mode == "mms", mass_solver=mass_solver,
    )
    pre.update(bcd)
    for s in ("bot", "top", "lft", "rgt"):
        for key in ("c2", "af", "cf", "bf"):
            pre[f"{s}_{key}"] = faces[s][key]
        pre[f"{s}_g0"] = g0[s]
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
    """Face arrays by face, interface jumps, projections and transposes (src/solver.jl:716-770)."""
    nq, nv, qh = pre["qu1"], pre["qv1"], pre["q_high"]
    E = N * N

    def hface(bot, top):       # (nq, N+1, N): rows 0..N-1 from bot, row N from the top of row N-1
        A = np.empty((nq, N + 1, N), order="F")
        A[:, :N, :] = np.transpose(bot, (2, 0, 1))
        A[:, N, :] = top[N - 1].T
        return A

    def vface(lft, rgt):       # (nq, N, N+1)
        A = np.empty((nq, N, N + 1), order="F")
        A[:, :, :N] = np.transpose(lft, (2, 0, 1))
        A[:, :, N] = rgt[:, N - 1, :].T
        return A

    def hfaceM(bot, top):
        A = np.empty((nq, N + 1, N), order="F")
        A[:, 0, :] = bot[0].T
        A[:, 1:, :] = np.transpose(top, (2, 0, 1))
        return A

    def vfaceM(lft, rgt):
        A = np.empty((nq, N, N + 1), order="F")
        A[:, :, 0] = lft[:, 0, :].T
        A[:, :, 1:] = np.transpose(rgt, (2, 0, 1))
        return A

    Ph, Wh = pre["P_h_v"], pre["W2d_h"]

    def proj(X):               # (N, N, qh, qh) -> (nv, nv, N, N)
        return _F(np.einsum("ra,jkrs,sb->abjk", Ph, Wh * X, Ph, optimize=True))

    def elast(X):
        return _F(np.transpose(X, (2, 3, 0, 1)))

    p = pre
    hc2, hc2m = hface(p["bot_c2"], p["top_c2"]), hfaceM(p["bot_c2"], p["top_c2"])
    haf, hafm = hface(p["bot_af"], p["top_af"]), hfaceM(p["bot_af"], p["top_af"])
    vc2, vc2m = vface(p["lft_c2"], p["rgt_c2"]), vfaceM(p["lft_c2"], p["rgt_c2"])
    vaf, vafm = vface(p["lft_af"], p["rgt_af"]), vfaceM(p["lft_af"], p["rgt_af"])
    hg0, hg0m = hface(p["bot_g0"], p["top_g0"]), hfaceM(p["bot_g0"], p["top_g0"])
    vg0, vg0m = vface(p["lft_g0"], p["rgt_g0"]), vfaceM(p["lft_g0"], p["rgt_g0"])
    jumps = not (np.array_equal(hc2m, hc2) and np.array_equal(hafm, haf)
                 and np.array_equal(vc2m, vc2) and np.array_equal(vafm, vaf))
    if p["mms_on"] and jumps:
        raise ArgumentErrorException("mode = :mms needs c and α continuous across the element faces; "
                         "use :initial_value or :source for coefficients that jump")
    hJC = _F(hc2m * hg0m - hc2 * hg0)
    vJC = _F(vc2m * vg0m - vc2 * vg0)
    hJC[:, 0, :] = 0.0
    hJC[:, N, :] = 0.0
    vJC[:, :, 0] = 0.0
    vJC[:, :, N] = 0.0
    one_sided = jumps or bool(np.any(hJC != 0)) or bool(np.any(vJC != 0))
    beta_hE = elast(p["mms_BF"])
    zero_proj = np.zeros((nv, nv, N, N), order="F")
    src = p["src_on"]
    return dict(
        hc2=hc2, haf=haf, hcf=hface(p["bot_cf"], p["top_cf"]), hbf=hface(p["bot_bf"], p["top_bf"]),
        vc2=vc2, vaf=vaf, vcf=vface(p["lft_cf"], p["rgt_cf"]), vbf=vface(p["lft_bf"], p["rgt_bf"]),
        hc2m=hc2m, hafm=hafm, vc2m=vc2m, vafm=vafm, hJC=hJC, vJC=vJC, one_sided=one_sided,
        bcB_sp=_F(p["bc_bot_sp"].T), bcB_spy=_F(p["bc_bot_spy"].T),
        bcT_sp=_F(p["bc_top_sp"].T), bcT_spy=_F(p["bc_top_spy"].T),
        bcL_sp=_F(p["bc_lft_sp"].T), bcL_spx=_F(p["bc_lft_spx"].T),
        bcR_sp=_F(p["bc_rgt_sp"].T), bcR_spx=_F(p["bc_rgt_spx"].T),
        PiSP=zero_proj if src else proj(p["mms_SP"]),
        PiBSP2=zero_proj if src else proj(p["mms_BF"] * p["mms_SP"] ** 2),
        PiCdiv=zero_proj if src else proj(p["mms_Cdiv"]),
        PiDdiv=zero_proj if src else proj(p["mms_Ddiv"]),
        src_projE=elast(p["src_proj"]), beta_hE=beta_hE,
        beta_hq=_F(np.transpose(beta_hE.reshape(qh, qh, E, order="F"), (0, 2, 1))),
        W_hq=_F(p["W2d_h"].reshape(qh, 1, qh, order="F")),
        P_h_vT=_F(p["P_h_v"].T), mass_tol=1e-14,
    )


def _face_values(f, xloc, yloc, N, h, horizontal=True, vertical=True):
    """The point values of one family on the faces that side_values reads (src/solver.jl:371-392):
    per orientation, the value at each face point and δ below (left of) and above (right of) it,
    the reference's arrays (nq, N+1, N) and (nq, N, N+1) (the δ values outside the domain are the
    face values, as there), and the family's tolerance term s."""
    nq = xloc.shape[1]
    d = FACE_SHIFT
    out, sh, sv = {}, 0.0, 0.0

    def fortran(a):   # the reference's column-major layout of an (nq, ., .) array evaluated in C order
        return np.asfortranarray(a)
    if horizontal:
        X = np.broadcast_to(xloc.T[:, None, :], (nq, N + 1, N))
        Yf = np.broadcast_to((np.arange(N + 1) * h)[None, :, None], (nq, N + 1, N))
        H0 = fortran(evaluate(f, X, Yf))
        HM, HP = H0.copy(order="F"), H0.copy(order="F")
        HM[:, 1:, :] = evaluate(f, X[:, 1:, :], Yf[:, 1:, :] - d)
        HP[:, :N, :] = evaluate(f, X[:, :N, :], Yf[:, :N, :] + d)
        out["h"] = (H0, HM, HP)
        sh = max(_amax(HM[:, 1:, :]), _amax(HP[:, :N, :]))
    if vertical:
        Xf = np.broadcast_to((np.arange(N + 1) * h)[None, None, :], (nq, N, N + 1))
        Y = np.broadcast_to(yloc.T[:, :, None], (nq, N, N + 1))
        V0 = fortran(evaluate(f, Xf, Y))
        VM, VP = V0.copy(order="F"), V0.copy(order="F")
        VM[:, :, 1:] = evaluate(f, Xf[:, :, 1:] - d, Y[:, :, 1:])
        VP[:, :, :N] = evaluate(f, Xf[:, :, :N] + d, Y[:, :, :N])
        out["v"] = (V0, VM, VP)
        sv = max(_amax(VM[:, :, 1:]), _amax(VP[:, :, :N]))
    return out, JUMP_TOL * max(sh, sv)


def precompute_points(q, N, *, mixed=True, flux="upwind", flux_params=None, sigma=0.0, boundary="absorbing_2beta",
                      sigma_dirichlet=None, kappa=0.0, phase=(0.0, 0.0), coefficients=None, mode="mms", kx=1, ky=1,
                      source=None, mass_solver="chebyshev", initial_profile=None):
    """``precompute`` for a workspace that builds ``pre``'s large arrays on the device
    (wedg_create_points): the 1D operators, scalars and boundary data of ``pre`` (src/solver.jl:
    428-490, 604-635, 665-690), and the values of the coefficient functions and data at the point
    grids, evaluated here (they are the caller's functions) in the memory order the device reads.
    The element matrices, one-sided face arrays, jump terms, projections and 2β are formed on the
    device from these values (precompute forms them on the host). Returns (pre, geo) like
    precompute; pre["points"] holds the point values, and pre has no element or face arrays."""
    mode = _sym(mode)
    mass_solver = _sym(mass_solver)
    if sigma_dirichlet is None:
        sigma_dirichlet = sigma
    coefficients = paper_coefficients() if coefficients is None else coefficients
    source = GaussianSource() if source is None else source
    if mass_solver not in ("cg", "chebyshev"):
        raise ArgumentErrorException(f"unknown mass_solver {mass_solver} (expected :cg or :chebyshev)")
    if initial_profile is not None and mode != "initial_value":
        raise ArgumentErrorException("initial_profile is only available in :initial_value mode")
    if mode not in ("mms", "initial_value", "source"):
        raise ArgumentErrorException(f"unknown mode {mode} (expected :mms, :initial_value or :source)")
    q_u = int(q)
    q_v = q_u - 1 if mixed else q_u
    qu1, qv1 = q_u + 1, q_v + 1
    h = 1.0 / N
    omega = 2 * math.pi * math.sqrt(kx ** 2 + ky ** 2)
    fp = flux_parameters(_sym(flux)) if flux_params is None else {
        k: float(flux_params[k]) for k in ("theta", "tau", "lambda_u", "lambda_v")}
    bc = boundary_sides(boundary, sigma, sigma_dirichlet, kappa)
    legacy = isinstance(boundary, str) and _sym(boundary) in ("absorbing", "dirichlet")
    gamma_abc = bc["bot"]["gamma_abc"] if legacy else math.nan
    px, py = phase
    C = coefficients
    pi = math.pi

    # ---- 1D bases (solver.jl:462-490), as precompute
    z, w = GaussQCofs(qu1)
    W2d = _F(np.outer(w, w))
    d_idx = range(qu1)
    P_u = _F(np.stack([JacobiP(z, 0, 0, d) for d in d_idx], axis=1))
    S_u = _F(np.stack([GradJacobiP(z, 0, 0, d) for d in d_idx], axis=1))
    Ebl_u = _F([[JacobiP(-1.0, 0, 0, d) for d in d_idx]])
    Ebr_u = _F([[JacobiP(1.0, 0, 0, d) for d in d_idx]])
    E1bl_u = _F([[GradJacobiP(-1.0, 0, 0, d) for d in d_idx]])
    E1br_u = _F([[GradJacobiP(1.0, 0, 0, d) for d in d_idx]])
    q_high = max(int(math.ceil(3 * q_v / 2) + 1), q_u + 1)
    z_h, w_h = GaussQCofs(q_high)
    W2d_h = _F(np.outer(w_h, w_h))
    P_h_v = _F(np.stack([JacobiP(z_h, 0, 0, d) for d in range(qv1)], axis=1))
    cells = np.arange(N)
    xloc = _F((cells[:, None] * h + (cells[:, None] + 1) * h + h * z[None, :]) / 2)
    xloc_h = _F((cells[:, None] * h + (cells[:, None] + 1) * h + h * z_h[None, :]) / 2)
    yloc, yloc_h = xloc.copy(order="F"), xloc_h.copy(order="F")

    # ---- point values in the device's order: an (N, N, n, n) array [j, k, r, s] with j fastest is
    #      the transpose of a C-order (n_s, n_r, N_k, N_j) array, so evaluate on that grid directly
    def grid(xl, yl):
        n = xl.shape[1]
        X = np.broadcast_to(xl.T[:, None, :, None], (n, n, N, N))     # [s, r, k, j] = x_s of column k
        Y = np.broadcast_to(yl.T[None, :, None, :], (n, n, N, N))     # = y_r of row j
        return X, Y

    def at(f, XY):
        return np.ascontiguousarray(evaluate(f, *XY)).T                # (N, N, n, n), Fortran-contiguous
    XQ, XH = grid(xloc, yloc), grid(xloc_h, yloc_h)

    # a constant coefficient (constant_coefficients, replace_coefficients) is passed as its value and
    # a table of cells (cell_coefficients) as the table: the device evaluates both at every point
    def field(f, XY):
        if isinstance(f, _Const):
            return dict(value=f.val)
        if isinstance(f, _Cells):
            return dict(table=f.tab)
        return dict(array=at(f, XY))

    def face(f):
        if isinstance(f, (_Const, _Cells)):
            return None
        return _face_values(f, xloc, yloc, N, h)
    pts = dict(c_q=field(C.c, XQ), alpha_q=field(C.alpha, XQ), beta_h=field(C.beta, XH),
               faces={key: face(fun) for key, fun in (("c", C.c), ("a", C.alpha), ("b", C.beta))})
    src_on = mode == "source"
    g0 = None
    if not src_on:
        if initial_profile is None:
            def u0_x(x, y):
                return -2 * pi * kx * np.sin(2 * pi * kx * x + px) * np.sin(2 * pi * ky * y + py)

            def u0_y(x, y):
                return 2 * pi * ky * np.cos(2 * pi * kx * x + px) * np.cos(2 * pi * ky * y + py)
        else:
            u0_x, u0_y = initial_profile["u0_x"], initial_profile["u0_y"]
        gy, sy = _face_values(u0_y, xloc, yloc, N, h, vertical=False)
        gx, sx = _face_values(u0_x, xloc, yloc, N, h, horizontal=False)
        g0 = dict(h=(gy["h"], sy), v=(gx["v"], sx))
        # data at the high-order points (solver.jl:570-602)
        XHa, YHa = XH
        if initial_profile is None:
            sp = np.cos(2 * pi * kx * XHa + px) * np.sin(2 * pi * ky * YHa + py)
            sp_x = -2 * pi * kx * np.sin(2 * pi * kx * XHa + px) * np.sin(2 * pi * ky * YHa + py)
            sp_y = 2 * pi * ky * np.cos(2 * pi * kx * XHa + px) * np.cos(2 * pi * ky * YHa + py)
            sp_xx = -(2 * pi * kx) ** 2 * sp
            sp_yy = -(2 * pi * ky) ** 2 * sp
        else:
            ip = initial_profile
            sp, sp_x, sp_y = (evaluate(ip[n], XHa, YHa) for n in ("u0", "u0_x", "u0_y"))
            sp_xx, sp_yy = evaluate(ip["u0_xx"], XHa, YHa), evaluate(ip["u0_yy"], XHa, YHa)
        cf = evaluate(C.c, XHa, YHa)
        c2 = cf ** 2
        c2x, c2y = 2 * cf * evaluate(C.c_x, XHa, YHa), 2 * cf * evaluate(C.c_y, XHa, YHa)
        pts["cdiv_h"] = np.ascontiguousarray(c2x * sp_x + c2y * sp_y + c2 * (sp_xx + sp_yy)).T
        if mode == "mms":
            af = evaluate(C.alpha, XHa, YHa)
            ax, ay = evaluate(C.alpha_x, XHa, YHa), evaluate(C.alpha_y, XHa, YHa)
            pts["sp_h"] = np.ascontiguousarray(sp).T
            pts["ddiv_h"] = np.ascontiguousarray(ax * sp_x + ay * sp_y + af * (sp_xx + sp_yy)).T
    pts["g0"] = g0

    # ---- Φ and ∇Φ on the physical boundary (solver.jl:604-635), (nq, N) as _rhs_data lays them out
    bcd = {}
    zx = np.zeros_like(xloc)
    if src_on:
        for n in ("bc_bot_sp", "bc_bot_spy", "bc_top_sp", "bc_top_spy",
                  "bc_lft_sp", "bc_lft_spx", "bc_rgt_sp", "bc_rgt_spx"):
            bcd[n] = np.zeros((N, qu1), order="F")
    elif initial_profile is None:
        cx = np.cos(2 * pi * kx * xloc + px)
        sy_ = np.sin(2 * pi * ky * yloc + py)
        bcd["bc_bot_sp"] = cx * math.sin(2 * pi * ky * 0 + py)
        bcd["bc_bot_spy"] = 2 * pi * ky * cx * math.cos(2 * pi * ky * 0 + py)
        bcd["bc_top_sp"] = cx * math.sin(2 * pi * ky * 1 + py)
        bcd["bc_top_spy"] = 2 * pi * ky * cx * math.cos(2 * pi * ky * 1 + py)
        bcd["bc_lft_sp"] = math.cos(2 * pi * kx * 0 + px) * sy_
        bcd["bc_lft_spx"] = -2 * pi * kx * math.sin(2 * pi * kx * 0 + px) * sy_
        bcd["bc_rgt_sp"] = math.cos(2 * pi * kx * 1 + px) * sy_
        bcd["bc_rgt_spx"] = -2 * pi * kx * math.sin(2 * pi * kx * 1 + px) * sy_
    else:
        ip = initial_profile
        bcd["bc_bot_sp"] = evaluate(ip["u0"], xloc, zx)
        bcd["bc_bot_spy"] = evaluate(ip["u0_y"], xloc, zx)
        bcd["bc_top_sp"] = evaluate(ip["u0"], xloc, zx + 1.0)
        bcd["bc_top_spy"] = evaluate(ip["u0_y"], xloc, zx + 1.0)
        bcd["bc_lft_sp"] = evaluate(ip["u0"], zx, yloc)
        bcd["bc_lft_spx"] = evaluate(ip["u0_x"], zx, yloc)
        bcd["bc_rgt_sp"] = evaluate(ip["u0"], zx + 1.0, yloc)
        bcd["bc_rgt_spx"] = evaluate(ip["u0_x"], zx + 1.0, yloc)
    names = dict(bcB_sp="bc_bot_sp", bcB_spy="bc_bot_spy", bcT_sp="bc_top_sp", bcT_spy="bc_top_spy",
                 bcL_sp="bc_lft_sp", bcL_spx="bc_lft_spx", bcR_sp="bc_rgt_sp", bcR_spx="bc_rgt_spx")
    pts["source"] = dict(amp=float(source.amplitude), x0=float(source.x0[0]), y0=float(source.x0[1]),
                         r0=float(source.r0))
    pts["grid"] = dict(xloc=xloc, yloc=yloc, xloc_h=xloc_h, yloc_h=yloc_h)

    pre = dict(
        N=N, qu1=qu1, qv1=qv1, q_high=q_high, omega=omega, w=w,
        P_u=P_u, P_v=_F(P_u[:, :qv1]), S_u=S_u, S_v=_F(S_u[:, :qv1]),
        Ebl_u=Ebl_u, Ebr_u=Ebr_u, E1bl_u=E1bl_u, E1br_u=E1br_u,
        W2d_h=W2d_h, P_h_v=P_h_v,
        theta=fp["theta"], tau=fp["tau"], lambda_u=fp["lambda_u"], lambda_v=fp["lambda_v"],
        gamma_abc=gamma_abc, eta_abc=math.sqrt(1.0 - gamma_abc ** 2) if legacy else math.nan,
        sigma=bc["bot"]["sigma"] if legacy else math.nan,
        bc=bc, src_on=src_on, source=source, mms_on=mode == "mms", mass_solver=mass_solver, mass_tol=1e-14,
        points=pts,
    )
    for k, n in names.items():
        pre[k] = _F(np.asarray(bcd[n]).T)
    lazy = dict(err_c2=lambda: at(C.c, XQ) ** 2, err_beta=lambda: at(C.beta, XQ))
    geo = _LazyGeo(lazy, S_u=S_u, W2d=W2d, xloc=xloc, yloc=yloc)
    return pre, geo


class _LazyGeo(dict):
    """geo of precompute_points: c² and β at the u-points (err_c2, err_beta, only used by the error
    norms and the source-mode diagnostics) are evaluated on first use."""

    def __init__(self, lazy, **kw):
        super().__init__(**kw)
        self._lazy = lazy

    def __missing__(self, key):
        if key not in self._lazy:
            raise KeyError(key)
        self[key] = val = self._lazy[key]()
        return val
