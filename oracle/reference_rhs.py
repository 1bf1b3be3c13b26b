"""Dense element-by-element RHS of WesterveltEDG.jl v0.1.0 (oracle).

Test infrastructure only. Restates ``test/reference_rhs.jl`` (the reference's
own second implementation, with dense volume operators, a Cholesky u-solve
and an LU mass solve) and the adaptors ``dense_volume`` /
``reference_pre`` of ``test/runtests.jl:11-20, 233-239``. It is independent of
``rhs_oracle.c`` in order of operations and in its mass solve, and is used to
pin the C oracle the way the reference pins src/rhs.jl
(``test/runtests.jl:189-293``).
"""
import numpy as np
from scipy.linalg import cho_factor, cho_solve, lu_factor, lu_solve

from .precompute import src_time


def dense_volume(pre):
    """test/runtests.jl:11-20: dense c²- and α-stiffness blocks and the pinned u-stiffness."""
    N = pre["N"]
    P_u, S_u, P_v, S_v = pre["P_u"], pre["S_u"], pre["P_v"], pre["S_v"]
    Pxu, Peu = np.kron(P_u, S_u), np.kron(S_u, P_u)
    Pxv, Pev = np.kron(P_v, S_v), np.kron(S_v, P_v)
    Mc2, Ma, Rut = {}, {}, {}
    for k in range(N):
        for j in range(N):
            e = j + k * N
            cw = pre["Cw"][:, e, :].reshape(-1, order="F")
            aw = pre["Aw"][:, e, :].reshape(-1, order="F")
            K = Pxu.T @ (cw[:, None] * Pxu) + Peu.T @ (cw[:, None] * Peu)
            K[0, 0] += 1.0
            Mc2[j, k] = Pxv.T @ (cw[:, None] * Pxu) + Pev.T @ (cw[:, None] * Peu)
            Ma[j, k] = Pxv.T @ (aw[:, None] * Pxv) + Pev.T @ (aw[:, None] * Pev)
            Rut[j, k] = cho_factor(K)
    out = dict(pre)
    out.update(Mc2_uv=Mc2, Ma_vv=Ma, R_ut=Rut)
    return out


def reference_pre(pre):
    """test/runtests.jl:233-239: a uniform boundary kind as the legacy (γ, η, σ, k) family."""
    b = pre["bc"]["bot"]
    if b["kind"] == "wall":
        g, e, s, k = 0.0, 1.0, -b["kappa"], 0.0
    else:
        g, e, s, k = b["gamma_abc"], b["eta_abc"], b["sigma"], b["kb"]
    out = dict(pre)
    out.update(gamma_abc=g, eta_abc=e, sigma=s)
    for side in ("bot", "top", "lft", "rgt"):
        out[f"{side}_bf"] = k * pre[f"{side}_bf"]
    return out


def _abc_face_reference(pre, c2f, af, cf, bf, v_fp, gun, gvn, gu_ex, gv_ex, v_ex):
    """test/reference_rhs.jl:33-46."""
    g, e, s = pre["gamma_abc"], pre["eta_abc"], pre["sigma"]
    rho_num = e * (c2f * gun + af * gvn) + g * cf * np.sqrt(1.0 - bf * v_fp) * v_fp
    rho_ex = e * (c2f * gu_ex + af * gv_ex) + g * cf * np.sqrt(1.0 - bf * v_ex) * v_ex
    rho = rho_num - rho_ex
    sqf = np.sqrt(1.0 - bf * v_fp)
    F1 = c2f * gun + af * gvn - (e + s * g) * rho
    dv = -(g - s * e) / (cf * sqf) * rho
    return F1, dv


def edg_rhs_reference(u, v, t, N, h, pre):
    """test/reference_rhs.jl:48-352, with pre = dense_volume(reference_pre(precompute(...)))."""
    qu1, qv1, om = pre["qu1"], pre["qv1"], pre["omega"]
    w = pre["w"]
    P_u, P_v = pre["P_u"], pre["P_v"]
    Ebl_u, Ebr_u, E1bl_u, E1br_u = (pre[n][0] for n in ("Ebl_u", "Ebr_u", "E1bl_u", "E1br_u"))
    Ebl_v, Ebr_v, E1bl_v, E1br_v = (pre[n][0] for n in ("Ebl_v", "Ebr_v", "E1bl_v", "E1br_v"))
    W2d_h, P_h_v, Phi2d_h_v = pre["W2d_h"], pre["P_h_v"], pre["Phi2d_h_v"]
    th, tau, lu, lv = pre["theta"], pre["tau"], pre["lambda_u"], pre["lambda_v"]
    two_h, four_hh = 2.0 / h, 4.0 / (h * h)
    ct = np.cos(om * t) if pre["mms_on"] else 0.0
    st = np.sin(om * t) if pre["mms_on"] else 0.0

    def pen_w(c2m, c2p, afm, afp):
        return 0.5 * (c2m + c2p) * lu + 0.5 * (afm + afp) * lv

    def lift(E, Pm, vals):       # E' * (P' * (w .* vals))'  -> outer product E[a] Y[b]
        return np.outer(E, Pm.T @ (w * vals))

    ut = np.zeros(u.shape, order="F")
    vt = np.zeros(v.shape, order="F")
    vt_rhs_all = np.zeros((N, N, qv1, qv1))
    for j in range(N):
        for k in range(N):
            U = u[j, k]
            V = v[j, k]
            vt_rhs = -four_hh * (pre["Mc2_uv"][j, k] @ U.reshape(-1, order="F")
                                 + pre["Ma_vv"][j, k] @ V.reshape(-1, order="F")).reshape(qv1, qv1, order="F")
            SP, Cdiv, Ddiv, BF = (pre[n][j, k] for n in ("mms_SP", "mms_Cdiv", "mms_Ddiv", "mms_BF"))
            v_h_mms = -om * st * SP
            vt_h_mms = -om ** 2 * ct * SP
            fv_h = (1.0 - 2.0 * BF * v_h_mms) * vt_h_mms - ct * Cdiv + om * st * Ddiv + Cdiv
            vt_rhs = vt_rhs + P_h_v.T @ (W2d_h * fv_h) @ P_h_v
            if pre["src_on"]:
                vt_rhs = vt_rhs + src_time(pre, t) * pre["src_proj"][j, k]
            f = np.zeros((qu1, qu1))

            # bottom face, n = (0, -1)
            if j == 0:
                c2f, af, cf, bf = (pre[f"bot_{n}"][j, k] for n in ("c2", "af", "cf", "bf"))
                v_fp = P_v @ (Ebl_v @ V)
                gun = -(P_u @ (two_h * (E1bl_u @ U)))
                gvn = -(P_v @ (two_h * (E1bl_v @ V)))
                sp, spy = pre["bc_bot_sp"][k], pre["bc_bot_spy"][k]
                F1, dv = _abc_face_reference(pre, c2f, af, cf, bf, v_fp, gun, gvn,
                                             -ct * spy + spy, om * st * spy, -om * st * sp)
                vt_rhs = vt_rhs + two_h * lift(Ebl_v, P_v, F1) - four_hh * lift(E1bl_v, P_v, af * dv)
                f = f + lift(E1bl_u, P_u, c2f * dv)
            else:
                Uo, Vo = u[j - 1, k], v[j - 1, k]
                c2p, afp = pre["bot_c2"][j, k], pre["bot_af"][j, k]
                c2m, afm = pre["top_c2"][j - 1, k], pre["top_af"][j - 1, k]
                K = c2m * pre["top_g0"][j - 1, k] - c2p * pre["bot_g0"][j, k]
                vj = P_v @ (Ebr_v @ Vo - Ebl_v @ V)
                gu_m, gu_p = P_u @ (E1br_u @ Uo), P_u @ (E1bl_u @ U)
                gv_m, gv_p = P_v @ (E1br_v @ Vo), P_v @ (E1bl_v @ V)
                jw = two_h * (c2m * gu_m - c2p * gu_p + afm * gv_m - afp * gv_p) + K
                flux_p = th * (c2p * gu_p + afp * gv_p) + (1 - th) * (c2m * gu_m + afm * gv_m)
                dv_p = th * vj - tau * jw
                pen_p = pen_w(c2m, c2p, afm, afp) * vj - (1 - th) * K
                f = f + lift(E1bl_u, P_u, c2p * dv_p)
                vt_rhs = (vt_rhs - four_hh * lift(Ebl_v, P_v, flux_p) - four_hh * lift(E1bl_v, P_v, afp * dv_p)
                          + two_h * lift(Ebl_v, P_v, pen_p))

            # top face, n = (0, +1)
            if j == N - 1:
                c2f, af, cf, bf = (pre[f"top_{n}"][j, k] for n in ("c2", "af", "cf", "bf"))
                v_fp = P_v @ (Ebr_v @ V)
                gun = P_u @ (two_h * (E1br_u @ U))
                gvn = P_v @ (two_h * (E1br_v @ V))
                sp, spy = pre["bc_top_sp"][k], pre["bc_top_spy"][k]
                F1, dv = _abc_face_reference(pre, c2f, af, cf, bf, v_fp, gun, gvn,
                                             ct * spy - spy, -om * st * spy, -om * st * sp)
                vt_rhs = vt_rhs + two_h * lift(Ebr_v, P_v, F1) + four_hh * lift(E1br_v, P_v, af * dv)
                f = f - lift(E1br_u, P_u, c2f * dv)
            else:
                Uo, Vo = u[j + 1, k], v[j + 1, k]
                c2m, afm = pre["top_c2"][j, k], pre["top_af"][j, k]
                c2p, afp = pre["bot_c2"][j + 1, k], pre["bot_af"][j + 1, k]
                K = c2m * pre["top_g0"][j, k] - c2p * pre["bot_g0"][j + 1, k]
                vj = P_v @ (Ebl_v @ Vo - Ebr_v @ V)
                gu_m, gu_p = P_u @ (E1br_u @ U), P_u @ (E1bl_u @ Uo)
                gv_m, gv_p = P_v @ (E1br_v @ V), P_v @ (E1bl_v @ Vo)
                jw = two_h * (c2m * gu_m - c2p * gu_p + afm * gv_m - afp * gv_p) + K
                flux_p = (1 - th) * (c2m * gu_m + afm * gv_m) + th * (c2p * gu_p + afp * gv_p)
                dv_p = (1 - th) * vj - tau * jw
                pen_p = pen_w(c2m, c2p, afm, afp) * vj - th * K
                f = f - lift(E1br_u, P_u, c2m * dv_p)
                vt_rhs = (vt_rhs + four_hh * lift(Ebr_v, P_v, flux_p) + four_hh * lift(E1br_v, P_v, afm * dv_p)
                          + two_h * lift(Ebr_v, P_v, pen_p))

            # left face, n = (-1, 0): the y-face pattern on transposes
            if k == 0:
                c2f, af, cf, bf = (pre[f"lft_{n}"][j, k] for n in ("c2", "af", "cf", "bf"))
                v_fp = P_v @ (Ebl_v @ V.T)
                gun = -(P_u @ (two_h * (E1bl_u @ U.T)))
                gvn = -(P_v @ (two_h * (E1bl_v @ V.T)))
                sp, spx = pre["bc_lft_sp"][j], pre["bc_lft_spx"][j]
                F1, dv = _abc_face_reference(pre, c2f, af, cf, bf, v_fp, gun, gvn,
                                             -ct * spx + spx, om * st * spx, -om * st * sp)
                vt_rhs = vt_rhs + (two_h * lift(Ebl_v, P_v, F1) - four_hh * lift(E1bl_v, P_v, af * dv)).T
                f = f + lift(E1bl_u, P_u, c2f * dv).T
            else:
                Uo, Vo = u[j, k - 1].T, v[j, k - 1].T
                c2p, afp = pre["lft_c2"][j, k], pre["lft_af"][j, k]
                c2m, afm = pre["rgt_c2"][j, k - 1], pre["rgt_af"][j, k - 1]
                K = c2m * pre["rgt_g0"][j, k - 1] - c2p * pre["lft_g0"][j, k]
                vj = P_v @ (Ebr_v @ Vo - Ebl_v @ V.T)
                gu_m, gu_p = P_u @ (E1br_u @ Uo), P_u @ (E1bl_u @ U.T)
                gv_m, gv_p = P_v @ (E1br_v @ Vo), P_v @ (E1bl_v @ V.T)
                jw = two_h * (c2m * gu_m - c2p * gu_p + afm * gv_m - afp * gv_p) + K
                flux_p = th * (c2p * gu_p + afp * gv_p) + (1 - th) * (c2m * gu_m + afm * gv_m)
                dv_p = th * vj - tau * jw
                pen_p = pen_w(c2m, c2p, afm, afp) * vj - (1 - th) * K
                f = f + lift(E1bl_u, P_u, c2p * dv_p).T
                vt_rhs = (vt_rhs - four_hh * lift(Ebl_v, P_v, flux_p).T - four_hh * lift(E1bl_v, P_v, afp * dv_p).T
                          + two_h * lift(Ebl_v, P_v, pen_p).T)

            # right face, n = (+1, 0)
            if k == N - 1:
                c2f, af, cf, bf = (pre[f"rgt_{n}"][j, k] for n in ("c2", "af", "cf", "bf"))
                v_fp = P_v @ (Ebr_v @ V.T)
                gun = P_u @ (two_h * (E1br_u @ U.T))
                gvn = P_v @ (two_h * (E1br_v @ V.T))
                sp, spx = pre["bc_rgt_sp"][j], pre["bc_rgt_spx"][j]
                F1, dv = _abc_face_reference(pre, c2f, af, cf, bf, v_fp, gun, gvn,
                                             ct * spx - spx, -om * st * spx, -om * st * sp)
                vt_rhs = vt_rhs + (two_h * lift(Ebr_v, P_v, F1) + four_hh * lift(E1br_v, P_v, af * dv)).T
                f = f - lift(E1br_u, P_u, c2f * dv).T
            else:
                Uo, Vo = u[j, k + 1].T, v[j, k + 1].T
                c2m, afm = pre["rgt_c2"][j, k], pre["rgt_af"][j, k]
                c2p, afp = pre["lft_c2"][j, k + 1], pre["lft_af"][j, k + 1]
                K = c2m * pre["rgt_g0"][j, k] - c2p * pre["lft_g0"][j, k + 1]
                vj = P_v @ (Ebl_v @ Vo - Ebr_v @ V.T)
                gu_m, gu_p = P_u @ (E1br_u @ U.T), P_u @ (E1bl_u @ Uo)
                gv_m, gv_p = P_v @ (E1br_v @ V.T), P_v @ (E1bl_v @ Vo)
                jw = two_h * (c2m * gu_m - c2p * gu_p + afm * gv_m - afp * gv_p) + K
                flux_p = (1 - th) * (c2m * gu_m + afm * gv_m) + th * (c2p * gu_p + afp * gv_p)
                dv_p = (1 - th) * vj - tau * jw
                pen_p = pen_w(c2m, c2p, afm, afp) * vj - th * K
                f = f - lift(E1br_u, P_u, c2m * dv_p).T
                vt_rhs = (vt_rhs + four_hh * lift(Ebr_v, P_v, flux_p).T + four_hh * lift(E1br_v, P_v, afm * dv_p).T
                          + two_h * lift(Ebr_v, P_v, pen_p).T)

            vt_rhs_all[j, k] = vt_rhs
            rhs_ut = pre["Mc2_uv"][j, k].T @ V.reshape(-1, order="F") - f.reshape(-1, order="F")
            rhs_ut[0] += V[0, 0]
            ut[j, k] = cho_solve(pre["R_ut"][j, k], rhs_ut).reshape(qu1, qu1, order="F")

    for j in range(N):
        for k in range(N):
            V = v[j, k]
            BF = pre["mms_BF"][j, k]
            vq = P_h_v @ V @ P_h_v.T
            wv = ((1.0 - 2.0 * BF * vq) * W2d_h).reshape(-1, order="F")
            M = Phi2d_h_v.T @ (wv[:, None] * Phi2d_h_v)
            vt[j, k] = lu_solve(lu_factor(M), vt_rhs_all[j, k].reshape(-1, order="F")).reshape(qv1, qv1, order="F")
    return ut, vt
