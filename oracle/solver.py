"""``solve`` and its end-of-run quantities, restated for the oracle.

Test infrastructure only. Follows ``src/solver.jl:167-228`` (``solve``),
``:774-810`` (``_mms_errors``), ``:819-836`` (``difference_norms``),
``:856-888`` (``_energy_diag!``) and ``:892-958`` (``_run_source``).
"""
import math

import numpy as np

from .precompute import precompute
from .quadrature import jacobi_p
from .rhs import OracleWorkspace


def solve(q, N, T, mixed=True, mode="mms", kx=1, ky=1, dt_fac=10, return_state=False,
          record_every=20, slice_y=0.5, receivers=((0.45, 0.5), (0.7, 0.5), (0.85, 0.5)),
          snap_times=(), phase=(0.0, 0.0), **kw):
    if mode not in ("mms", "initial_value", "source"):
        raise ValueError(f"unknown mode {mode} (expected :mms, :initial_value or :source)")
    pre, geo = precompute(q, N, mixed=mixed, mode=mode, kx=kx, ky=ky, phase=phase, **kw)
    h = 1.0 / N
    u = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
    v = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
    dt = h / (dt_fac * q ** 2)
    nsteps = int(round(T / dt))
    dt = T / nsteps
    ws = OracleWorkspace(pre)
    if mode == "source":
        return run_source(u, v, dt, nsteps, N, h, pre, geo, ws, record_every=record_every, slice_y=slice_y,
                          receivers=receivers, snap_times=snap_times)
    t = 0.0
    for _ in range(nsteps):
        ws.rk4_step(u, v, t, dt)
        t += dt
    if return_state:
        return dict(u=u, v=v, N=N, h=h, P_u=pre["P_u"], P_v=pre["P_v"], S_u=geo["S_u"], W2d=geo["W2d"],
                    err_c2=geo["err_c2"])
    if mode != "mms":
        raise ValueError("errors are only available in :mms mode; use return_state = true")
    return mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase)


def mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase=(0.0, 0.0)):
    """L² errors of u, v, ∇u and the energy error at T (src/solver.jl:774-810)."""
    px, py = phase
    P_u, P_v, S_u, W2d = pre["P_u"], pre["P_v"], geo["S_u"], geo["W2d"]
    qu1 = pre["qu1"]
    om = pre["omega"]
    ct_T, st_T = math.cos(om * T), math.sin(om * T)
    pi = math.pi
    erru = errv = errgradu = errE = 0.0
    for j in range(N):
        for k in range(N):
            Xq = np.tile(geo["xloc"][k, :][None, :], (qu1, 1))
            Yq = np.tile(geo["yloc"][j, :][:, None], (1, qu1))
            sp = np.cos(2 * pi * kx * Xq + px) * np.sin(2 * pi * ky * Yq + py)
            sp_x = -2 * pi * kx * np.sin(2 * pi * kx * Xq + px) * np.sin(2 * pi * ky * Yq + py)
            sp_y = 2 * pi * ky * np.cos(2 * pi * kx * Xq + px) * np.cos(2 * pi * ky * Yq + py)
            utrue = (ct_T - 1.0) * sp
            vtrue = -om * st_T * sp
            uxtrue = (ct_T - 1.0) * sp_x
            uytrue = (ct_T - 1.0) * sp_y
            U = u[j, k]
            V = v[j, k]
            u_h = P_u @ U @ P_u.T
            v_h = P_v @ V @ P_v.T
            ux_h = (2 / h) * (P_u @ U @ S_u.T)
            uy_h = (2 / h) * (S_u @ U @ P_u.T)
            c2q = geo["err_c2"][j, k]
            erru += np.sum(W2d * (utrue - u_h) ** 2)
            errv += np.sum(W2d * (vtrue - v_h) ** 2)
            g = (uxtrue - ux_h) ** 2 + (uytrue - uy_h) ** 2
            errgradu += np.sum(W2d * g)
            errE += np.sum(W2d * (0.5 * c2q * g + 0.5 * (vtrue - v_h) ** 2))
    s = h / 2
    return dict(erru=s * math.sqrt(erru), errv=s * math.sqrt(errv), errgradu=s * math.sqrt(errgradu),
                errE=s * math.sqrt(errE))


def difference_norms(A, B):
    """src/solver.jl:819-836."""
    N, h = B["N"], B["h"]
    P_u, P_v, S_u, W2d = B["P_u"], B["P_v"], B["S_u"], B["W2d"]
    erru = errv = errE = 0.0
    for j in range(N):
        for k in range(N):
            eu = A["u"][j, k] - B["u"][j, k]
            ev = A["v"][j, k] - B["v"][j, k]
            du = P_u @ eu @ P_u.T
            dux = (2 / h) * (P_u @ eu @ S_u.T)
            duy = (2 / h) * (S_u @ eu @ P_u.T)
            dv = P_v @ ev @ P_v.T
            c2q = B["err_c2"][j, k]
            erru += np.sum(W2d * du ** 2)
            errv += np.sum(W2d * dv ** 2)
            errE += np.sum(W2d * (0.5 * c2q * (dux ** 2 + duy ** 2) + 0.5 * dv ** 2))
    s = h / 2
    return dict(erru=s * math.sqrt(erru), errv=s * math.sqrt(errv), errE=s * math.sqrt(errE))


def energy_diag(u, v, pre, geo, N, h):
    """Per-element energy, max|v_h| and min(1 - 2βv_h) (src/solver.jl:868-888), reduced in (j, k) order."""
    W2d = geo["W2d"]
    P_u, S_u, P_v = pre["P_u"], geo["S_u"], pre["P_v"]
    Etot, vmax, ndmin = 0.0, 0.0, math.inf
    for j in range(N):
        for k in range(N):
            U = u[j, k]
            V = v[j, k]
            ux = (2 / h) * (P_u @ U @ S_u.T)
            uy = (2 / h) * (S_u @ U @ P_u.T)
            vh = P_v @ V @ P_v.T
            c2q = geo["err_c2"][j, k]
            bq = geo["err_beta"][j, k]
            Z = W2d * (0.5 * c2q * (ux ** 2 + uy ** 2) + (0.5 - (2 / 3) * bq * vh) * vh ** 2)
            Etot += (h ** 2 / 4) * np.sum(Z)
            vmax = max(vmax, float(np.max(np.abs(vh))))
            ndmin = min(ndmin, float(np.min(1 - 2 * bq * vh)))
    return Etot, vmax, ndmin


def _locate(s, N):
    i = min(max(int(math.ceil(s * N)), 1), N)
    return i, min(max(2 * (s * N - (i - 1)) - 1, -1.0), 1.0)


def _vrow(r, qv1):
    return np.array([jacobi_p(r, 0, 0, d) for d in range(qv1)])


def run_source(u, v, dt, nsteps, N, h, pre, geo, ws, record_every, slice_y, receivers, snap_times):
    """Source mode: RK4 with receivers every step and diagnostics every record_every steps
    (src/solver.jl:892-958)."""
    qu1, qv1, P_v = pre["qu1"], pre["qv1"], pre["P_v"]
    j0, eta0 = _locate(slice_y, N)
    Pveta0 = _vrow(eta0, qv1)
    slice_x = np.concatenate([geo["xloc"][k, :] for k in range(N)])
    rcv = []
    for xr, yr in receivers:
        kr, xir = _locate(xr, N)
        jr, etar = _locate(yr, N)
        rcv.append((jr - 1, kr - 1, _vrow(etar, qv1), _vrow(xir, qv1)))

    def recvf(vv):
        return [float(r[2] @ vv[r[0], r[1]] @ r[3]) for r in rcv]

    def slicef(vv):
        return np.concatenate([P_v @ (Pveta0 @ vv[j0 - 1, k]) for k in range(N)])

    def vgrid(vv):
        G = np.zeros((N * qu1, N * qu1))
        for j in range(N):
            for k in range(N):
                G[j * qu1:(j + 1) * qu1, k * qu1:(k + 1) * qu1] = P_v @ vv[j, k] @ P_v.T
        return G

    t = 0.0
    rec_t, rec_slice, rec_E, rec_vmax, rec_nd, rt_t, rt_v, snaps = [], [], [], [], [], [], [], []
    snap_left = sorted(snap_times)
    for it in range(1, nsteps + 1):
        ws.rk4_step(u, v, t, dt)
        t += dt
        if not ws.fin:
            raise RuntimeError(f"blow-up at t={t}")
        rt_t.append(t)
        rt_v.append(recvf(v))
        if it % record_every == 0 or it == nsteps:
            E, vmax, nd = energy_diag(u, v, pre, geo, N, h)
            rec_t.append(t)
            rec_slice.append(slicef(v))
            rec_E.append(E)
            rec_vmax.append(vmax)
            rec_nd.append(nd)
        if snap_left and t >= snap_left[0]:
            snaps.append((t, vgrid(v)))
            snap_left.pop(0)
    return dict(t=np.array(rec_t), slice_x=slice_x, slices=np.array(rec_slice).T, energy=np.array(rec_E),
                vmax=np.array(rec_vmax), ndmin=np.array(rec_nd), recv_t=np.array(rt_t), recv=np.array(rt_v),
                receivers=list(receivers), snaps=snaps, dt=dt)
