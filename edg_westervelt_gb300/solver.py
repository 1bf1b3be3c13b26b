"""``solve``, error norms and the source-mode run, driving the GPU workspace.

Mirrors src/solver.jl:88-228 (``solve``), :772-836 (``_mms_errors``,
``difference_norms``), :838-888 (energy diagnostics) and :890-958
(``_run_source``) of WesterveltEDG.jl. The time loop runs on the GPU
(libwedg); the state crosses to the host only where a result is read
(final errors, receivers, diagnostics).
"""
import math

import numpy as np

from .coefficients import GaussianSource, _sym
from .precompute import precompute
from .quadrature import JacobiP
from .workspace import ErrorException, Workspace


def solve(q, N, T, *, mixed=True, flux="upwind", flux_params=None, sigma=0.0, boundary="absorbing_2beta",
          sigma_dirichlet=None, kappa=0.0, phase=(0.0, 0.0), coefficients=None, mode="mms", kx=1, ky=1,
          dt_fac=10, mass_solver="chebyshev", nblocks=None, initial_profile=None, return_state=False,
          source=None, record_every=20, slice_y=0.5, receivers=((0.45, 0.5), (0.7, 0.5), (0.85, 0.5)),
          snap_times=(), cheb_steps="per_element"):
    """Integrate the EDG scheme on (0,1)² up to T with RK4 (src/solver.jl:167-228).

    Returns the errors (erru, errv, errgradu, errE) in :mms mode, the final
    state with ``return_state=True``, or the time series of :source mode.
    """
    mode = _sym(mode)
    if mode not in ("mms", "initial_value", "source"):
        raise ErrorException(f"unknown mode {mode} (expected :mms, :initial_value or :source)")
    source = GaussianSource() if source is None else source
    pre, geo = precompute(q, N, mixed=mixed, flux=flux, flux_params=flux_params, sigma=sigma, boundary=boundary,
                          sigma_dirichlet=sigma_dirichlet, kappa=kappa, phase=phase, coefficients=coefficients,
                          mode=mode, kx=kx, ky=ky, source=source, mass_solver=mass_solver,
                          initial_profile=initial_profile)
    h = 1.0 / N
    u = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
    v = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
    dt = h / (dt_fac * q ** 2)
    nsteps = int(round(T / dt))
    dt = T / nsteps
    ws = Workspace(pre, N, nblocks=nblocks, cheb_steps=cheb_steps)
    if mode == "source":
        return run_source(u, v, dt, nsteps, N, h, pre, geo, ws, record_every=record_every, slice_y=slice_y,
                          receivers=receivers, snap_times=snap_times)
    ws.rk4_steps(u, v, 0.0, dt, nsteps)
    if return_state:
        return dict(u=u, v=v, N=N, h=h, P_u=pre["P_u"], P_v=pre["P_v"], S_u=geo["S_u"], W2d=geo["W2d"],
                    err_c2=geo["err_c2"])
    if mode != "mms":
        raise ErrorException("errors are only available in :mms mode; use return_state = true")
    return mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase)


def _elem(x):
    """(N, N, n, n) -> (N, N, n, n) C-ordered view for einsum over the element blocks."""
    return np.ascontiguousarray(x)


def mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase=(0.0, 0.0)):
    """L² errors of u, v, ∇u and the energy error against u = cos(ωT) Φ (src/solver.jl:774-810)."""
    px, py = phase
    P_u, P_v, S_u, W2d = pre["P_u"], pre["P_v"], geo["S_u"], geo["W2d"]
    om = pre["omega"]
    ctT, stT = math.cos(om * T), math.sin(om * T)
    pi = math.pi
    X = geo["xloc"][None, :, None, :]
    Y = geo["yloc"][:, None, :, None]
    sp = np.cos(2 * pi * kx * X + px) * np.sin(2 * pi * ky * Y + py)
    sp_x = -2 * pi * kx * np.sin(2 * pi * kx * X + px) * np.sin(2 * pi * ky * Y + py)
    sp_y = 2 * pi * ky * np.cos(2 * pi * kx * X + px) * np.cos(2 * pi * ky * Y + py)
    U, V = _elem(u), _elem(v)
    u_h = np.einsum("ra,jkab,sb->jkrs", P_u, U, P_u, optimize=True)
    v_h = np.einsum("ra,jkab,sb->jkrs", P_v, V, P_v, optimize=True)
    ux_h = (2 / h) * np.einsum("ra,jkab,sb->jkrs", P_u, U, S_u, optimize=True)
    uy_h = (2 / h) * np.einsum("ra,jkab,sb->jkrs", S_u, U, P_u, optimize=True)
    g = ((ctT - 1.0) * sp_x - ux_h) ** 2 + ((ctT - 1.0) * sp_y - uy_h) ** 2
    ev = (-om * stT * sp - v_h) ** 2
    s = h / 2
    return dict(erru=s * math.sqrt(np.sum(W2d * ((ctT - 1.0) * sp - u_h) ** 2)),
                errv=s * math.sqrt(np.sum(W2d * ev)),
                errgradu=s * math.sqrt(np.sum(W2d * g)),
                errE=s * math.sqrt(np.sum(W2d * (0.5 * geo["err_c2"] * g + 0.5 * ev))))


def difference_norms(A, B):
    """L² norms of u_A - u_B, v_A - v_B and the energy norm of the difference of two final
    states of ``solve(...; return_state=True)`` (src/solver.jl:819-836)."""
    h = B["h"]
    P_u, P_v, S_u, W2d = B["P_u"], B["P_v"], B["S_u"], B["W2d"]
    eu = _elem(A["u"] - B["u"])
    ev = _elem(A["v"] - B["v"])
    du = np.einsum("ra,jkab,sb->jkrs", P_u, eu, P_u, optimize=True)
    dux = (2 / h) * np.einsum("ra,jkab,sb->jkrs", P_u, eu, S_u, optimize=True)
    duy = (2 / h) * np.einsum("ra,jkab,sb->jkrs", S_u, eu, P_u, optimize=True)
    dv = np.einsum("ra,jkab,sb->jkrs", P_v, ev, P_v, optimize=True)
    s = h / 2
    return dict(erru=s * math.sqrt(np.sum(W2d * du ** 2)), errv=s * math.sqrt(np.sum(W2d * dv ** 2)),
                errE=s * math.sqrt(np.sum(W2d * (0.5 * B["err_c2"] * (dux ** 2 + duy ** 2) + 0.5 * dv ** 2))))


def energy_diag(u, v, pre, geo, N, h):
    """Westervelt energy Σ (h²/4) Σ W (½c²|∇u_h|² + (½ - ⅔βv_h) v_h²), max|v_h| and
    min(1 - 2βv_h) (src/solver.jl:864-888, 914-926)."""
    P_u, P_v, S_u, W2d = pre["P_u"], pre["P_v"], geo["S_u"], geo["W2d"]
    U, V = _elem(u), _elem(v)
    ux = (2 / h) * np.einsum("ra,jkab,sb->jkrs", P_u, U, S_u, optimize=True)
    uy = (2 / h) * np.einsum("ra,jkab,sb->jkrs", S_u, U, P_u, optimize=True)
    vh = np.einsum("ra,jkab,sb->jkrs", P_v, V, P_v, optimize=True)
    c2q, bq = geo["err_c2"], geo["err_beta"]
    Z = W2d * (0.5 * c2q * (ux ** 2 + uy ** 2) + (0.5 - (2 / 3) * bq * vh) * vh ** 2)
    Ee = (h ** 2 / 4) * Z.sum(axis=(2, 3))
    return float(np.sum(Ee)), float(np.max(np.abs(vh))), float(np.min(1 - 2 * bq * vh))


def _locate(s, N):
    i = min(max(int(math.ceil(s * N)), 1), N)
    return i, min(max(2 * (s * N - (i - 1)) - 1, -1.0), 1.0)


def _vrow(r, qv1):
    return np.array([JacobiP(r, 0, 0, d) for d in range(qv1)])


def run_source(u, v, dt, nsteps, N, h, pre, geo, ws, record_every, slice_y, receivers, snap_times):
    """Source mode (src/solver.jl:892-958): the RK4 loop with the receivers after every step,
    the slice, energy, max|v_h| and min(1 - 2βv_h) every record_every steps and the
    snapshots, all on the GPU in one call (wedg_run_source). The host computes what the
    reference computes on the host: receiver elements and basis rows (`locate`, `vrow`),
    the times (t += dt after every step) and the steps after which snapshots are taken."""
    qu1, qv1 = pre["qu1"], pre["qv1"]
    j0, eta0 = _locate(slice_y, N)
    slice_x = np.concatenate([geo["xloc"][k, :] for k in range(N)])
    rec_jk, rec_py, rec_px = [], [], []
    for xr, yr in receivers:
        kr, xir = _locate(xr, N)
        jr, etar = _locate(yr, N)
        rec_jk.append((jr - 1, kr - 1))
        rec_py.append(_vrow(etar, qv1))
        rec_px.append(_vrow(xir, qv1))
    # the times after each step and the snapshot steps, as the reference's loop finds them
    ts = np.empty(nsteps)
    t = 0.0
    snap_left, snap_after = sorted(snap_times), []
    for it in range(1, nsteps + 1):
        t += dt
        ts[it - 1] = t
        if snap_left and t >= snap_left[0]:
            snap_after.append(it)
            snap_left.pop(0)
    done, recv, E, vmax, nd, slices, snaps_g = ws.run_source(
        u, v, 0.0, dt, nsteps, record_every, rec_jk, np.array(rec_py).reshape(len(rec_jk), qv1),
        np.array(rec_px).reshape(len(rec_jk), qv1), j0 - 1, _vrow(eta0, qv1), snap_after,
        geo["err_c2"], geo["err_beta"])
    if done < nsteps or not ws.fin:
        raise ErrorException(f"blow-up at t={ts[done - 1] if done else dt}")
    rec_steps = [it for it in range(1, nsteps + 1) if it % record_every == 0 or it == nsteps]
    rec_t = [ts[it - 1] for it in rec_steps]
    snaps = [(ts[it - 1], G) for it, G in zip(snap_after, snaps_g)]
    rt_t = ts
    rt_v = recv
    rec_slice, rec_E, rec_vmax, rec_nd = list(slices), E, vmax, nd
    grid = np.concatenate([geo["xloc"][k, :] for k in range(N)])
    return dict(t=np.array(rec_t), slice_x=slice_x, slices=np.array(rec_slice).T, energy=np.array(rec_E),
                vmax=np.array(rec_vmax), ndmin=np.array(rec_nd), recv_t=np.array(rt_t), recv=np.array(rt_v),
                receivers=list(receivers), snaps=snaps, grid_x=grid, grid_y=grid.copy(), dt=dt)
