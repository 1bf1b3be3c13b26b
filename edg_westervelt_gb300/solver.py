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
from .workspace import ErrorException, Workspace, rk4_adjoint_forward_many, rk4_adjoint_reverse_many


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
                    err_c2=geo["err_c2"], w=pre["w"])
    if mode != "mms":
        raise ErrorException("errors are only available in :mms mode; use return_state = true")
    return mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase)


def _norms(N, qu1, qv1, w, P_u, S_u, err_c2, uA, vA, uB=None, vB=None, omega=0.0, T=0.0, kx=1, ky=1,
           phase=(0.0, 0.0), xloc=None, yloc=None):
    """wedg_norms: the error norms of src/solver.jl:774-836 on the GPU."""
    import ctypes
    from . import _lib as L
    keep = []

    def ptr(x):
        if x is None:
            return None
        x = np.asfortranarray(x, dtype=np.float64)
        keep.append(x)
        return x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    a = L.NormArgs()
    a.N, a.qu1, a.qv1 = int(N), int(qu1), int(qv1)
    a.w, a.P_u, a.S_u, a.err_c2 = ptr(w), ptr(P_u), ptr(S_u), ptr(err_c2)
    a.uA, a.vA, a.uB, a.vB = ptr(uA), ptr(vA), ptr(uB), ptr(vB)
    a.where = L.WEDG_HOST
    a.omega, a.ctT, a.stT = float(omega), math.cos(omega * T), math.sin(omega * T)
    a.kx, a.ky, a.px, a.py = int(kx), int(ky), float(phase[0]), float(phase[1])
    a.xloc, a.yloc = ptr(xloc), ptr(yloc)
    out = (ctypes.c_double * 4)()
    rc = L.lib().wedg_norms(ctypes.byref(a), out)
    if rc != L.WEDG_OK:
        raise RuntimeError(f"wedg_norms failed: {L.lib().wedg_status_string(rc).decode()}")
    return list(out)


def mms_errors(u, v, T, N, h, pre, geo, kx, ky, phase=(0.0, 0.0)):
    """L² errors of u, v, ∇u and the energy error against u = cos(ωT) Φ (src/solver.jl:774-810),
    summed on the GPU (wedg_norms)."""
    eu, ev, eg, eE = _norms(N, pre["qu1"], pre["qv1"], pre["w"], pre["P_u"], geo["S_u"], geo["err_c2"], u, v,
                            omega=pre["omega"], T=T, kx=kx, ky=ky, phase=phase, xloc=geo["xloc"], yloc=geo["yloc"])
    return dict(erru=eu, errv=ev, errgradu=eg, errE=eE)


def difference_norms(A, B):
    """L² norms of u_A - u_B, v_A - v_B and the energy norm of the difference of two final
    states of ``solve(...; return_state=True)`` (src/solver.jl:819-836), summed on the GPU."""
    N = B["N"]
    nu, nv = B["u"].shape[2], B["v"].shape[2]
    w = B["w"] if "w" in B else np.sqrt(np.diag(B["W2d"]))
    eu, ev, _, eE = _norms(N, nu, nv, w, B["P_u"], B["S_u"], B["err_c2"], A["u"], A["v"], B["u"], B["v"])
    return dict(erru=eu, errv=ev, errE=eE)


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


def piecewise_coefficients(c2, alpha, beta):
    """Coefficients constant on the cells of an m × n grid of (0,1)²: c2, alpha, beta are (m, n)
    arrays indexed [row (y), column (x)] of c², α and β (the parameter fields of the misfit
    gradient). The derivatives of c and α vanish inside the cells."""
    from .coefficients import cell_coefficients
    c2, alpha, beta = (np.asarray(a, dtype=np.float64) for a in (c2, alpha, beta))
    return cell_coefficients(np.sqrt(c2), alpha, beta)


def _misfit_problem(q, N, T, c2, alpha, beta, dt_fac, kw):
    """The forward problem of the misfit: pre, the workspace and the steps (src/solver.jl:198-206)."""
    c2 = np.asarray(c2, dtype=np.float64)
    m, n = c2.shape
    if N % m or N % n:
        raise ErrorException(f"the {m} × {n} parameter cells must be unions of elements (N = {N})")
    pre, _ = precompute(q, N, mode="source", coefficients=piecewise_coefficients(c2, alpha, beta), target="device",
                        **kw)
    dt = (1.0 / N) / (dt_fac * q ** 2)
    nsteps = int(round(T / dt))
    return pre, Workspace(pre, N), T / nsteps, nsteps, (m, n)


def _misfit_value(u, N, receivers, u_obs):
    """J = ½ Σ_r (u_h(x_r) - u_obs_r)² of the final u and its adjoint λ_u = ∂J/∂U."""
    nu = u.shape[2]
    lam_u = np.zeros_like(u)
    J = 0.0
    for (xr, yr), obs in zip(receivers, u_obs):
        kr, xi = _locate(xr, N)
        jr, eta = _locate(yr, N)
        py, px = _vrow(eta, nu), _vrow(xi, nu)
        res = float(py @ u[jr - 1, kr - 1] @ px) - obs
        J += 0.5 * res * res
        lam_u[jr - 1, kr - 1] += res * np.outer(py, px)
    return J, lam_u


def misfit(q, N, T, c2, alpha, beta, receivers, u_obs, *, dt_fac=10, **kw):
    """The final-time misfit J = ½ Σ_r (u_h(x_r, T) - u_obs_r)² of a source-mode run from the zero
    state, for c², α and β constant on the cells of the grid of the (m, n) arrays c2, alpha, beta
    (the forward problem of misfit_gradient, without the reverse sweep)."""
    pre, ws, dt, nsteps, _ = _misfit_problem(q, N, T, c2, alpha, beta, dt_fac, kw)
    u = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
    v = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
    if ws.rk4_steps(u, v, 0.0, dt, nsteps) != nsteps or not ws.fin:
        raise ErrorException("the forward run of the misfit did not complete")
    return _misfit_value(u, N, receivers, u_obs)[0]


def misfit_gradient(q, N, T, c2, alpha, beta, receivers, u_obs, *, dt_fac=10, every=32, **kw):
    """The discrete adjoint's gradient of the final-time misfit J = ½ Σ_r (u_h(x_r, T) - u_obs_r)²
    of a source-mode run from the zero state with respect to c², α and β constant on the cells
    of the grid of the (m, n) arrays c2, alpha, beta (every cell a block of N/m × N/n elements).
    Returns (J, dict(c2=..., alpha=..., beta=...)) with gradients of the cells' shape. The forward
    run, the misfit and the final-time adjoint λ_u = Σ_r (u_h(x_r) - u_obs_r) ∂u_h(x_r)/∂U are
    computed here; the forward run (keeping checkpoints every `every` steps) and the reverse
    sweep are wedg_rk4_adjoint_forward and wedg_rk4_adjoint_reverse."""
    pre, ws, dt, nsteps, (m, n) = _misfit_problem(q, N, T, c2, alpha, beta, dt_fac, kw)
    nu, nv = pre["qu1"], pre["qv1"]
    u0 = np.zeros((N, N, nu, nu), order="F")
    v0 = np.zeros((N, N, nv, nv), order="F")
    u, v = ws.rk4_adjoint_forward(u0, v0, 0.0, dt, nsteps, every=every)
    J, lam_u = _misfit_value(u, N, receivers, u_obs)
    _, _, gc2, gal, gbe = ws.rk4_adjoint_reverse(lam_u, np.zeros_like(v), params=True)
    # element (j, k) lies in cell (j // (N/m), k // (N/n))
    cells = lambda g: g.reshape(m, N // m, n, N // n).sum(axis=(1, 3))
    return J, dict(c2=cells(gc2), alpha=cells(gal), beta=cells(gbe))


def misfit_gradients(q, N, T, fields, receivers, u_obs, *, dt_fac=10, every=32, **kw):
    """misfit_gradient for several parameter fields at once: fields is a list of (c2, alpha, beta)
    cell arrays and u_obs a list of observation vectors (one per field, or one for all). The
    forward runs and the reverse sweeps of all of them run together (wedg_rk4_adjoint_forward_many,
    wedg_rk4_adjoint_reverse_many), so that problems too small to fill the GPU alone fill it
    together. Returns a list of (J, dict(c2=..., alpha=..., beta=...))."""
    n = len(fields)
    obs = list(u_obs) if len(u_obs) == n and np.ndim(u_obs[0]) == 1 else [u_obs] * n
    probs = [_misfit_problem(q, N, T, c2, al, be, dt_fac, kw) for c2, al, be in fields]
    dt, nsteps = probs[0][2], probs[0][3]
    wss = [p[1] for p in probs]
    pre = probs[0][0]
    nu, nv = pre["qu1"], pre["qv1"]
    u0 = [np.zeros((N, N, nu, nu), order="F") for _ in range(n)]
    v0 = [np.zeros((N, N, nv, nv), order="F") for _ in range(n)]
    uT, vT = rk4_adjoint_forward_many(wss, u0, v0, 0.0, dt, nsteps, every=every)
    Js, lams = zip(*[_misfit_value(uT[i], N, receivers, obs[i]) for i in range(n)])
    out = rk4_adjoint_reverse_many(wss, list(lams), [np.zeros_like(x) for x in vT], params=True)
    res = []
    for i in range(n):
        m, nn = probs[i][4]
        cells = lambda g: g.reshape(m, N // m, nn, N // nn).sum(axis=(1, 3))   # noqa: E731
        _, _, gc2, gal, gbe = out[i]
        res.append((Js[i], dict(c2=cells(gc2), alpha=cells(gal), beta=cells(gbe))))
    return res
