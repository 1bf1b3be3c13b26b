"""GPU ``Workspace``, ``edg_rhs!`` and ``rk4_step!`` behind the reference's API.

Mirrors src/rhs.jl:166-220 (``Workspace``), :475-571 (``edg_rhs!``,
``edg_rhs``) and src/solver.jl:278-339 (``rk4_step!``, ``rk4_step``) of
WesterveltEDG.jl. The workspace holds a libwedg handle: the data of ``pre``
are copied to the GPU once, and every call runs the sm_103a kernels.

State arrays follow the reference's layout: numpy arrays of shape
(N, N, q+1, q+1) in Fortran (column-major) order, like Julia's
``Array{Float64,4}``, or CUDA tensors holding the same bytes (any
contiguous torch tensor with N²(q+1)² doubles, read as that column-major array).
"""
import ctypes
import warnings

import numpy as np

from . import _lib as L
from .errors import ArgumentErrorException, DimensionMismatch, ErrorException


def _f64(a):
    return np.require(a, dtype=np.float64, requirements=["F_CONTIGUOUS", "ALIGNED"])


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _is_device(x):
    return hasattr(x, "is_cuda") and x.is_cuda


def _dptr(x):
    if x.dtype.__str__() != "torch.float64" or not x.is_contiguous():
        raise TypeError("device state must be a contiguous torch.float64 CUDA tensor")
    return ctypes.cast(ctypes.c_void_p(x.data_ptr()), ctypes.POINTER(ctypes.c_double))


def _shape(x, nu, N):
    """Julia shape of a state array (numpy: its shape; device: from the element count)."""
    if _is_device(x):
        n = x.numel()
        q = int(round((n / (N * N)) ** 0.5)) if N > 0 else 0
        shp = (N, N, q, q) if N * N * q * q == n else (n, 1, 1, 1)
    else:
        shp = tuple(x.shape) + (1,) * (4 - x.ndim) if x.ndim <= 4 else (x.size, 1, 1, 1)
    return (ctypes.c_int64 * 4)(*shp)


def _points_struct(points, keep):
    """wedg_points for the point values of precompute_points (arrays kept alive in keep)."""
    P = L.Points()
    null = ctypes.POINTER(ctypes.c_double)()

    def arr(a):
        if a is None:
            return null
        a = _f64(a)
        keep[id(a)] = a
        return _ptr(a)
    for name, value, cells in (("c_q", "c_value", "c_cells"), ("alpha_q", "alpha_value", "alpha_cells"),
                               ("beta_h", "beta_value", "beta_cells")):
        f = points[name]
        setattr(P, name, arr(f.get("array")))
        setattr(P, value, float(f.get("value", 0.0)))
        if "table" in f:
            t = getattr(P, cells)
            t.values = arr(np.asfortranarray(f["table"].T))       # row-major (m, n) bytes
            t.rows, t.cols = f["table"].shape

    def face(fv, values, scale=None):
        if values is None:                      # a constant family: (None, value)
            return
        fv.at, fv.lo, fv.hi = (arr(x) for x in values)
        fv.jump_scale = float(scale)
    for key, fld, (hn, vn) in (("c", "c_q", ("hc", "vc")), ("a", "alpha_q", ("ha", "va")),
                               ("b", "beta_h", ("hb", "vb"))):
        fam = points["faces"][key]
        if fam is None:                         # a constant (its value) or a table (looked up on the device)
            getattr(P, hn).value = getattr(P, vn).value = float(points[fld].get("value", 0.0))
        else:
            out, s = fam
            face(getattr(P, hn), out["h"], s)
            face(getattr(P, vn), out["v"], s)
    if points.get("g0") is not None:
        (hv, hs), (vv, vs) = points["g0"]["h"], points["g0"]["v"]
        face(P.hg0, hv, hs)
        face(P.vg0, vv, vs)
    for name in ("sp_h", "cdiv_h", "ddiv_h"):
        setattr(P, name, arr(points.get(name)))
    src, grid = points["source"], points["grid"]
    P.xloc, P.yloc = arr(grid["xloc"]), arr(grid["yloc"])
    P.xloc_h, P.yloc_h = arr(grid["xloc_h"]), arr(grid["yloc_h"])
    P.src_amp, P.src_x0, P.src_y0, P.src_r0 = src["amp"], src["x0"], src["y0"], src["r0"]
    return P


def _default_nblocks(pre, N):
    """src/rhs.jl:139-142 (kept for the `nb` attribute; the GPU grid replaces the blocks)."""
    import os
    w = N * N * pre["qu1"] ** 2
    nt = os.cpu_count() or 1
    return 1 if w < 5000 else min(4, nt) if w < 20000 else nt


class Workspace:
    """GPU counterpart of ``Workspace(pre, N; nblocks)`` (src/rhs.jl:184-220).

    Holds the device copy of ``pre`` and all scratch. ``nblocks`` is accepted
    for compatibility (it must be ≥ 1, as in the reference) and only sets the
    informational ``nb``: one GPU launch covers every element.

    cheb_steps: "per_element" (default; every element takes the Chebyshev step
    count its own spectral interval needs, each to the same tolerance) or
    "common_max" (all elements take the largest count, as src/rhs.jl:911-918).
    fast_path=False keeps the quadrature form of the volume terms and the stored
    inverses; modal_traces=False keeps the traces at the face points (the interior
    flux slots are then evaluated point by point, as src/rhs.jl:589-700 does).
    """

    def __init__(self, pre, N, nblocks=None, cheb_steps="per_element", fast_path=True, modal_traces=True):
        if nblocks is None:
            nblocks = _default_nblocks(pre, N)
        if not nblocks >= 1:
            raise ErrorException(f"nblocks must be ≥ 1 (got {nblocks})")
        E = N * N
        self.nb = min(int(nblocks), max(1, E // 4))
        self.pre = pre
        self.N = N
        self.nu, self.nv = pre["qu1"], pre["qv1"]
        self._h = None
        self.ut = np.zeros((N, N, self.nu, self.nu), order="F")
        self.vt = np.zeros((N, N, self.nv, self.nv), order="F")
        self.fin = True
        # pre of another mesh: the reference's Workspace accepts it and its edg_rhs! refuses it
        # with a DimensionMismatch (src/rhs.jl:500-503); no device workspace is made from it
        self._mismatch = (pre["N"] != N) if "points" in pre else pre["Cw"].shape[1] != E
        if self._mismatch:
            return
        cfg = L.Config()
        cfg.N, cfg.qu1, cfg.qv1, cfg.q_high = N, pre["qu1"], pre["qv1"], pre["q_high"]
        cfg.theta, cfg.tau, cfg.lambda_u, cfg.lambda_v = pre["theta"], pre["tau"], pre["lambda_u"], pre["lambda_v"]
        cfg.omega = pre["omega"]
        cfg.mms_on, cfg.src_on = int(pre["mms_on"]), int(pre["src_on"])
        cfg.one_sided = int(pre.get("one_sided", False))     # a pre of point values: the device decides
        cfg.mass_solver = 0 if pre["mass_solver"] == "chebyshev" else 1
        cfg.mass_tol = pre["mass_tol"]
        cfg.src_omega, cfg.src_Ts = pre["source"].omega, pre["source"].Ts
        for i, side in enumerate(("bot", "top", "lft", "rgt")):
            bs = pre["bc"][side]
            cfg.kind[i] = L.KINDS[bs["kind"]]
            cfg.gamma_abc[i], cfg.eta_abc[i], cfg.sigma[i] = bs["gamma_abc"], bs["eta_abc"], bs["sigma"]
            cfg.kb[i], cfg.kappa[i] = bs["kb"], bs["kappa"]
        cfg.cheb_steps = {"per_element": 0, "common_max": 1}[cheb_steps]
        cfg.general_only = 0 if fast_path else 1
        cfg.point_traces = 0 if modal_traces else 1
        self._cfg = cfg
        keep = {}
        p = L.Pre()
        points = pre.get("points")
        for name in L.PRE_FIELDS:
            a = pre.get(name)
            if a is None or (name == "Ainv_u" and not a.flags.f_contiguous):
                # NULL: Ainv_u is not needed by the constant-coefficient kernels, else computed on the
                # device; a pre of point values has no element or face arrays
                setattr(p, name, ctypes.POINTER(ctypes.c_double)())
                continue
            a = _f64(np.ascontiguousarray(a) if not a.flags.f_contiguous else a)
            keep[name] = a
            setattr(p, name, _ptr(a))
        h = ctypes.c_void_p()
        if points is None:
            rc = L.lib().wedg_create(ctypes.byref(cfg), ctypes.byref(p), ctypes.byref(h))
            msg = ""
        else:
            pts = _points_struct(points, keep)
            buf = ctypes.create_string_buffer(512)
            rc = L.lib().wedg_create_points(ctypes.byref(cfg), ctypes.byref(p), ctypes.byref(pts), buf, 512,
                                            ctypes.byref(h))
            msg = buf.value.decode("utf-8")
            if rc == L.WEDG_ERR_ARGUMENT and msg.startswith("mode = :mms"):
                raise ArgumentErrorException(msg)   # the device-side form of src/solver.jl:744-747
        if rc == L.WEDG_ERR_NO_DEVICE:
            raise RuntimeError("libwedg: no CUDA device available")
        if rc != L.WEDG_OK:
            raise RuntimeError(f"wedg_create failed: {L.lib().wedg_status_string(rc).decode()}" +
                               (f": {msg}" if msg else ""))
        self._h = h
        self.one_sided = bool(L.lib().wedg_one_sided(h))

    def __del__(self):
        if getattr(self, "_h", None):
            L.lib().wedg_destroy(self._h)
            self._h = None

    # ---- status handling
    def _message(self):
        buf = ctypes.create_string_buffer(512)
        L.lib().wedg_error_message(self._h, buf, 512)
        return buf.value.decode("utf-8")

    def _check(self, rc):
        if rc == L.WEDG_OK:
            return
        if rc == L.WEDG_WARN_CG_NOT_CONVERGED:
            warnings.warn(self._message())
            return
        msg = self._message()
        if rc == L.WEDG_ERR_DIMENSION:
            raise DimensionMismatch(msg)
        if rc in (L.WEDG_ERR_BOUNDARY_WEIGHT, L.WEDG_ERR_MASS_NOT_PD, L.WEDG_ERR_ARGUMENT):
            raise ErrorException(msg)
        raise RuntimeError(f"libwedg: {L.lib().wedg_status_string(rc).decode()}: {msg}")

    def stats(self):
        self._refuse_mismatch()
        s = L.Stats()
        L.lib().wedg_get_stats(self._h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    @property
    def error_key(self):
        return int(L.lib().wedg_error_key(self._h))

    @property
    def stream(self):
        """The cudaStream_t the workspace launches on (an int)."""
        return L.lib().wedg_get_stream(self._h)

    def set_stream(self, stream_ptr):
        L.lib().wedg_set_stream(self._h, ctypes.c_void_p(stream_ptr))

    # ---- calls
    def _refuse_mismatch(self):
        if self._mismatch:
            raise DimensionMismatch(f"state, workspace and pre do not match (N = {self.N}, q_u + 1 = {self.nu}, "
                                    f"q_v + 1 = {self.nv})")

    def rhs(self, u, v, t, ut=None, vt=None):
        """edg_rhs!: the right-hand side at time t into ut, vt (default the workspace's own)."""
        self._refuse_mismatch()
        N, nu, nv = self.N, self.nu, self.nv
        if _is_device(u):
            if ut is None or vt is None:
                raise ValueError("device inputs need device outputs ut, vt")
            rc = L.lib().wedg_rhs(self._h, _dptr(u), _dptr(v), float(t), _dptr(ut), _dptr(vt),
                                  _shape(u, nu, N), _shape(v, nv, N), L.WEDG_DEVICE)
            self._check(rc)
            return ut, vt
        u = _f64(u)
        v = _f64(v)
        ut = self.ut if ut is None else ut
        vt = self.vt if vt is None else vt
        rc = L.lib().wedg_rhs(self._h, _ptr(u), _ptr(v), float(t), _ptr(ut), _ptr(vt),
                              _shape(u, nu, N), _shape(v, nv, N), L.WEDG_HOST)
        self._check(rc)
        return ut, vt

    def rhs_adjoint(self, u, v, t, lam_u, lam_v):
        """wedg_rhs_adjoint: Jᵀ(λ_u, λ_v), the gradient of λ_u·ut + λ_v·vt with respect to u and
        v, where (ut, vt) is the right-hand side at (u, v, t). Host arrays in, new arrays out."""
        self._refuse_mismatch()
        N, nu, nv = self.N, self.nu, self.nv
        u, v, lam_u, lam_v = _f64(u), _f64(v), _f64(lam_u), _f64(lam_v)
        gu = np.zeros((N, N, nu, nu), order="F")
        gv = np.zeros((N, N, nv, nv), order="F")
        rc = L.lib().wedg_rhs_adjoint(self._h, _ptr(u), _ptr(v), float(t), _ptr(lam_u), _ptr(lam_v), _ptr(gu),
                                      _ptr(gv), _shape(u, nu, N), _shape(v, nv, N), L.WEDG_HOST)
        self._check(rc)
        return gu, gv

    def rk4_adjoint(self, u0, v0, t0, dt, nsteps, lam_u, lam_v, every=32, params=False):
        """wedg_rk4_adjoint: the gradient with respect to the initial state (u0, v0) of
        λ_u·u(T) + λ_v·v(T) after nsteps RK4 steps (the adjoint state at t0 for the final-time
        adjoint (λ_u, λ_v)); checkpoints every `every` steps. With params, also the gradients with
        respect to every element's c², α and β (source mode, coefficients constant per element),
        as (N, N) arrays. Host arrays in, new arrays out."""
        self._refuse_mismatch()
        N, nu, nv = self.N, self.nu, self.nv
        u0, v0, lam_u, lam_v = _f64(u0), _f64(v0), _f64(lam_u), _f64(lam_v)
        gu = np.zeros((N, N, nu, nu), order="F")
        gv = np.zeros((N, N, nv, nv), order="F")
        gp = [np.zeros((N, N), order="F") for _ in range(3)] if params else None
        null = ctypes.POINTER(ctypes.c_double)()
        pc = [_ptr(g) for g in gp] if params else [null, null, null]
        rc = L.lib().wedg_rk4_adjoint(self._h, _ptr(u0), _ptr(v0), float(t0), float(dt), int(nsteps), int(every),
                                      _ptr(lam_u), _ptr(lam_v), _ptr(gu), _ptr(gv), pc[0], pc[1], pc[2],
                                      _shape(u0, nu, N), _shape(v0, nv, N), L.WEDG_HOST)
        self._check(rc)
        return (gu, gv, *gp) if params else (gu, gv)

    def rk4_adjoint_forward(self, u0, v0, t0, dt, nsteps, every=32):
        """wedg_rk4_adjoint_forward: the forward run of a reverse sweep, checkpoints kept in the
        workspace; returns the final state (new arrays)."""
        self._refuse_mismatch()
        N, nu, nv = self.N, self.nu, self.nv
        u0, v0 = _f64(u0), _f64(v0)
        uT = np.zeros((N, N, nu, nu), order="F")
        vT = np.zeros((N, N, nv, nv), order="F")
        rc = L.lib().wedg_rk4_adjoint_forward(self._h, _ptr(u0), _ptr(v0), float(t0), float(dt), int(nsteps),
                                              int(every), _ptr(uT), _ptr(vT), _shape(u0, nu, N), _shape(v0, nv, N),
                                              L.WEDG_HOST)
        self._check(rc)
        return uT, vT

    @property
    def launch_shape(self):
        """(k_prep threads per block, mass-solve threads per block) (wedg_get_launch_shape)."""
        p, m = ctypes.c_int(), ctypes.c_int()
        self._check(L.lib().wedg_get_launch_shape(self._h, ctypes.byref(p), ctypes.byref(m)))
        return p.value, m.value

    def set_launch_shape(self, prep_threads, mass_threads):
        """wedg_set_launch_shape: 32, 64, 96 or 128 threads per block each; results do not
        depend on them."""
        self._check(L.lib().wedg_set_launch_shape(self._h, int(prep_threads), int(mass_threads)))

    def autotune(self, u, v, t0, dt, steps=4):
        """wedg_autotune on the CUDA state tensors (u, v), which are left unchanged: keeps the
        fastest launch shape; returns the best milliseconds per RK4 step."""
        if not (_is_device(u) and _is_device(v)):
            raise TypeError("autotune takes CUDA tensors")
        best = ctypes.c_double(0.0)
        self._check(L.lib().wedg_autotune(self._h, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                          float(t0), float(dt), int(steps), ctypes.byref(best)))
        return best.value

    def set_adjoint_memory(self, nbytes):
        """wedg_set_adjoint_memory: device bytes the reverse sweep may use to keep the forward
        data of one checkpoint segment's stages (negative: half the free memory; 0: never)."""
        self._check(L.lib().wedg_set_adjoint_memory(self._h, int(nbytes)))

    def rk4_adjoint_reverse(self, lam_u, lam_v, params=False):
        """wedg_rk4_adjoint_reverse: the reverse sweep of the last rk4_adjoint_forward for the
        final-time adjoint (λ_u, λ_v); returns (gu, gv) and, with params, the per-element
        gradients with respect to c², α, β."""
        N, nu, nv = self.N, self.nu, self.nv
        lam_u, lam_v = _f64(lam_u), _f64(lam_v)
        gu = np.zeros((N, N, nu, nu), order="F")
        gv = np.zeros((N, N, nv, nv), order="F")
        gp = [np.zeros((N, N), order="F") for _ in range(3)] if params else None
        null = ctypes.POINTER(ctypes.c_double)()
        pc = [_ptr(g) for g in gp] if params else [null, null, null]
        rc = L.lib().wedg_rk4_adjoint_reverse(self._h, _ptr(lam_u), _ptr(lam_v), _ptr(gu), _ptr(gv), pc[0], pc[1],
                                              pc[2], L.WEDG_HOST)
        self._check(rc)
        return (gu, gv, *gp) if params else (gu, gv)

    def rk4_steps(self, u, v, t0, dt, nsteps, stop_nonfinite=False):
        """nsteps RK4 steps in place from t0 (t advancing by repeated addition of dt).
        Returns the number of steps completed; sets self.fin."""
        self._refuse_mismatch()
        N = self.N
        done = ctypes.c_int64(0)
        fin = ctypes.c_int(1)
        if _is_device(u):
            pu, pv, where = _dptr(u), _dptr(v), L.WEDG_DEVICE
        else:
            if not (isinstance(u, np.ndarray) and u.dtype == np.float64 and u.flags.f_contiguous
                    and isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags.f_contiguous):
                raise TypeError("rk4_step! updates u, v in place: pass Fortran-ordered float64 arrays")
            pu, pv, where = _ptr(u), _ptr(v), L.WEDG_HOST
        rc = L.lib().wedg_rk4_steps(self._h, pu, pv, float(t0), float(dt), int(nsteps), _shape(u, self.nu, N),
                                    _shape(v, self.nv, N), where, int(stop_nonfinite), ctypes.byref(done),
                                    ctypes.byref(fin))
        self.fin = bool(fin.value)
        self._check(rc)
        return int(done.value)


    def run_source(self, u, v, t0, dt, nsteps, record_every, rec_jk, rec_py, rec_px, slice_j, slice_py,
                   snap_after, err_c2, err_beta):
        """The source-mode loop with its diagnostics on the device (wedg_run_source): u, v
        advance in place; returns (steps_done, recv (nsteps × nrec), energy, vmax, ndmin,
        slices (records × N q_u1), snapshots (nsnap × (N q_u1)², column-major))."""
        self._refuse_mismatch()
        N, nq = self.N, self.nu
        if not (isinstance(u, np.ndarray) and u.flags.f_contiguous and isinstance(v, np.ndarray)
                and v.flags.f_contiguous and u.dtype == np.float64 and v.dtype == np.float64):
            raise TypeError("run_source advances u, v in place: pass Fortran-ordered float64 arrays")
        nrec = len(rec_jk)
        nrecord = nsteps // record_every + (1 if nsteps % record_every else 0)
        keep = []

        def arr(a, dtype=np.float64):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(np.ctypeslib.as_ctypes_type(dtype)))

        out = dict(recv=np.zeros((max(nsteps, 0), nrec)), energy=np.zeros(nrecord), vmax=np.zeros(nrecord),
                   ndmin=np.zeros(nrecord), slices=np.zeros((nrecord, N * nq)),
                   snaps=np.zeros((len(snap_after), N * nq * N * nq)))
        r = L.SourceRun()
        r.nsteps, r.record_every, r.t0, r.dt = int(nsteps), int(record_every), float(t0), float(dt)
        r.nrec = nrec
        jk = np.array(rec_jk, dtype=np.int32).reshape(nrec, 2)
        r.rec_j, r.rec_k = arr(jk[:, 0], np.int32), arr(jk[:, 1], np.int32)
        r.rec_py, r.rec_px = arr(np.reshape(rec_py, (nrec, self.nv))), arr(np.reshape(rec_px, (nrec, self.nv)))
        r.slice_j, r.slice_py = int(slice_j), arr(slice_py)
        r.nsnap, r.snap_after = len(snap_after), arr(np.array(snap_after, dtype=np.int64), np.int64)
        r.err_c2 = arr(np.asarray(err_c2, dtype=np.float64).reshape(-1, order="F"))
        r.err_beta = arr(np.asarray(err_beta, dtype=np.float64).reshape(-1, order="F"))
        for k in ("recv", "energy", "vmax", "ndmin", "slices", "snaps"):
            setattr(r, k, out[k].ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        done = ctypes.c_int64(0)
        fin = ctypes.c_int(1)
        rc = L.lib().wedg_run_source(self._h, _ptr(u), _ptr(v), _shape(u, self.nu, N), _shape(v, self.nv, N),
                                     L.WEDG_HOST, ctypes.byref(r), ctypes.byref(done), ctypes.byref(fin))
        self.fin = bool(fin.value)
        self._check(rc)
        snaps = [s.reshape((N * nq, N * nq), order="F") for s in out["snaps"]]
        return int(done.value), out["recv"], out["energy"], out["vmax"], out["ndmin"], out["slices"], snaps


class Batch:
    """Many independent instances advanced together (wedg_batch_*): each a Workspace of its own
    N, degrees, flux, boundary kinds and coefficients. Instances that run the same kernels form a
    bucket, whose instances run their own launches on their own streams (the default) or every
    stage kernel once over all of them (set_shape, autotune); the steps are replays of CUDA graphs
    of one and of four RK4 steps of all instances. No counterpart in the reference (there,
    batching is a loop over solves)."""

    def __init__(self, workspaces):
        self.ws = list(workspaces)
        n = len(self.ws)
        arr = (ctypes.c_void_p * n)(*[w._h for w in self.ws])
        h = ctypes.c_void_p()
        rc = L.lib().wedg_batch_create(n, arr, ctypes.byref(h))
        if rc != L.WEDG_OK:
            raise RuntimeError(f"wedg_batch_create failed: {L.lib().wedg_status_string(rc).decode()}")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            L.lib().wedg_batch_destroy(self._h)
            self._h = None

    def rk4_steps(self, us, vs, t0s, dts, nsteps, stop_nonfinite=True):
        """nsteps RK4 steps of every instance in place on its CUDA state tensors (contiguous
        float64, the reference's layout). Returns (steps_done, finite, status) per instance and
        raises the first instance error like Workspace.rk4_steps."""
        n = len(self.ws)
        if not (len(us) == len(vs) == len(t0s) == len(dts) == n):
            raise ValueError("one state, t0 and dt per instance")
        for w, u, v in zip(self.ws, us, vs):
            if not (_is_device(u) and _is_device(v)):
                raise TypeError("batched steps take CUDA tensors")
            if u.numel() != w.N * w.N * w.nu * w.nu or v.numel() != w.N * w.N * w.nv * w.nv:
                raise DimensionMismatch(f"state, workspace and pre do not match (N = {w.N}, q_u + 1 = {w.nu}, "
                                        f"q_v + 1 = {w.nv})")
        pu = (ctypes.c_void_p * n)(*[u.data_ptr() for u in us])
        pv = (ctypes.c_void_p * n)(*[v.data_ptr() for v in vs])
        t0 = np.array(t0s, dtype=np.float64)
        dt = np.array(dts, dtype=np.float64)
        done = np.zeros(n, dtype=np.int64)
        fin = (ctypes.c_int * n)()
        st = (ctypes.c_int * n)()
        L.lib().wedg_batch_rk4_steps(self._h, pu, pv, _ptr(t0), _ptr(dt), int(nsteps), int(stop_nonfinite),
                                     done.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), fin, st)
        for i, w in enumerate(self.ws):
            w.fin = bool(fin[i])
        for i, w in enumerate(self.ws):
            w._check(st[i])
        return [int(x) for x in done], [bool(x) for x in fin], [int(x) for x in st]

    def shapes(self):
        """The buckets and their launch shapes (wedg_batch_get_shape): a list of dicts with the
        degrees + 1, the instances, the kernel family and the shape."""
        out = []
        for k in range(L.lib().wedg_batch_bucket_count(self._h)):
            s = L.BatchShape()
            if L.lib().wedg_batch_get_shape(self._h, k, ctypes.byref(s)) != L.WEDG_OK:
                raise RuntimeError("wedg_batch_get_shape failed")
            out.append({f: int(getattr(s, f)) for f, _ in s._fields_})
        return out

    def set_shape(self, bucket, prep_threads, mass_threads, persist=-1):
        """wedg_batch_set_shape: the launch shape of one bucket (results do not depend on it);
        persist -1 launches the bucket's instances one by one (the default), 0 runs each stage
        kernel once over them, p > 0 the same on a persistent grid."""
        rc = L.lib().wedg_batch_set_shape(self._h, int(bucket), int(prep_threads), int(mass_threads), int(persist))
        if rc != L.WEDG_OK:
            raise ErrorException("launch shapes are 32, 64, 96 or 128 threads per block and persist -1 to 8")

    def autotune(self, us, vs, t0s, dts, steps=3):
        """wedg_batch_autotune: the launch shapes of every bucket, each tuned alone from copies of
        its instances' states (left unchanged), then kept only if the whole batch's step beats the
        shapes it had before in paired trials. Returns the median milliseconds per batch step of
        the shapes kept."""
        n = len(self.ws)
        if not (len(us) == len(vs) == len(t0s) == len(dts) == n):
            raise ValueError("one state, t0 and dt per instance")
        pu = (ctypes.c_void_p * n)(*[u.data_ptr() for u in us])
        pv = (ctypes.c_void_p * n)(*[v.data_ptr() for v in vs])
        t0 = np.array(t0s, dtype=np.float64)
        dt = np.array(dts, dtype=np.float64)
        best = ctypes.c_double(0.0)
        rc = L.lib().wedg_batch_autotune(self._h, pu, pv, _ptr(t0), _ptr(dt), int(steps), ctypes.byref(best))
        if rc != L.WEDG_OK:
            for w in self.ws:
                w._check(rc)
            raise RuntimeError(f"wedg_batch_autotune failed: {L.lib().wedg_status_string(rc).decode()}")
        return best.value


def _ptr_array(arrays):
    return (ctypes.POINTER(ctypes.c_double) * len(arrays))(*[_ptr(a) for a in arrays])


def _check_group(wss, rc):
    if rc == L.WEDG_OK:
        return
    for w in wss:                                 # the workspace that failed carries the message
        if L.lib().wedg_error_message(w._h, None, 0) != L.WEDG_OK:
            w._check(rc)
    raise RuntimeError(f"libwedg: {L.lib().wedg_status_string(rc).decode()}")


def rk4_adjoint_forward_many(wss, u0s, v0s, t0, dt, nsteps, every=32):
    """wedg_rk4_adjoint_forward_many: the forward runs of several workspaces (same degrees,
    coefficient kernels and mass solver) at once, each stage one multi-instance launch over all of
    them; checkpoints kept in each workspace. Host arrays in; returns the final states."""
    n = len(wss)
    for w in wss:
        w._refuse_mismatch()
    u0s = [_f64(a) for a in u0s]
    v0s = [_f64(a) for a in v0s]
    uT = [np.zeros((w.N, w.N, w.nu, w.nu), order="F") for w in wss]
    vT = [np.zeros((w.N, w.N, w.nv, w.nv), order="F") for w in wss]
    h = (ctypes.c_void_p * n)(*[w._h for w in wss])
    rc = L.lib().wedg_rk4_adjoint_forward_many(n, h, _ptr_array(u0s), _ptr_array(v0s), float(t0), float(dt),
                                               int(nsteps), int(every), _ptr_array(uT), _ptr_array(vT), L.WEDG_HOST)
    _check_group(wss, rc)
    return uT, vT


def rk4_adjoint_reverse_many(wss, lam_us, lam_vs, params=False):
    """wedg_rk4_adjoint_reverse_many: the reverse sweeps of the workspaces' last forward runs
    (rk4_adjoint_forward_many) for the final-time adjoints (λ_u, λ_v) of each; returns per workspace
    (gu, gv) and, with params, the per-element gradients with respect to c², α, β."""
    n = len(wss)
    lam_us = [_f64(a) for a in lam_us]
    lam_vs = [_f64(a) for a in lam_vs]
    gu = [np.zeros((w.N, w.N, w.nu, w.nu), order="F") for w in wss]
    gv = [np.zeros((w.N, w.N, w.nv, w.nv), order="F") for w in wss]
    gp = [[np.zeros((w.N, w.N), order="F") for w in wss] for _ in range(3)] if params else None
    null = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))()
    pc = [_ptr_array(g) for g in gp] if params else [null, null, null]
    h = (ctypes.c_void_p * n)(*[w._h for w in wss])
    rc = L.lib().wedg_rk4_adjoint_reverse_many(n, h, _ptr_array(lam_us), _ptr_array(lam_vs), _ptr_array(gu),
                                               _ptr_array(gv), pc[0], pc[1], pc[2], L.WEDG_HOST)
    _check_group(wss, rc)
    if params:
        return [(gu[i], gv[i], gp[0][i], gp[1][i], gp[2][i]) for i in range(n)]
    return [(gu[i], gv[i]) for i in range(n)]


def edg_rhs_(ws, u, v, t, N, h, pre):
    """``edg_rhs!(ws, u, v, t, N, h, pre) -> (ws.ut, ws.vt)`` (src/rhs.jl:490-494); the
    returned arrays are overwritten by the next call."""
    if ws.pre is not pre and (N != ws.N or pre["qu1"] != ws.nu or pre["qv1"] != ws.nv):
        raise DimensionMismatch(f"state, workspace and pre do not match (N = {N}, q_u + 1 = {pre['qu1']}, "
                                f"q_v + 1 = {pre['qv1']})")
    if N != ws.N:
        raise DimensionMismatch(f"state, workspace and pre do not match (N = {N}, q_u + 1 = {ws.nu}, "
                                f"q_v + 1 = {ws.nv})")
    return ws.rhs(u, v, t)


def edg_rhs(u, v, t, N, h, pre, nblocks=None):
    """Allocating ``edg_rhs`` (src/rhs.jl:560-571): copies of the right-hand side."""
    ws = Workspace(pre, N, nblocks=nblocks)
    ut, vt = edg_rhs_(ws, u, v, t, N, h, pre)
    return ut.copy(order="F"), vt.copy(order="F")


def rk4_step_(u, v, t, dt, N, h, pre, ws):
    """``rk4_step!(u, v, t, dt, N, h, pre, ws) -> (u, v)`` in place (src/solver.jl:289-297);
    afterwards ``ws.fin`` tells whether all entries are finite."""
    if N != ws.N:
        raise DimensionMismatch(f"state, workspace and pre do not match (N = {N}, q_u + 1 = {ws.nu}, "
                                f"q_v + 1 = {ws.nv})")
    ws.rk4_steps(u, v, t, dt, 1)
    return u, v


def rk4_step(u, v, t, dt, N, h, pre, nblocks=None):
    """Allocating ``rk4_step`` (src/solver.jl:331-339): u, v are not modified."""
    ws = Workspace(pre, N, nblocks=nblocks)
    u2 = np.array(u, dtype=np.float64, order="F", copy=True)
    v2 = np.array(v, dtype=np.float64, order="F", copy=True)
    return rk4_step_(u2, v2, t, dt, N, h, pre, ws)
