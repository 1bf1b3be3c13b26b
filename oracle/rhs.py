"""ctypes binding of the C oracle (rhs_oracle.c). Test infrastructure only.

``OracleWorkspace(pre)`` owns the C workspace; ``rhs``, ``rk4_step`` and
``rk4_steps`` mirror ``edg_rhs!`` / ``rk4_step!`` of src/rhs.jl and
src/solver.jl, raising the reference's error messages
(src/rhs.jl:112-116, 768-776, 845, 916).
"""
import ctypes
import math
import os
import subprocess
import warnings

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "liboracle.so")
KINDS = {"absorbing_2beta": 0, "absorbing": 1, "dirichlet": 2, "wall": 3}

_D = ctypes.POINTER(ctypes.c_double)


class _Pre(ctypes.Structure):
    _fields_ = ([("N", ctypes.c_int), ("nu", ctypes.c_int), ("nv", ctypes.c_int), ("qh", ctypes.c_int)]
                + [(n, ctypes.c_double) for n in ("theta", "tau", "lu", "lv", "omega")]
                + [(n, ctypes.c_int) for n in ("mms_on", "src_on", "one_sided", "cheb")]
                + [(n, ctypes.c_double) for n in ("mass_tol", "src_omega", "src_Ts")]
                + [("kind", ctypes.c_int * 4)]
                + [(n, ctypes.c_double * 4) for n in ("gam", "eta", "sig", "kb", "kap")]
                + [(n, _D) for n in ("w", "P_u", "S_u", "Ebl_u", "Ebr_u", "E1bl_u", "E1br_u", "P_h", "W_h",
                                      "Cw", "Aw", "Ainv", "hc2", "haf", "hcf", "hbf", "vc2", "vaf", "vcf", "vbf",
                                      "hc2m", "hafm", "vc2m", "vafm", "hJC", "vJC",
                                      "bcB_sp", "bcB_spy", "bcT_sp", "bcT_spy", "bcL_sp", "bcL_spx",
                                      "bcR_sp", "bcR_spx", "PiSP", "PiBSP2", "PiCdiv", "PiDdiv", "src_projE",
                                      "beta_hq", "beta_hE")])


def build(force=False):
    """Compile rhs_oracle.c into oracle/_build/liboracle.so (gcc + OpenMP)."""
    src = os.path.join(_HERE, "rhs_oracle.c")
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(src):
        return _LIB
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-o", tmp, src, "-lm"])
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [ctypes.POINTER(_Pre)]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_rhs.argtypes = [ctypes.c_void_p, _D, _D, ctypes.c_double, _D, _D, ctypes.POINTER(ctypes.c_long)]
        L.or_rk4_step.argtypes = [ctypes.c_void_p, _D, _D, ctypes.c_double, ctypes.c_double,
                                  ctypes.POINTER(ctypes.c_long)]
        L.or_rk4_steps.argtypes = [ctypes.c_void_p, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_long,
                                   ctypes.POINTER(ctypes.c_long)]
        L.or_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_D)


def _f(a):
    return np.require(a, dtype=np.float64, requirements=["F_CONTIGUOUS", "ALIGNED"])


def weight_error_message(bs, check):
    """src/rhs.jl:112-116."""
    k = "2" if bs["kb"] == 2.0 else ""
    if check == 1:
        return f"boundary weight 1 - {k}βv_h ≤ 0 at a face point ({bs['kind']} side)"
    return f"boundary weight 1 - {k}βg ≤ 0 for the boundary data g ({bs['kind']} side)"


class OracleWorkspace:
    """The oracle's counterpart of ``Workspace(pre, N)`` (one block; OpenMP inside)."""

    def __init__(self, pre):
        self.pre = pre
        N = pre["N"]
        self.N = N
        keep = {}

        def arr(name, a=None):
            a = _f(pre[name] if a is None else a)
            keep[name] = a
            return _ptr(a)

        s = _Pre()
        s.N, s.nu, s.nv, s.qh = N, pre["qu1"], pre["qv1"], pre["q_high"]
        s.theta, s.tau, s.lu, s.lv = pre["theta"], pre["tau"], pre["lambda_u"], pre["lambda_v"]
        s.omega = pre["omega"]
        s.mms_on, s.src_on, s.one_sided = int(pre["mms_on"]), int(pre["src_on"]), int(pre["one_sided"])
        s.cheb = int(pre["mass_solver"] == "chebyshev")
        s.mass_tol = pre["mass_tol"]
        s.src_omega, s.src_Ts = pre["source"].omega, pre["source"].Ts
        for i, side in enumerate(("bot", "top", "lft", "rgt")):
            bs = pre["bc"][side]
            s.kind[i] = KINDS[bs["kind"]]
            s.gam[i], s.eta[i], s.sig[i], s.kb[i], s.kap[i] = (bs["gamma_abc"], bs["eta_abc"], bs["sigma"],
                                                               bs["kb"], bs["kappa"])
        s.w = arr("w")
        s.P_u, s.S_u = arr("P_u"), arr("S_u")
        s.Ebl_u, s.Ebr_u, s.E1bl_u, s.E1br_u = arr("Ebl_u"), arr("Ebr_u"), arr("E1bl_u"), arr("E1br_u")
        s.P_h, s.W_h = arr("P_h_v"), arr("W2d_h")
        for n in ("Cw", "Aw", "hc2", "haf", "hcf", "hbf", "vc2", "vaf", "vcf", "vbf", "hc2m", "hafm", "vc2m",
                  "vafm", "hJC", "vJC", "bcB_sp", "bcB_spy", "bcT_sp", "bcT_spy", "bcL_sp", "bcL_spx", "bcR_sp",
                  "bcR_spx", "PiSP", "PiBSP2", "PiCdiv", "PiDdiv", "src_projE", "beta_hq", "beta_hE"):
            setattr(s, n, arr(n))
        s.Ainv = arr("Ainv_u")
        self._keep = keep
        self._s = s
        self._ws = lib().or_create(ctypes.byref(s))
        nu, nv = pre["qu1"], pre["qv1"]
        self.ut = np.zeros((N, N, nu, nu), order="F")
        self.vt = np.zeros((N, N, nv, nv), order="F")
        self.nsteps = 0
        self.nfail = 0
        self.fin = True

    def __del__(self):
        if getattr(self, "_ws", None):
            lib().or_destroy(self._ws)
            self._ws = None

    def _raise(self, rc, info):
        pre = self.pre
        N = self.N
        if rc == 2:
            key = int(info[0])
            s = (key - 1) // (2 * pre["qu1"] * N)
            side = ("bot", "top", "lft", "rgt")[s]
            raise RuntimeError(weight_error_message(pre["bc"][side], 1 if key % 2 == 1 else 2))
        if rc == 3:
            e = int(info[0])
            if pre["mass_solver"] == "chebyshev":
                raise RuntimeError(f"mass matrix not positive definite on element {e}: 1 - 2βv_h ≤ 0")
            j = (e - 1) % N + 1
            k = (e - 1) // N + 1
            raise RuntimeError(f"mass matrix not positive definite on element ({j}, {k}): 1 - 2βv_h ≤ 0")
        raise RuntimeError(f"oracle error {rc}")

    def _cg_report(self, nfail):
        if nfail > 0 and self.pre["mass_solver"] == "cg":
            warnings.warn(f"mass solve: {nfail} element systems did not reach the tolerance {self.pre['mass_tol']}")

    def rhs(self, u, v, t):
        """edg_rhs!: returns (ut, vt), arrays owned by the workspace."""
        u = _f(u)
        v = _f(v)
        self._check(u, v)
        info = (ctypes.c_long * 5)()
        rc = lib().or_rhs(self._ws, _ptr(u), _ptr(v), float(t), _ptr(self.ut), _ptr(self.vt), info)
        if rc:
            self._raise(rc, info)
        self.nsteps = int(info[1])
        self._cg_report(int(info[2]))
        return self.ut, self.vt

    def _check(self, u, v):
        N, nu, nv = self.N, self.pre["qu1"], self.pre["qv1"]
        if u.shape != (N, N, nu, nu) or v.shape != (N, N, nv, nv):
            raise ValueError(f"state, workspace and pre do not match (N = {N}, q_u + 1 = {nu}, q_v + 1 = {nv})")

    def rk4_step(self, u, v, t, dt):
        """rk4_step!: u, v (Fortran float64 arrays) are updated in place."""
        self._check(u, v)
        assert u.flags.f_contiguous and v.flags.f_contiguous
        info = (ctypes.c_long * 5)()
        rc = lib().or_rk4_step(self._ws, _ptr(u), _ptr(v), float(t), float(dt), info)
        if rc:
            self._raise(rc, info)
        self.nsteps = int(info[1])
        self.fin = bool(info[3])
        self._cg_report(int(info[2]))
        return u, v

    def rk4_steps(self, u, v, t0, dt, n):
        """n RK4 steps from t0 (t advances by repeated addition of dt, as solve does)."""
        self._check(u, v)
        info = (ctypes.c_long * 5)()
        rc = lib().or_rk4_steps(self._ws, _ptr(u), _ptr(v), float(t0), float(dt), int(n), info)
        if rc:
            self._raise(rc, info)
        self.fin = bool(info[3]) if n > 0 else True
        return u, v


def edg_rhs(u, v, t, N, h, pre):
    """Allocating edg_rhs (src/rhs.jl:560-571)."""
    ws = OracleWorkspace(pre)
    ut, vt = ws.rhs(u, v, t)
    return ut.copy(order="F"), vt.copy(order="F")


def max_threads():
    return int(lib().or_max_threads())


def stage_src_time(pre, t):
    s = pre["source"]
    if pre["src_on"] and t < s.Ts:
        return math.sin(s.omega * t) * math.sin(math.pi * t / s.Ts) ** 2
    return 0.0
