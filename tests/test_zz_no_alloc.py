"""wedg_rhs_noalloc: the right-hand side for callers that cannot let a library allocate.

Programs whose GPU memory belongs to another runtime's pool allocator, or code that
must not allocate or free device memory where it needs a right-hand side, cannot
create a workspace. wedg_rhs_noalloc needs none: it keeps its device scratch in a
fixed static array of the library. These tests call it through the C ABI twice in
a row on different states and compare it with the workspace entry point wedg_rhs
on the same inputs (max-norm relative 1e-12, the bar of the other GPU tests), and
check that a mesh too large for the static array is refused with a message, and that
its errors (a boundary weight and a mass matrix that is not positive definite, for
both mass solvers) carry the status and the message that wedg_rhs gives.
This file is collected last, so a failure here comes after every other test ran.
"""
import ctypes

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from edg_westervelt_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _abi_structs(pre, N):
    """wedg_config and wedg_pre for `pre` (the same fields wedg_create reads)."""
    cfg = L.Config()
    cfg.N, cfg.qu1, cfg.qv1, cfg.q_high = N, pre["qu1"], pre["qv1"], pre["q_high"]
    cfg.theta, cfg.tau, cfg.lambda_u, cfg.lambda_v = pre["theta"], pre["tau"], pre["lambda_u"], pre["lambda_v"]
    cfg.omega = pre["omega"]
    cfg.mms_on, cfg.src_on, cfg.one_sided = int(pre["mms_on"]), int(pre["src_on"]), int(pre["one_sided"])
    cfg.mass_solver = 0 if pre["mass_solver"] == "chebyshev" else 1
    cfg.mass_tol = pre["mass_tol"]
    cfg.src_omega, cfg.src_Ts = pre["source"].omega, pre["source"].Ts
    for i, side in enumerate(("bot", "top", "lft", "rgt")):
        bs = pre["bc"][side]
        cfg.kind[i] = L.KINDS[bs["kind"]]
        cfg.gamma_abc[i], cfg.eta_abc[i], cfg.sigma[i] = bs["gamma_abc"], bs["eta_abc"], bs["sigma"]
        cfg.kb[i], cfg.kappa[i] = bs["kb"], bs["kappa"]
    p = L.Pre()
    keep = []
    for name in L.PRE_FIELDS:
        a = np.require(np.ascontiguousarray(pre[name]) if not pre[name].flags.f_contiguous else pre[name],
                       dtype=np.float64, requirements=["F_CONTIGUOUS", "ALIGNED"])
        keep.append(a)
        setattr(p, name, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return cfg, p, keep


def _rel(a, b):
    return max(float(np.max(np.abs(a[0] - b[0])) / np.max(np.abs(a[0]))),
               float(np.max(np.abs(a[1] - b[1])) / np.max(np.abs(a[1]))))


CASES = {
    "general kernels, mms": (3, 6, dict(flux="upwind", mixed=True)),
    "constant-coefficient kernels, source": (
        6, 8, dict(mixed=False, mode="source", kappa=0.5, flux="alternating",
                   coefficients=W.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0),
                   boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))),
    "CG mass solver, mixed sides": (
        4, 5, dict(mixed=True, mode="initial_value", flux="central", mass_solver="cg", kappa=0.5,
                   boundary=dict(bot="dirichlet", top="absorbing", lft="absorbing_2beta", rgt="wall"))),
}


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_workspace_twice(case):
    """Calls in a row on different states, alternating between the default stream and a stream of
    the caller's; from the second call on, device memory stays as it is."""
    import torch
    assert torch.cuda.is_available()
    q, N, kw = CASES[case]
    side = torch.cuda.Stream(device=torch.device("cuda:0"))
    pre, _ = W.precompute(q, N, inverses="host", **kw)     # wedg_rhs_noalloc reads Ainv_u from pre
    nu, nv = pre["qu1"], pre["qv1"]
    cfg, p, keep = _abi_structs(pre, N)
    ws = W.Workspace(pre, N)
    dev = torch.device("cuda:0")
    lib = L.lib()
    rng = np.random.default_rng(42)
    free_before = None
    for call in range(4):
        u = np.asfortranarray(rng.standard_normal((N, N, nu, nu)))
        v = np.asfortranarray(1e-4 * rng.standard_normal((N, N, nv, nv)))
        t = 0.037 + 0.1 * call
        ref = tuple(x.copy() for x in ws.rhs(u, v, t))            # wedg_rhs, the workspace entry point
        du = torch.from_numpy(u.reshape(-1, order="F").copy()).to(dev)
        dv = torch.from_numpy(v.reshape(-1, order="F").copy()).to(dev)
        ut = torch.full_like(du, float("nan"))
        vt = torch.full_like(dv, float("nan"))
        torch.cuda.synchronize()
        msg = ctypes.create_string_buffer(512)
        stream = side.cuda_stream if call % 2 else None
        rc = lib.wedg_rhs_noalloc(ctypes.byref(cfg), ctypes.byref(p), du.data_ptr(), dv.data_ptr(), t,
                                  ut.data_ptr(), vt.data_ptr(), stream, msg, 512)
        assert rc == L.WEDG_OK, msg.value.decode()
        got = (ut.cpu().numpy().reshape((N, N, nu, nu), order="F"),
               vt.cpu().numpy().reshape((N, N, nv, nv), order="F"))
        assert _rel(ref, got) < 1e-12, (call, _rel(ref, got))
        torch.cuda.synchronize()
        if call == 1:
            # the static array is placed when the library's device code is loaded (at the latest
            # by the first call), and the first use of a stream may set up driver state of its own;
            # from then on the calls take no device memory
            free_before = torch.cuda.mem_get_info(dev)[0]
    assert abs(torch.cuda.mem_get_info(dev)[0] - free_before) < (1 << 20)
    del keep


def test_noalloc_refuses_a_mesh_beyond_the_static_array():
    N = 128
    pre, _ = W.precompute(6, N, **CASES["constant-coefficient kernels, source"][2])
    cfg, p, keep = _abi_structs(pre, N)
    import torch
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    msg = ctypes.create_string_buffer(512)
    rc = L.lib().wedg_rhs_noalloc(ctypes.byref(cfg), ctypes.byref(p), dummy.data_ptr(), dummy.data_ptr(), 0.0,
                                  dummy.data_ptr(), dummy.data_ptr(), None, msg, 512)
    assert rc == L.WEDG_ERR_ARGUMENT
    assert "mesh too large for wedg_rhs_noalloc" in msg.value.decode()
    del keep


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_noalloc_errors_match_workspace(solver):
    """A state whose boundary weight 1 - 2βv_h fails at a face point, and one whose mass matrix is
    not positive definite on two elements: the status and the message (the first failing point or
    element, in the reference's words) are those of wedg_rhs on the same inputs, and the static
    array serves a good call again afterwards."""
    import torch
    N = 8
    co = W.replace_coefficients(W.paper_coefficients(), alpha=1e-6, beta=1.0)
    bd = dict(bot="absorbing_2beta", top="absorbing", lft="absorbing", rgt="wall")
    pre, _ = W.precompute(3, N, coefficients=co, boundary=bd, mass_solver=solver, inverses="host")
    nu, nv = pre["qu1"], pre["qv1"]
    cfg, p, keep = _abi_structs(pre, N)
    ws = W.Workspace(pre, N)
    dev = torch.device("cuda:0")
    u = np.zeros((N, N, nu, nu), order="F")
    v_bnd = np.zeros((N, N, nv, nv), order="F")
    v_bnd[0, N - 1, 0, 0] = 2.5
    v_bnd[3, 0, 0, 0] = 2.5
    v_mass = np.zeros((N, N, nv, nv), order="F")
    v_mass[3, 5, 0, 0] = 2.5
    v_mass[4, 1, 0, 0] = 2.5
    du = torch.from_numpy(u.reshape(-1, order="F").copy()).to(dev)
    ut = torch.empty_like(du)
    for v, status in ((v_bnd, L.WEDG_ERR_BOUNDARY_WEIGHT), (v_mass, L.WEDG_ERR_MASS_NOT_PD)):
        with pytest.raises(W.ErrorException) as ei:
            ws.rhs(u, v, 0.0)
        dv = torch.from_numpy(v.reshape(-1, order="F").copy()).to(dev)
        vt = torch.empty_like(dv)
        msg = ctypes.create_string_buffer(512)
        rc = L.lib().wedg_rhs_noalloc(ctypes.byref(cfg), ctypes.byref(p), du.data_ptr(), dv.data_ptr(), 0.0,
                                      ut.data_ptr(), vt.data_ptr(), None, msg, 512)
        assert rc == status
        assert msg.value.decode() == str(ei.value)
    # a good state after the errors: the error word starts clear again
    rng = np.random.default_rng(5)
    u = np.asfortranarray(0.1 * rng.standard_normal((N, N, nu, nu)))
    v = np.asfortranarray(1e-3 * rng.standard_normal((N, N, nv, nv)))
    du = torch.from_numpy(u.reshape(-1, order="F").copy()).to(dev)
    dv = torch.from_numpy(v.reshape(-1, order="F").copy()).to(dev)
    vt = torch.empty_like(dv)
    msg = ctypes.create_string_buffer(512)
    rc = L.lib().wedg_rhs_noalloc(ctypes.byref(cfg), ctypes.byref(p), du.data_ptr(), dv.data_ptr(), 0.0,
                                  ut.data_ptr(), vt.data_ptr(), None, msg, 512)
    assert rc == L.WEDG_OK, msg.value.decode()
    ref = ws.rhs(u, v, 0.0)
    got = (ut.cpu().numpy().reshape((N, N, nu, nu), order="F"), vt.cpu().numpy().reshape((N, N, nv, nv), order="F"))
    assert _rel(ref, got) < 1e-12
    del keep
