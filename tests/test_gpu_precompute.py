"""pre built on the device (wedg_create_points): the workspace forms the element matrices, the
one-sided face arrays and jump terms, the projections and 2β from the coefficient functions'
values at the point grids (precompute(..., target="device")). Each device array, read back in
the reference's layout (wedg_export), is checked against the oracle's restatement of precompute
(src/solver.jl:428-770): to 1e-14 of the array's size. The coefficient functions are evaluated by
numpy on the device's point grid, a 4-D broadcast whose vectorised sin, cos and exp may round in
the last place unlike the oracle's evaluation on its own grid; per-cell tables give c² and α per
element directly where the oracle divides c²W by W; the projections are sums in another order.
Then the one-sided choice, the refusal of jumping coefficients in :mms mode, and the RHS of such a
workspace against the oracle's RHS."""
import ctypes
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from conftest import rel_max
from edg_westervelt_gb300 import _lib as L
from oracle import coefficients as oc
from oracle.precompute import precompute as opre
from oracle.rhs import OracleWorkspace
from test_oracle import quadrant_coefficients

pytestmark = pytest.mark.gpu

FACES = ("hc2", "haf", "hcf", "hbf", "hc2m", "hafm", "hJC", "vc2", "vaf", "vcf", "vbf", "vc2m", "vafm", "vJC")


def _export(ws, name, shape):
    out = np.zeros(shape, order="F")
    rc = L.lib().wedg_export(ws._h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size)
    assert rc == L.WEDG_OK, name
    return out


def _gauss_profile():
    def g(d):
        def f(x, y):
            X, Y = np.asarray(x, dtype=float) - 0.45, np.asarray(y, dtype=float) - 0.5
            gv = np.exp(-(X * X + Y * Y) / 0.02)
            return {"": gv, "x": -2 * X / 0.02 * gv, "y": -2 * Y / 0.02 * gv,
                    "xx": (4 * X * X / 0.02 ** 2 - 2 / 0.02) * gv, "yy": (4 * Y * Y / 0.02 ** 2 - 2 / 0.02) * gv}[d]
        return f
    return dict(u0=g(""), u0_x=g("x"), u0_y=g("y"), u0_xx=g("xx"), u0_yy=g("yy"))


CASES = {
    # jumping coefficients, one-sided faces, every side kind; the source projection
    "source, jumps": (3, 6, dict(mode="source", mixed=True, coefficients=quadrant_coefficients(0.5, 0.5, smooth=False),
                                 boundary=dict(bot="absorbing_2beta", top="wall", lft="dirichlet", rgt="absorbing"),
                                 kappa=0.5, flux="alternating")),
    # initial data whose derivative enters the jump terms JC; jumping coefficients
    "initial value, jumps": (4, 5, dict(mode="initial_value", mixed=False,
                                        coefficients=quadrant_coefficients(0.4, 0.6, smooth=False),
                                        initial_profile=_gauss_profile(), flux="central",
                                        boundary=dict(bot="dirichlet", top="absorbing", lft="absorbing_2beta",
                                                      rgt="wall"), kappa=0.5)),
    # the manufactured solution with the paper coefficients: the general kernels, all four projections
    "mms, paper": (3, 5, dict(mode="mms", mixed=True, flux="upwind", phase=(0.4, 0.3))),
    # constant coefficients, passed as their values: the constant-coefficient kernels
    "source, constant": (6, 4, dict(mode="source", mixed=False, coefficients=None, flux="alternating",
                                    boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"),
                                    kappa=0.5)),
    # tables of cells, looked up on the device (faces on cell boundaries: one-sided)
    "source, cell tables": (4, 8, dict(mode="source", mixed=True, flux="upwind", kappa=0.5,
                                       coefficients=W.cell_coefficients(np.array([[1.0, 0.7], [1.3, 0.9]]),
                                                                        np.array([[1e-4, 3e-4], [2e-4, 1e-5]]),
                                                                        np.array([[0.5, 2.0], [1.0, 3.0]])),
                                       boundary=dict(bot="absorbing", top="absorbing_2beta", lft="wall",
                                                     rgt="dirichlet"))),
    "initial value, cell tables": (3, 6, dict(mode="initial_value", mixed=False, flux="alternating", kappa=0.5,
                                              coefficients=W.cell_coefficients(np.array([[1.0, 0.6, 1.2]]),
                                                                               np.array([[1e-4, 2e-4, 5e-5]]),
                                                                               np.array([[0.1, 0.2, 0.05]])),
                                              initial_profile=_gauss_profile())),
}


@pytest.mark.parametrize("case", list(CASES))
def test_device_built_pre_against_the_oracle(gpu, case):
    q, N, kw = CASES[case]
    kw = dict(kw)
    if kw.get("coefficients", 0) is None:
        kw_w = dict(kw, coefficients=W.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0))
        kw_o = dict(kw, coefficients=oc.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0))
    else:
        kw_w = kw_o = kw
    po, _ = opre(q, N, **kw_o)
    pd, _ = W.precompute(q, N, target="device", **kw_w)
    assert "points" in pd and "hc2" not in pd
    ws = W.Workspace(pd, N)
    assert ws.one_sided == bool(po["one_sided"])
    nq, nv, qh, E = po["qu1"], po["qv1"], po["q_high"], N * N
    def close(name, got, ref):
        err = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)
        assert err <= 1e-14, (name, err)

    for name in FACES:
        shape = (nq, N + 1, N) if name[0] == "h" else (nq, N, N + 1)
        close(name, _export(ws, name, shape), po[name])
    close("beta_hq", _export(ws, "beta_hq", (qh, E, qh)), po["beta_hq"])
    names = ["src_projE"] if kw["mode"] == "source" else ["PiCdiv"] + (
        ["PiSP", "PiBSP2", "PiDdiv"] if kw["mode"] == "mms" else [])
    for name in names:
        close(name, _export(ws, name, (nv, nv, N, N)), po[name])
    if ws.stats()["fast_path"]:
        w00 = po["w"][0] ** 2
        close("c2e", _export(ws, "c2e", (E,)), po["Cw"][0, :, 0] / w00)
        close("ae", _export(ws, "ae", (E,)), po["Aw"][0, :, 0] / w00)
    else:
        close("Cw", _export(ws, "Cw", (nq, E, nq)), po["Cw"])
        close("Aw", _export(ws, "Aw", (nq, E, nq)), po["Aw"])
    # the workspace's RHS against the oracle's
    rng = np.random.default_rng(71)
    u = np.asfortranarray(0.1 * rng.standard_normal((N, N, nq, nq)))
    v = np.asfortranarray(1e-3 * rng.standard_normal((N, N, nv, nv)))
    assert rel_max(OracleWorkspace(po).rhs(u, v, 0.037), ws.rhs(u, v, 0.037)) < 1e-12


def test_device_built_pre_refuses_jumps_in_mms_mode(gpu):
    """src/solver.jl:745-747: the manufactured solution needs c and α continuous across faces."""
    pd, _ = W.precompute(2, 4, target="device", mode="mms", coefficients=quadrant_coefficients(0.5, 0.5, smooth=False))
    with pytest.raises(W.ErrorException, match="mode = :mms needs c and α continuous"):
        W.Workspace(pd, 4)


def test_device_built_pre_runs_like_the_host_built_one(gpu):
    """Twenty RK4 steps of the bench's headline configuration on a small mesh, the workspace built
    from point values against the one built from the host's pre: the same states to rounding."""
    import bench
    N = 12
    kw = dict(bench.KW, coefficients=W.constant_coefficients(**bench.COEF))
    ph, _ = W.precompute(bench.Q, N, **kw)
    pd, _ = W.precompute(bench.Q, N, target="device", **kw)
    u, v = bench.synthetic_state(N, ph["qu1"], ph["qv1"], 0, "front")
    dt = (1.0 / N) / (10 * bench.Q ** 2)
    out = []
    for pre in (ph, pd):
        uu, vv = u.copy(order="F"), v.copy(order="F")
        assert W.Workspace(pre, N).rk4_steps(uu, vv, bench.T0, dt, 20) == 20
        out.append((uu, vv))
    assert rel_max(out[0], out[1]) < 1e-13
