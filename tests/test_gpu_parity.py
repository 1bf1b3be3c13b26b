"""GPU parity: libwedg (through the C ABI) against the oracle on the same inputs.

The grid is the reference's own differential test grid (test/runtests.jl:189-293,
716-732): every mode, every boundary kind, q ∈ {1, 3, 4}, N ∈ {1, 2, 4}, three
fluxes, both pairings, seeded random states; the bar is the reference's,
max-norm relative < 1e-12 for the RHS. The product computes its own ``pre``
(edg_westervelt_gb300.precompute), the oracle its own (oracle/precompute.py).
"""
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from conftest import rel_max
from oracle import coefficients as oc
from oracle.precompute import precompute as opre
from oracle.rhs import OracleWorkspace
from test_oracle import quadrant_coefficients

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _state(rng, pre, N, su=1.0, sv=0.05):
    u = np.asfortranarray(su * rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
    v = np.asfortranarray(sv * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
    return u, v


def _pair(q, N, **kw):
    return W.precompute(q, N, **kw)[0], opre(q, N, **kw)[0]


@pytest.mark.parametrize("mode", ["mms", "initial_value", "source"])
@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_rhs_grid(gpu, mode, solver):
    rng = np.random.default_rng(2)
    worst = 0.0
    for boundary in ("absorbing", "dirichlet", "absorbing_2beta", "wall"):
        for q in (1, 3, 4):
            for N in (1, 2, 4):
                for flux in ("upwind", "central", "alternating"):
                    for mixed in (True, False):
                        kw = dict(flux=flux, mixed=mixed, mode=mode, boundary=boundary, sigma=0.3,
                                  sigma_dirichlet=0.6, kappa=0.7, phase=(0.4, 0.3), mass_solver=solver)
                        pp, po = _pair(q, N, **kw)
                        u, v = _state(rng, pp, N)
                        a = OracleWorkspace(po).rhs(u, v, 0.037)
                        b = W.edg_rhs(u, v, 0.037, N, 1.0 / N, pp)
                        worst = max(worst, rel_max(a, b))
    assert worst < TOL, worst


def test_rhs_mixed_kinds_lambda_and_piecewise(gpu):
    """Per-side kinds, λ_u ≠ λ_v (test/runtests.jl:281-293) and jumping coefficients with the
    one-sided face kernel (test/runtests.jl:716-732)."""
    rng = np.random.default_rng(3)
    worst = 0.0
    mixed_b = (dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing"),
               dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"))
    fp = dict(theta=1.0, tau=0.4, lambda_u=0.7, lambda_v=0.2)
    for q in (1, 3, 5):
        for N in (2, 3, 4):
            for mixed in (True, False):
                for mode in ("mms", "source", "initial_value"):
                    for bd in mixed_b:
                        pp, po = _pair(q, N, flux_params=fp, mixed=mixed, mode=mode, boundary=bd, sigma=0.3,
                                       sigma_dirichlet=0.6, kappa=0.7, phase=(0.4, 0.3))
                        u, v = _state(rng, pp, N)
                        worst = max(worst, rel_max(OracleWorkspace(po).rhs(u, v, 0.037),
                                                   W.edg_rhs(u, v, 0.037, N, 1.0 / N, pp)))
    co = quadrant_coefficients(0.5, 0.5, smooth=True)
    fps = (oc.flux_parameters("upwind"), oc.flux_parameters("central"), oc.flux_parameters("alternating"),
           dict(theta=0.3, tau=0.7, lambda_u=0.4, lambda_v=0.9))
    for mode in ("initial_value", "source"):
        for q in (1, 3):
            for N in (2, 4):
                for boundary in ("absorbing_2beta", "dirichlet", "wall"):
                    for f in fps:
                        pp, po = _pair(q, N, flux_params=f, mode=mode, boundary=boundary, coefficients=co,
                                       sigma=0.3, sigma_dirichlet=0.6, kappa=0.7, phase=(0.4, 0.3))
                        assert pp["one_sided"]
                        u, v = _state(rng, pp, N)
                        worst = max(worst, rel_max(OracleWorkspace(po).rhs(u, v, 0.037),
                                                   W.edg_rhs(u, v, 0.037, N, 1.0 / N, pp)))
    assert worst < TOL, worst


@pytest.mark.parametrize("q", [1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("mixed", [True, False])
def test_every_degree_fast_and_general(gpu, q, mixed):
    """Every compiled (q_u, q_v): the constant-coefficient kernels and the stored-inverse
    kernels both against the oracle, N = 5 (odd, every kind of side)."""
    rng = np.random.default_rng(10 + q)
    N = 5
    co = oc.constant_coefficients(c=1.3, alpha=2e-3, beta=0.5)
    kw = dict(mixed=mixed, mode="source", coefficients=co, flux="upwind",
              boundary=dict(bot="absorbing_2beta", top="wall", lft="dirichlet", rgt="absorbing"), kappa=0.5)
    pp, po = _pair(q, N, **kw)
    u, v = _state(rng, pp, N, 1.0, 0.02)
    a = OracleWorkspace(po).rhs(u, v, 0.21)
    ws_fast = W.Workspace(pp, N)
    assert ws_fast.stats()["fast_path"] == 1
    b = tuple(x.copy() for x in ws_fast.rhs(u, v, 0.21))
    ws_gen = W.Workspace(pp, N, fast_path=False)
    assert ws_gen.stats()["fast_path"] == 0
    c = tuple(x.copy() for x in ws_gen.rhs(u, v, 0.21))
    assert rel_max(a, b) < TOL and rel_max(a, c) < TOL, (rel_max(a, b), rel_max(a, c))
    # paper coefficients: general kernels only
    pp, po = _pair(q, N, mixed=mixed, mode="mms", phase=(0.4, 0.3))
    u, v = _state(rng, pp, N)
    ws = W.Workspace(pp, N)
    assert ws.stats()["fast_path"] == 0
    assert rel_max(OracleWorkspace(po).rhs(u, v, 0.037), ws.rhs(u, v, 0.037)) < TOL


def test_chebyshev_step_policies_and_cg(gpu):
    """Large β v: per-element and common step counts both meet the tolerance; CG agrees
    (test/runtests.jl:418-457, 503-519)."""
    rng = np.random.default_rng(5)
    N = 9
    co = oc.replace_coefficients(oc.paper_coefficients(), beta=8.0)
    pp, po = _pair(4, N, coefficients=co, mode="source")
    # u small enough that c²Δu does not push 2βv past 1 within the three steps (β = 8)
    u = np.asfortranarray(1e-4 * rng.standard_normal((N, N, pp["qu1"], pp["qu1"])))
    v = np.asfortranarray(1e-4 * rng.standard_normal((N, N, pp["qv1"], pp["qv1"])))
    v[:, 0:2, 1, 0] = 0.04
    ow = OracleWorkspace(po)
    a = tuple(x.copy() for x in ow.rhs(u, v, 0.1))
    assert ow.nsteps > 20
    for policy in ("per_element", "common_max"):
        ws = W.Workspace(pp, N, cheb_steps=policy)
        b = ws.rhs(u, v, 0.1)
        assert rel_max(a, b) < TOL, policy
        assert ws.stats()["cheb_steps_max"] == ow.nsteps
    pc, _ = _pair(4, N, coefficients=co, mode="source", mass_solver="cg")
    assert rel_max(a, W.Workspace(pc, N).rhs(u, v, 0.1)) < TOL


def test_mass_solve_zero_state_exact(gpu):
    """v_h = 0: M = I and one Chebyshev step, so vt equals the right-hand side of the mass
    system exactly (test/runtests.jl:441)."""
    N = 3
    pp, po = _pair(3, N, mode="source")
    u = np.asfortranarray(np.random.default_rng(1).standard_normal((N, N, pp["qu1"], pp["qu1"])))
    v = np.zeros((N, N, pp["qv1"], pp["qv1"]), order="F")
    ws = W.Workspace(pp, N, cheb_steps="common_max")
    ws.rhs(u, v, 0.3)
    assert ws.stats()["cheb_steps_max"] == 1


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_rk4_steps_match_oracle(gpu, solver):
    """Two RK4 steps (test/runtests.jl:481-495) against the oracle's, several configurations."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for q, N, su, sv, kw in ((1, 7, 1e-2, 0.05, dict(mixed=False)), (2, 7, 1e-2, 0.05, dict(mode="initial_value")),
                             (3, 7, 1e-2, 0.05, dict(mode="source")),
                             (6, 4, 1e-5, 3e-4, dict(mode="source", mixed=False,
                                            coefficients=oc.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0),
                                            boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"),
                                            kappa=0.5, flux="alternating"))):
        pp, po = _pair(q, N, mass_solver=solver, sigma=0.3, sigma_dirichlet=0.6, phase=(0.4, 0.3), **kw)
        u, v = _state(rng, pp, N, su, sv)
        uo, vo = u.copy(order="F"), v.copy(order="F")
        ug, vg = u.copy(order="F"), v.copy(order="F")
        ow, ws = OracleWorkspace(po), W.Workspace(pp, N)
        for k in (1, 2):
            ow.rk4_step(uo, vo, 0.01 * k, 1e-4)
            W.rk4_step_(ug, vg, 0.01 * k, 1e-4, N, 1.0 / N, pp, ws)
        assert ws.fin
        worst = max(worst, rel_max((uo, vo), (ug, vg)))
    assert worst < TOL, worst


def test_initialization(gpu):
    """Zero state solves the initialization system (test/runtests.jl:168-184, 340-357)."""
    N = 4
    for boundary in ("absorbing_2beta", "dirichlet", "wall",
                     dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing")):
        for flux in ("upwind", "central", "alternating"):
            for mixed in (True, False):
                pre, _ = W.precompute(3, N, flux=flux, mixed=mixed, boundary=boundary, sigma=0.3, kappa=0.5,
                                      phase=(0.4, 0.3))
                ut0, vt0 = W.edg_rhs(np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F"),
                                     np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F"), 0.0, N, 1.0 / N, pre)
                assert np.max(np.abs(ut0)) < 1e-12
                M = pre["Phi2d_h_v"].T @ (pre["W2d_h"].reshape(-1, order="F")[:, None] * pre["Phi2d_h_v"])
                r = s = 0.0
                for j in range(N):
                    for k in range(N):
                        b = pre["P_h_v"].T @ (pre["W2d_h"] * (-pre["omega"] ** 2 * pre["mms_SP"][j, k])) @ pre["P_h_v"]
                        proj = np.linalg.solve(M, b.reshape(-1, order="F")).reshape(pre["qv1"], pre["qv1"], order="F")
                        r = max(r, np.max(np.abs(vt0[j, k] - proj)))
                        s = max(s, np.max(np.abs(proj)))
                assert r / s < 1e-12


def test_kernel_reduction_one_sided(gpu):
    """The one-sided face kernel reduces to the continuous one (test/runtests.jl:702-710)."""
    rng = np.random.default_rng(5)
    bd = dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing")
    for flux in ("upwind", "central"):
        for mode in ("mms", "initial_value"):
            fp = dict(theta=0.3, tau=0.7, lambda_u=0.4, lambda_v=0.9) if flux == "upwind" else W.flux_parameters(flux)
            pre, _ = W.precompute(3, 4, flux_params=fp, mode=mode, boundary=bd, phase=(0.4, 0.3))
            u, v = _state(rng, pre, 4)
            a = W.edg_rhs(u, v, 0.037, 4, 0.25, pre)
            b = W.edg_rhs(u, v, 0.037, 4, 0.25, dict(pre, one_sided=True))
            assert rel_max(a, b) < 1e-14


def test_boundary_sides_are_local(gpu):
    """Changing one side's kind changes only the adjacent elements, and the changes
    superpose (test/runtests.jl:319-338)."""
    N = 4
    A4 = dict(bot="absorbing", top="absorbing", lft="absorbing", rgt="absorbing")
    S = dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="wall")
    rng = np.random.default_rng(9)

    def prep(bd):
        return W.precompute(3, N, boundary=bd, sigma=0.3, kappa=0.5, phase=(0.4, 0.3))[0]

    p0 = prep(A4)
    u, v = _state(rng, p0, N)

    def r(bd):
        return W.edg_rhs(u, v, 0.037, N, 1.0 / N, prep(bd))

    r0 = r(A4)
    su, sv = r0[0].copy(), r0[1].copy()
    adj = dict(bot=lambda j, k: j == 0, top=lambda j, k: j == N - 1, lft=lambda j, k: k == 0,
               rgt=lambda j, k: k == N - 1)
    for s in ("bot", "top", "lft", "rgt"):
        r1 = r(dict(A4, **{s: S[s]}))
        for j in range(N):
            for k in range(N):
                d = np.max(np.abs(r1[0][j, k] - r0[0][j, k])) + np.max(np.abs(r1[1][j, k] - r0[1][j, k]))
                assert (d > 0) if adj[s](j, k) else (d == 0), (s, j, k)
        su += r1[0] - r0[0]
        sv += r1[1] - r0[1]
    assert rel_max(r(S), (su, sv)) < 1e-12


def test_exact_consistency_at_interface(gpu):
    """c and α jump across a mesh line, walls, β = 0: piecewise quadratic profiles solving the
    transmission problem are reproduced to round-off (test/runtests.jl:790-811)."""
    c1, c2, a1, a2 = 1.0, 0.6, 0.02, 0.005

    def prof(k1, k2):
        B = -k1 / k2
        A = 0.25 * (1 - B)
        return (lambda s: s * s if s < 0.5 else A + B * (1 - s) ** 2), (lambda s: 2 * k1 if s < 0.5 else 2 * k2 * B)

    wu, du = prof(c1 ** 2, c2 ** 2)
    wv, dv = prof(a1, a2)
    worst = 0.0
    z0 = lambda x, y: 0.0   # noqa: E731
    for d in (1, 2):
        for q, N, mixed in ((2, 4, False), (3, 4, True), (3, 6, False), (4, 8, True)):
            for fp in (W.flux_parameters("upwind"), W.flux_parameters("central"), W.flux_parameters("alternating"),
                       dict(theta=0.0, tau=0.0, lambda_u=0.0, lambda_v=0.0),
                       dict(theta=0.3, tau=0.8, lambda_u=0.5, lambda_v=2.0)):
                def sel(x, y, d=d):
                    return x if d == 1 else y
                co = W.Coefficients(lambda x, y: c1 if sel(x, y) < 0.5 else c2, z0, z0,
                                    lambda x, y: a1 if sel(x, y) < 0.5 else a2, z0, z0, z0)
                pre, _ = W.precompute(q, N, mixed=mixed, flux_params=fp, boundary="wall", kappa=0.7, coefficients=co,
                                      mode="source", source=W.GaussianSource(amplitude=0.0))
                U = _project(lambda x, y: wu(sel(x, y)), pre, N, pre["P_u"])
                V = _project(lambda x, y: wv(sel(x, y)), pre, N, pre["P_v"])
                Ue = _project(lambda x, y: wv(sel(x, y)), pre, N, pre["P_u"])
                Ve = _project(lambda x, y: du(sel(x, y)) + dv(sel(x, y)), pre, N, pre["P_v"])
                ut, vt = W.edg_rhs(U, V, 0.3, N, 1.0 / N, pre)
                worst = max(worst, np.max(np.abs(ut - Ue)) / np.max(np.abs(Ue)),
                            np.max(np.abs(vt - Ve)) / np.max(np.abs(Ve)))
    assert worst < 1e-9, worst


def _project(f, pre, N, P):
    """L² projection on the element bases (test/runtests.jl:111-118)."""
    h = 1.0 / N
    z, w = W.GaussQCofs(pre["qu1"])
    n = P.shape[1]
    U = np.zeros((N, N, n, n), order="F")
    for k in range(N):
        xs = (k * h + (k + 1) * h + h * z) / 2
        for j in range(N):
            ys = (j * h + (j + 1) * h + h * z) / 2
            F = np.array([[f(x, y) for x in xs] for y in ys])
            U[j, k] = (P.T * w[None, :]) @ F @ (w[:, None] * P)
    return U


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_error_messages(gpu, solver):
    """Boundary weight before mass matrix, the first failing point / element, the reference's
    words (test/runtests.jl:548-577); a failing RK4 step leaves u, v unchanged."""
    N = 8
    co = W.replace_coefficients(W.paper_coefficients(), alpha=1e-6, beta=1.0)
    bd = dict(bot="absorbing_2beta", top="absorbing", lft="absorbing", rgt="wall")
    pre, _ = W.precompute(3, N, coefficients=co, boundary=bd, mass_solver=solver)
    u = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
    v = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
    v[0, N - 1, 0, 0] = 2.5
    v[3, 0, 0, 0] = 2.5
    ws = W.Workspace(pre, N)
    with pytest.raises(W.ErrorException) as ei:
        ws.rhs(u, v, 0.0)
    assert str(ei.value) == "boundary weight 1 - 2βv_h ≤ 0 at a face point (absorbing_2beta side)"
    w = np.zeros_like(v)
    w[3, 5, 0, 0] = 2.5
    w[4, 1, 0, 0] = 2.5
    msg = ("mass matrix not positive definite on element 13: 1 - 2βv_h ≤ 0" if solver == "chebyshev"
           else "mass matrix not positive definite on element (5, 2): 1 - 2βv_h ≤ 0")
    with pytest.raises(W.ErrorException) as ei:
        ws.rhs(u, w, 0.0)
    assert str(ei.value) == msg
    w0, u0 = w.copy(), u.copy()
    with pytest.raises(W.ErrorException):
        W.rk4_step_(u, w, 0.0, 1e-3, N, 1.0 / N, pre, ws)
    assert np.array_equal(w, w0) and np.array_equal(u, u0)
    # the workspace is still usable after an error
    ut, vt = ws.rhs(u, np.zeros_like(v), 0.0)
    assert np.all(np.isfinite(ut)) and np.all(np.isfinite(vt))
    pre, _ = W.precompute(3, N, coefficients=co, phase=(0.4, 0.3),
                          boundary=dict(bot="wall", top="wall", lft="absorbing", rgt="absorbing_2beta"))
    with pytest.raises(W.ErrorException) as ei:
        W.edg_rhs(np.zeros((N, N, 4, 4), order="F"), np.zeros((N, N, 3, 3), order="F"), 0.07, N, 1.0 / N, pre)
    assert str(ei.value) == "boundary weight 1 - βg ≤ 0 for the boundary data g (absorbing side)"


def test_dimension_mismatch_and_arguments(gpu):
    """test/runtests.jl:586-599 and the nblocks check of src/rhs.jl:186."""
    pre, _ = W.precompute(2, 8)
    pre9, _ = W.precompute(2, 9)
    with pytest.raises(W.DimensionMismatch):
        W.edg_rhs(np.zeros((8, 8, 3, 3), order="F"), np.zeros((8, 7, 2, 2), order="F"), 0.0, 8, 1 / 8, pre)
    with pytest.raises(W.DimensionMismatch):
        W.edg_rhs_(W.Workspace(pre9, 9), np.zeros((8, 8, 3, 3), order="F"), np.zeros((8, 8, 2, 2), order="F"),
                   0.0, 8, 1 / 8, pre)
    with pytest.raises(W.DimensionMismatch):
        W.edg_rhs(np.zeros((8, 8, 3, 3), order="F"), np.zeros((8, 8, 2, 2), order="F"), 0.0, 8, 1 / 8, pre9)
    with pytest.raises(W.ErrorException):
        W.Workspace(pre, 8, nblocks=0)
    assert W.Workspace(W.precompute(2, 3)[0], 3, nblocks=8).nb == 2


def test_mirror_parity_of_the_rules(gpu):
    """The kernels rely on the mirror symmetry of the Gauss-Legendre rules: arrays that have
    it to round-off are accepted (and give the oracle's result), a rule without it is refused."""
    pre, opre_ = _pair(4, 6, flux="upwind", mixed=True)
    rng = np.random.default_rng(3)
    u = np.asfortranarray(rng.standard_normal((6, 6, 5, 5)))
    v = np.asfortranarray(1e-3 * rng.standard_normal((6, 6, 4, 4)))
    near = dict(pre)
    for k in ("P_h_v", "P_u", "S_u", "w"):
        near[k] = np.asfortranarray(pre[k] * (1 + 1e-16 * rng.standard_normal(pre[k].shape)))
    ours = W.Workspace(near, 6).rhs(u, v, 0.2)
    ref = OracleWorkspace(opre_).rhs(u, v, 0.2)
    assert rel_max(ours, ref) < TOL
    bad = dict(pre)
    bad["P_h_v"] = np.asfortranarray(pre["P_h_v"].copy())
    bad["P_h_v"][0, 1] += 1e-6
    with pytest.raises(RuntimeError, match="wedg_create failed"):
        W.Workspace(bad, 6)


def test_blow_up_flag(gpu):
    """A non-finite state makes ws.fin false after the step (src/solver.jl:311-321, 940). With the
    CG solver the step completes (a NaN residual ends CG at once, src/rhs.jl:841); with Chebyshev
    the NaN stage state is a non-positive-definite mass matrix at the next stage, as in the
    reference (src/rhs.jl:897-899), and the step raises."""
    N = 4
    for solver in ("cg", "chebyshev"):
        pre, _ = W.precompute(2, N, mode="source", coefficients=W.constant_coefficients(c=1.0, alpha=0.0, beta=0.0),
                              mass_solver=solver)
        u = np.zeros((N, N, 3, 3), order="F")
        v = np.zeros((N, N, 2, 2), order="F")
        u[1, 1, 0, 0] = math.inf
        ws = W.Workspace(pre, N)
        if solver == "cg":
            W.rk4_step_(u, v, 0.0, 1e-3, N, 1.0 / N, pre, ws)
            assert not ws.fin
        else:
            with pytest.raises(W.ErrorException, match="mass matrix not positive definite"):
                W.rk4_step_(u, v, 0.0, 1e-3, N, 1.0 / N, pre, ws)


def test_full_size_rhs_against_oracle(gpu):
    """Plain method at GPU scale: N = 512, q_u = q_v = 6, source mode, alternating flux,
    constant coefficients (c = 1, α = 1e-6, β = 8), bottom absorbing, three walls κ = 0.5:
    one RHS on a seeded state with 1 - 2βv spanning about [0.4, 1.6], against the oracle's RHS
    on the same pre (the product's precompute, checked array by array against the oracle's
    restatement in test_host.py; the oracle's own precompute is too slow at this size)."""
    N = 512
    kw = dict(mixed=False, mode="source", kappa=0.5, flux="alternating",
              boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))
    pp = W.precompute(6, N, coefficients=W.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0), **kw)[0]
    po = dict(pp, Ainv_u=np.asfortranarray(pp["Ainv_u"]))
    rng = np.random.default_rng(0)
    u = np.asfortranarray(1e-3 * rng.standard_normal((N, N, 7, 7)))
    v = np.asfortranarray(1e-3 * rng.standard_normal((N, N, 7, 7)) / np.arange(1, 8)[None, None, :, None] ** 2)
    v[:, :, 0, 0] += 0.03 * np.sin(np.linspace(0, 6 * np.pi, N))[:, None]
    a = OracleWorkspace(po).rhs(u, v, 0.3)
    ws = W.Workspace(pp, N)
    assert ws.stats()["fast_path"] == 1
    b = ws.rhs(u, v, 0.3)
    assert rel_max(a, b) < TOL


def test_inverses_computed_on_the_device(gpu):
    """Coefficients that vary inside the elements need the packed inverse stiffnesses of
    src/solver.jl:528-535; without them in pre, wedg_create computes them on the device. The
    RHS then matches the one from the host-computed inverses, and the oracle."""
    rng = np.random.default_rng(31)
    for q, N, mixed in ((2, 9, True), (5, 9, False), (7, 9, True)):
        pd, po = _pair(q, N, mixed=mixed, mode="mms", phase=(0.4, 0.3))
        ph = W.precompute(q, N, mixed=mixed, mode="mms", phase=(0.4, 0.3), inverses="host")[0]
        assert pd["Ainv_u"] is None and ph["Ainv_u"] is not None
        u, v = _state(rng, pd, N)
        a = W.Workspace(pd, N).rhs(u, v, 0.037)
        a = tuple(x.copy() for x in a)
        b = W.Workspace(ph, N).rhs(u, v, 0.037)
        assert rel_max(a, b) < 1e-13
        assert rel_max(OracleWorkspace(po).rhs(u, v, 0.037), a) < TOL


def test_rk4_many_steps_on_a_mesh_with_fewer_elements_than_bins(gpu):
    """Twenty RK4 steps on a 4 × 4 mesh (16 elements, fewer than the 48 Chebyshev-count bins of
    the mass kernel) while the step counts climb past 16: every stage must start from empty
    bins, whatever the element count (a stale bin once dropped an element from the solve)."""
    rng = np.random.default_rng(5)
    q, N = 3, 4
    kw = dict(mode="source", flux="upwind", boundary="absorbing_2beta")
    pp = W.precompute(q, N, coefficients=W.constant_coefficients(c=1.1, alpha=1e-3, beta=3.0), **kw)[0]
    po = opre(q, N, coefficients=oc.constant_coefficients(c=1.1, alpha=1e-3, beta=3.0), **kw)[0]
    nu, nv = pp["qu1"], pp["qv1"]
    d = lambda n: 1.0 / (1.0 + np.add.outer(np.arange(n), np.arange(n))) ** 2
    u = np.asfortranarray(0.01 * rng.standard_normal((N, N, nu, nu)) * d(nu))
    v = np.asfortranarray(0.001 * rng.standard_normal((N, N, nv, nv)) * d(nv))
    dt = (1.0 / N) / (10 * q * q)
    uo, vo = u.copy(order="F"), v.copy(order="F")
    OracleWorkspace(po).rk4_steps(uo, vo, 0.02, dt, 20)
    ws = W.Workspace(pp, N)
    assert ws.rk4_steps(u, v, 0.02, dt, 20) == 20
    assert ws.stats()["cheb_steps_max"] > N * N       # counts beyond the element count
    assert rel_max((u, v), (uo, vo)) < TOL, rel_max((u, v), (uo, vo))


def test_mms_n10_per_evaluation_rhs_seeds(gpu):
    """The manufactured-solution run solve(3, 10, 0.1; flux=:upwind, mixed=true) with its defaults (paper
    coefficients, absorbing_2beta on every side, σ = 0): the per-evaluation RHS against the
    oracle's on the seeded states u ~ N(0, 1), v ~ 0.05 N(0, 1) of test/runtests.jl:273, seeds 0 to 9,
    at t = 0.037, one workspace for all ten calls."""
    N, q = 10, 3
    pp, po = _pair(q, N, flux="upwind", mixed=True)
    ws, ow = W.Workspace(pp, N), OracleWorkspace(po)
    worst = 0.0
    for seed in range(10):
        u, v = _state(np.random.default_rng(seed), pp, N)
        worst = max(worst, rel_max(ow.rhs(u, v, 0.037), ws.rhs(u, v, 0.037)))
    assert worst < TOL, worst


def test_jumping_coefficients_n256_against_oracle(gpu):
    """The jumping-coefficient workload at its size: N = 256, q_u = 5, q_v = 4, initial-value mode, c, α, β constant on 4 × 4
    subsquares (the bench's default_rng(3) draw), dirichlet / absorbing / absorbing_2beta / wall
    sides, central flux, one-sided faces. One RHS and two RK4 steps on a seeded state against the
    oracle on the same pre (src/rhs.jl:490-550, src/solver.jl:289-321)."""
    from bench import config3_problem
    pp, N, dt = config3_problem()
    assert pp["one_sided"] and pp["Ainv_u"] is not None
    po = dict(pp, Ainv_u=np.asfortranarray(pp["Ainv_u"]))
    nu, nv = pp["qu1"], pp["qv1"]
    rng = np.random.default_rng(33)
    d = lambda n: 1.0 / (1.0 + np.add.outer(np.arange(n), np.arange(n))) ** 2   # noqa: E731
    # rough random data: at 1e-4 the stages already drive 2βv past 1 somewhere (β ≤ 10); at 1e-5 |v| stays
    # near 2e-3
    u = np.asfortranarray(1e-5 * rng.standard_normal((N, N, nu, nu)) * d(nu))
    v = np.asfortranarray(2e-6 * rng.standard_normal((N, N, nv, nv)) * d(nv))
    ow, ws = OracleWorkspace(po), W.Workspace(pp, N)
    assert ws.stats()["fast_path"] == 1
    assert rel_max(ow.rhs(u, v, 0.01), ws.rhs(u, v, 0.01)) < TOL
    uo, vo = u.copy(order="F"), v.copy(order="F")
    ug, vg = u.copy(order="F"), v.copy(order="F")
    for k in range(2):
        ow.rk4_step(uo, vo, 0.01 + k * dt, dt)
        W.rk4_step_(ug, vg, 0.01 + k * dt, dt, N, 1.0 / N, pp, ws)
    assert ws.fin
    assert rel_max((uo, vo), (ug, vg)) < TOL, rel_max((uo, vo), (ug, vg))


def test_headline_front_state_rk4_step_against_oracle(gpu):
    """The bench's headline workload and state: N = 512, q_u = q_v = 6, source mode, c = 1, α = 1e-6,
    β = 8, bottom absorbing_2beta and three walls (κ = 0.5), alternating flux, and the seeded
    steepened circular front (1 - 2βv_h across [0.42, 1.58], up to about 20 Chebyshev steps). One
    RK4 step at the bench's t0 and dt against the oracle's on the same pre; the GPU takes every
    element's own Chebyshev count, the oracle the reference's common maximum."""
    import bench
    N = 512
    pp = W.precompute(bench.Q, N, coefficients=W.constant_coefficients(**bench.COEF), **bench.KW)[0]
    po = dict(pp, Ainv_u=np.asfortranarray(pp["Ainv_u"]))
    u, v = bench.synthetic_state(N, pp["qu1"], pp["qv1"], 0, "front")
    dt = (1.0 / N) / (10 * bench.Q ** 2)
    ug, vg = u.copy(order="F"), v.copy(order="F")
    ws = W.Workspace(pp, N)
    W.rk4_step_(ug, vg, bench.T0, dt, N, 1.0 / N, pp, ws)
    assert ws.fin and ws.stats()["cheb_steps_max"] >= 10
    ow = OracleWorkspace(po)
    ow.rk4_step(u, v, bench.T0, dt)
    assert rel_max((u, v), (ug, vg)) < TOL, rel_max((u, v), (ug, vg))


def test_rk4_steps_common_count_against_oracle(gpu):
    """The reference's Chebyshev policy over RK4 steps: every element of a stage takes that stage's
    largest count (src/rhs.jl:911-918), which changes from stage to stage as v_h changes. Three RK4
    steps from a state whose counts differ widely over the elements, against the oracle's."""
    rng = np.random.default_rng(61)
    N = 9
    co = oc.replace_coefficients(oc.paper_coefficients(), beta=8.0)
    pp, po = _pair(4, N, coefficients=co, mode="source")
    # u small enough that c²Δu does not push 2βv past 1 within the three steps (β = 8)
    u = np.asfortranarray(1e-4 * rng.standard_normal((N, N, pp["qu1"], pp["qu1"])))
    v = np.asfortranarray(1e-4 * rng.standard_normal((N, N, pp["qv1"], pp["qv1"])))
    v[:, 0:2, 1, 0] = 0.04
    uo, vo = u.copy(order="F"), v.copy(order="F")
    ow = OracleWorkspace(po)
    ws = W.Workspace(pp, N, cheb_steps="common_max")
    dt = (1.0 / N) / (10 * 16)
    for k in range(3):
        ow.rk4_step(uo, vo, 0.1 + k * dt, dt)
        W.rk4_step_(u, v, 0.1 + k * dt, dt, N, 1.0 / N, pp, ws)
    assert ws.stats()["cheb_steps_max"] > 20
    assert rel_max((uo, vo), (u, v)) < TOL, rel_max((uo, vo), (u, v))


def test_modal_traces_against_oracle(gpu):
    """The traces kept as modal end sums (interior faces with one coefficient value along them:
    constant coefficients, and coefficients constant on cells of the mesh, whose one-sided faces
    carry jump terms in initial-value mode), against the oracle's point form: one RHS and two RK4
    steps over the fluxes, side kinds, pairings and degrees, and the RHS with jump terms; the point
    form where a face's coefficients vary along it (paper coefficients)."""
    rng = np.random.default_rng(23)
    worst = 0.0
    kinds = (dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing"),
             dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta"), "absorbing_2beta")
    cells = W.cell_coefficients(np.array([[1.0, 0.7], [1.3, 0.9]]), np.array([[1e-4, 3e-4], [2e-4, 1e-5]]),
                                np.array([[0.05, 0.2], [0.1, 0.3]]))   # β small enough for the source's v
    for q in (1, 3, 6):
        for N in (1, 2, 3, 4):
            for mixed in (True, False):
                for flux in ("upwind", "central", "alternating"):
                    for bd in kinds:
                        for co in ("constant", "cells"):
                            if co == "cells" and N % 2:
                                continue
                            if N < 3 and (flux != "upwind" or q == 6):
                                continue       # N = 1 (no interior face) and 2: a few cases
                            kw = dict(flux=flux, mixed=mixed, mode="source", boundary=bd, sigma=0.3,
                                      sigma_dirichlet=0.6, kappa=0.7)
                            if co == "constant":
                                pp = W.precompute(q, N, coefficients=W.constant_coefficients(c=1.2, alpha=3e-4,
                                                                                              beta=0.5), **kw)[0]
                                po = opre(q, N, coefficients=oc.constant_coefficients(c=1.2, alpha=3e-4, beta=0.5),
                                          **kw)[0]
                            else:
                                pp, po = _pair(q, N, coefficients=cells, **kw)
                                assert pp["one_sided"]
                            ws = W.Workspace(pp, N)
                            assert ws.stats()["modal_traces"] == 1, (q, N, co)
                            u, v = _state(rng, pp, N, 1e-3, 1e-4)
                            ow = OracleWorkspace(po)
                            worst = max(worst, rel_max(ow.rhs(u, v, 0.037), ws.rhs(u, v, 0.037)))
                            if q == 3 and flux == "alternating":
                                uo, vo = u.copy(order="F"), v.copy(order="F")
                                dt = (1.0 / N) / (10 * q * q)
                                for k in range(2):
                                    ow.rk4_step(uo, vo, 0.02 + k * dt, dt)
                                    W.rk4_step_(u, v, 0.02 + k * dt, dt, N, 1.0 / N, pp, ws)
                                worst = max(worst, rel_max((uo, vo), (u, v)))
    assert worst < TOL, worst
    pp = W.precompute(3, 4, mode="source")[0]                                        # paper coefficients
    assert W.Workspace(pp, 4).stats()["modal_traces"] == 0
    # jump terms from the initial data across jumping coefficients: projected on the face modes
    for q, N, flux in ((3, 4, "central"), (5, 4, "upwind"), (2, 6, "alternating")):
        pp, po = _pair(q, N, mode="initial_value", flux=flux, boundary="dirichlet", sigma=0.3,
                       coefficients=quadrant_coefficients(0.5, 0.5, smooth=False))
        assert pp["one_sided"] and (np.any(pp["hJC"] != 0) or np.any(pp["vJC"] != 0))
        ws = W.Workspace(pp, N)
        assert ws.stats()["modal_traces"] == 1
        u, v = _state(rng, pp, N, 1e-3, 1e-4)
        assert rel_max(OracleWorkspace(po).rhs(u, v, 0.037), ws.rhs(u, v, 0.037)) < TOL


def test_modal_and_point_traces_agree(gpu):
    """The same workspace with modal traces and with point traces (modal_traces=False): the RHS and
    ten RK4 steps agree to rounding, for the constant-coefficient and the general kernels."""
    rng = np.random.default_rng(29)
    for q, N, fast in ((6, 6, True), (3, 5, True), (4, 4, False)):
        kw = dict(flux="alternating", mixed=False, mode="source", kappa=0.5,
                  boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))
        pp = W.precompute(q, N, coefficients=W.constant_coefficients(c=1.0, alpha=1e-4, beta=2.0), **kw)[0]
        wm = W.Workspace(pp, N, fast_path=fast)
        wp = W.Workspace(pp, N, fast_path=fast, modal_traces=False)
        assert wm.stats()["modal_traces"] == 1 and wp.stats()["modal_traces"] == 0
        u, v = _state(rng, pp, N, 1e-6, 1e-7)      # rough data: small, so that 1 - 2βv stays positive
        assert rel_max(wm.rhs(u, v, 0.2), wp.rhs(u, v, 0.2)) < 1e-13
        um, vm = u.copy(order="F"), v.copy(order="F")
        dt = (1.0 / N) / (10 * q * q)
        assert wm.rk4_steps(um, vm, 0.2, dt, 10) == 10 and wp.rk4_steps(u, v, 0.2, dt, 10) == 10
        assert rel_max((um, vm), (u, v)) < 1e-13


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_host_state_steps_match_device_state(gpu, solver):
    """rk4_steps on a host state -- copied in by ranges of elements while the first stage's k_prep
    runs on the ranges that have arrived, the final u copied out beside the last mass solve --
    against the same steps on a device state: bit for bit (N = 64, every range boundary inside the
    mesh)."""
    import torch
    N, q = 64, 3
    pp = W.precompute(q, N, flux="upwind", mixed=True, mode="source", mass_solver=solver, kappa=0.5,
                      coefficients=W.constant_coefficients(c=1.1, alpha=1e-4, beta=2.0))[0]
    rng = np.random.default_rng(37)
    u, v = _state(rng, pp, N, 1e-6, 1e-7)
    dt = (1.0 / N) / (10 * q * q)
    wh, wd = W.Workspace(pp, N), W.Workspace(pp, N)
    uh, vh = u.copy(order="F"), v.copy(order="F")
    assert wh.rk4_steps(uh, vh, 0.05, dt, 3) == 3
    ud = torch.from_numpy(u.reshape(-1, order="F").copy()).cuda()
    vd = torch.from_numpy(v.reshape(-1, order="F").copy()).cuda()
    assert wd.rk4_steps(ud, vd, 0.05, dt, 3) == 3
    assert np.array_equal(uh.reshape(-1, order="F"), ud.cpu().numpy())
    assert np.array_equal(vh.reshape(-1, order="F"), vd.cpu().numpy())


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_rhs_on_device_state_matches_host_state(gpu, solver):
    """edg_rhs! with device pointers (wedg_rhs, WEDG_DEVICE: no copies) against the host-state call
    on the same inputs, bit for bit, and against the oracle; twice in a row on different states."""
    import torch
    N, q = 6, 4
    kw = dict(flux="alternating", mixed=True, mode="mms", mass_solver=solver,
              boundary=dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing"))
    pp, po = _pair(q, N, **kw)
    ws = W.Workspace(pp, N)
    rng = np.random.default_rng(41)
    for t in (0.037, 0.11):
        u, v = _state(rng, pp, N)
        host = tuple(x.copy() for x in ws.rhs(u, v, t))
        ud = torch.from_numpy(u.reshape(-1, order="F").copy()).to(gpu)
        vd = torch.from_numpy(v.reshape(-1, order="F").copy()).to(gpu)
        utd, vtd = torch.full_like(ud, float("nan")), torch.full_like(vd, float("nan"))
        ws.rhs(ud, vd, t, utd, vtd)
        dev = (utd.cpu().numpy().reshape(u.shape, order="F"), vtd.cpu().numpy().reshape(v.shape, order="F"))
        assert np.array_equal(host[0], dev[0]) and np.array_equal(host[1], dev[1])
        assert rel_max(OracleWorkspace(po).rhs(u, v, t), dev) < TOL


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
def test_mass_solves_against_the_dense_reference(gpu, solver):
    """The mass systems at max 2β|v_q| of 1e-3, 0.5 and 0.9 (test/runtests.jl:418-441): the RHS of the
    GPU (both mass solvers; up to 45 Chebyshev steps at q = 6) against the dense restatement of
    test/reference_rhs.jl, whose mass solve is an LU factorisation of each element matrix. Walls
    (no boundary weight) so that only the mass matrices bound v."""
    from oracle.reference_rhs import dense_volume, edg_rhs_reference, reference_pre
    rng = np.random.default_rng(7)
    worst = 0.0
    for q, mixed, N in ((1, True, 3), (3, True, 4), (4, False, 3), (6, True, 2)):
        pp, po = _pair(q, N, mixed=mixed, mass_solver=solver, boundary="wall", kappa=0.5)
        nv, E = pp["qv1"], N * N
        V0 = rng.standard_normal((N, N, nv, nv))
        U = np.asfortranarray(rng.standard_normal((N, N, pp["qu1"], pp["qu1"])))
        vq = np.einsum("ra,eab,sb->ers", po["P_h_v"], V0.reshape(E, nv, nv, order="F"), po["P_h_v"])
        g0 = np.max(np.abs(2 * np.transpose(po["beta_hq"], (1, 0, 2)) * vq))
        dense = dense_volume(reference_pre(po))
        ws = W.Workspace(pp, N)
        for gmax in (1e-3, 0.5, 0.9):
            V = np.asfortranarray(V0 * (gmax / g0))
            a = edg_rhs_reference(U, V, 0.037, N, 1.0 / N, dense)
            worst = max(worst, rel_max(a, ws.rhs(U, V, 0.037)))
    assert worst < TOL, worst


@pytest.mark.parametrize("solver", ["chebyshev", "cg"])
@pytest.mark.parametrize("q", [1, 2, 3, 6])
def test_nblocks_bitwise_rhs_and_rk4(gpu, solver, q):
    """test/runtests.jl:468-500: every nblocks gives the same RHS and RK4 steps bit for bit (N = 7,
    both pairings, every mode, two mixed side layouts, the paper's coefficients and jumping ones on
    the mesh lines x = 3/7, y = 4/7). Here nblocks is accepted and recorded (ws.nb); each workspace
    is a separate allocation, so this also checks that runs are reproducible bit for bit although
    k_prep lists the elements by Chebyshev count with atomics."""
    N, h = 7, 1.0 / 7
    mixed2 = dict(bot="wall", top="absorbing", lft="dirichlet", rgt="absorbing_2beta")
    mixed1 = dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing")
    pw7 = quadrant_coefficients(3 / 7, 4 / 7, alpha=(1e-5, 4e-6, 2e-5, 1e-6), smooth=True)
    for mixed in (True, False):
        for mode in ("mms", "initial_value", "source"):
            for boundary in (mixed1, mixed2):
                for coef in (None, pw7):
                    if mode == "mms" and coef is not None:
                        continue
                    kw = dict(mixed=mixed, mode=mode, boundary=boundary, mass_solver=solver, sigma=0.3,
                              sigma_dirichlet=0.6, kappa=0.7, phase=(0.4, 0.3))
                    if coef is not None:
                        kw["coefficients"] = coef
                    pre = W.precompute(q, N, **kw)[0]
                    assert bool(pre["one_sided"]) == (coef is not None)
                    rng = np.random.default_rng(q)
                    u, v = _state(rng, pre, N, 1e-2, 0.05)
                    ws1 = W.Workspace(pre, N, nblocks=1)
                    r1 = tuple(x.copy() for x in ws1.rhs(u, v, 0.037))
                    s1 = (u.copy(order="F"), v.copy(order="F"))
                    for k in (1, 2):
                        W.rk4_step_(*s1, 0.01 * k, 1e-4, N, h, pre, ws1)
                    for nb in (3, 5, 8):
                        ws = W.Workspace(pre, N, nblocks=nb)
                        assert ws.nb == nb
                        r = ws.rhs(u, v, 0.037)
                        assert np.array_equal(r[0], r1[0]) and np.array_equal(r[1], r1[1])
                        s = (u.copy(order="F"), v.copy(order="F"))
                        for k in (1, 2):
                            W.rk4_step_(*s, 0.01 * k, 1e-4, N, h, pre, ws)
                        assert np.array_equal(s[0], s1[0]) and np.array_equal(s[1], s1[1])
