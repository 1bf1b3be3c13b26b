"""Whole-run properties of the reference's own test suite, through ``solve`` on the GPU.

These need no second implementation: they are the reference's integration tests
(test/runtests.jl), run here through the product's ``solve`` (the time loop, the
source-mode diagnostics and the error norms on the GPU).
- boundary spellings give bit-identical runs (test/runtests.jl:243-264);
- after the source stops, the energy is conserved by walls with κ = 0 and Dirichlet sides
  with σ_D = 0 under the central flux, and dissipated otherwise (test/runtests.jl:386-406);
- every boundary kind converges at the reference's orders on meshes 6 → 12
  (test/runtests.jl:408-413), and so does a jump of β alone (:824-835);
- with c, α, β jumping on mesh lines and absorbing sides the energy decays after the source
  stops (test/runtests.jl:838-848);
- the interface terms of an initial profile u₀ (test/runtests.jl:760-784);
- the semi-discrete energy identity with jumping coefficients (test/runtests.jl:734-761);
- the convergence of a two-layer standing mode across a jump of c (test/runtests.jl:816-823).
"""
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from reference_properties import ENERGY_FLUXES, energy_terms, lin_profile, project_u, two_layer_error

pytestmark = pytest.mark.gpu

MIXED = dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing")


def test_boundary_spellings_bitwise(gpu):
    e = W.solve(2, 4, 0.05)
    assert e == W.solve(2, 4, 0.05, boundary="absorbing_2beta")
    assert e == W.solve(2, 4, 0.05, boundary=dict(rgt="absorbing_2beta", lft="absorbing_2beta",
                                                  top="absorbing_2beta", bot="absorbing_2beta"),
                        kappa=0.7, phase=(0.0, 0.0))
    assert W.solve(2, 4, 0.05, boundary="absorbing") == W.solve(
        2, 4, 0.05, boundary=dict(rgt="absorbing", lft="absorbing", top="absorbing", bot="absorbing"))
    d4 = dict(bot="dirichlet", top="dirichlet", lft="dirichlet", rgt="dirichlet")
    assert W.solve(2, 4, 0.05, boundary="dirichlet", sigma=0.3) == W.solve(2, 4, 0.05, boundary=d4,
                                                                           sigma_dirichlet=0.3)


def _energy_after(**kw):
    src = W.GaussianSource(x0=(0.3, 0.6), r0=0.1, omega=8 * math.pi, Ts=0.25)
    co = W.constant_coefficients(c=1.0, alpha=0.0, beta=0.0)
    H = W.solve(3, 8, 0.75, mode="source", coefficients=co, source=src, record_every=5, **kw)
    return H["energy"][H["t"] > 0.25]


@pytest.mark.parametrize("kw", [dict(boundary="wall", flux="central"), dict(boundary="dirichlet", flux="central"),
                                dict(boundary=dict(bot="dirichlet", top="wall", lft="wall", rgt="dirichlet"),
                                     flux="central")])
def test_energy_conserved_after_the_source(gpu, kw):
    E = _energy_after(**kw)
    assert len(E) > 10
    assert np.max(np.abs(E - E[0])) / E[0] < 1e-6


@pytest.mark.parametrize("kw", [dict(boundary="wall", kappa=0.5, flux="central"),
                                dict(boundary="dirichlet", sigma_dirichlet=1.0, flux="central"),
                                dict(boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))])
def test_energy_dissipated_after_the_source(gpu, kw):
    E = _energy_after(**kw)
    assert len(E) > 10
    assert np.max(np.diff(E)) <= 1e-10 * E[0]
    assert E[-1] / E[0] < 0.95


@pytest.mark.parametrize("boundary", ["absorbing_2beta", "dirichlet", "wall", "mixed"])
def test_convergence_per_boundary_kind(gpu, boundary):
    bd = MIXED if boundary == "mixed" else boundary
    kw = dict(boundary=bd, sigma_dirichlet=1.0, kappa=1.0, phase=(0.4, 0.3))
    e1 = W.solve(2, 6, 0.1, **kw)
    e2 = W.solve(2, 12, 0.1, **kw)
    assert math.log2(e1["erru"] / e2["erru"]) > 2.5
    assert math.log2(e1["errE"] / e2["errE"]) > 1.5


@pytest.mark.parametrize("flux", ["upwind", "central"])
def test_energy_decay_with_jumping_coefficients(gpu, flux):
    """test/runtests.jl:838-848: c, α, β jumping on x = ½ and y = ½ (one-sided faces), absorbing
    sides; after the source stops the energy does not increase and falls below 95 %."""
    from test_oracle import quadrant_coefficients
    co = quadrant_coefficients(0.5, 0.5, alpha=(1e-5, 4e-6, 2e-5, 1e-6), beta=(1e-4, 3e-4, 0.0, 2e-4))
    src = W.GaussianSource(x0=(0.45, 0.55), r0=0.08, amplitude=50.0, omega=8 * math.pi, Ts=0.25)
    H = W.solve(3, 8, 0.75, mode="source", coefficients=co, flux=flux, source=src, record_every=5)
    E = H["energy"][H["t"] > 0.25]
    assert len(E) > 10
    assert np.max(np.diff(E)) <= 1e-10 * E[0]
    assert E[-1] / E[0] < 0.95


def test_convergence_with_a_jump_of_beta_alone(gpu):
    """test/runtests.jl:824-835: a jump of β alone keeps the continuous face kernel and the
    manufactured solution; the orders on meshes 6 → 12 with mixed sides."""
    from test_oracle import quadrant_coefficients
    cb = quadrant_coefficients(0.5, 0.5, c=(1.0, 1.0, 1.0, 1.0), alpha=(1e-3, 1e-3, 1e-3, 1e-3))
    assert not W.precompute(2, 6, coefficients=cb)[0]["one_sided"]
    kw = dict(coefficients=cb, boundary=MIXED, kappa=0.5, sigma_dirichlet=1.0, phase=(0.4, 0.3))
    e1 = W.solve(2, 6, 0.1, **kw)
    e2 = W.solve(2, 12, 0.1, **kw)
    assert math.log2(e1["erru"] / e2["erru"]) > 2.5
    assert math.log2(e1["errE"] / e2["errE"]) > 1.5


def test_interface_terms_of_the_initial_profile(gpu):
    """test/runtests.jl:760-784: with u = ũ + u₀, the :initial_value RHS at (ũ, v) = (0, 0) equals
    the plain RHS at (u, v) = (u₀, 0) when u₀ lies in U_h: c jumping at x = ½ where ∂_n u₀ ≠ 0, and
    u₀ = |x - ½| + y/2 for a constant c. The jump terms of u₀ enter the one-sided faces (here
    projected on the face modes, the coefficients being one value along every face)."""
    from test_host import Step
    z0 = lambda x, y: 0.0   # noqa: E731
    N, h = 8, 1.0 / 8
    for c1, c2, ip in ((1.0, 0.5, lin_profile(0.0, 1.0)), (0.8, 0.8, lin_profile(1.0, 0.0))):
        coef = W.Coefficients(Step(1, 0.5, c1, c2), z0, z0, Step(1, 0.5, 1e-3 * c1 ** 2, 1e-3 * c2 ** 2), z0, z0, z0)
        for flux in ("upwind", "central", "alternating"):
            for q in (1, 3):
                kw = dict(coefficients=coef, boundary="wall", flux=flux)
                pI, _ = W.precompute(q, N, mode="initial_value", initial_profile=ip, **kw)
                pS, _ = W.precompute(q, N, mode="source", source=W.GaussianSource(amplitude=0.0), **kw)
                assert pI["one_sided"]
                zu, zv = np.zeros((N, N, pI["qu1"], pI["qu1"]), order="F"), np.zeros((N, N, pI["qv1"], pI["qv1"]), order="F")
                rI = tuple(x.copy() for x in W.Workspace(pI, N).rhs(zu, zv, 0.3))
                rS = W.Workspace(pS, N).rhs(project_u(ip["u0"], pS, N), zv, 0.3)
                assert np.max(np.abs(rI[1] - rS[1])) <= 1e-11 * np.max(np.abs(rS[1])), (c1, flux, q)
                assert np.max(np.abs(rI[0] - rS[0])) <= 1e-11, (c1, flux, q)


def test_energy_identity_with_jumping_coefficients(gpu):
    """test/runtests.jl:734-761: for random states, c, α, β jumping on x = ½ and y = ½ (one-sided
    faces), four walls with κ = 0 and no source, the GPU RHS satisfies dE/dt = -Σ∫α|∇v_h|² - D_I to
    1e-12 of the terms' size (D_I = 0 for the fluxes without dissipation), so dE/dt ≤ 0; q = 1..4,
    both pairings, six flux parameter sets."""
    from test_oracle import quadrant_coefficients
    co = quadrant_coefficients(0.5, 0.5, beta=(0.0, 0.3, 0.1, 0.2))
    N, worst, rise = 4, 0.0, -math.inf
    for q in (1, 2, 3, 4):
        for mixed in (True, False):
            for fp in ENERGY_FLUXES:
                pre, _ = W.precompute(q, N, flux_params=fp, mixed=mixed, mode="source", boundary="wall", kappa=0.0,
                                      coefficients=co, source=W.GaussianSource(amplitude=0.0))
                rng = np.random.default_rng(10 * q + mixed)
                u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                ut, vt = (x.copy() for x in W.Workspace(pre, N).rhs(u, v, 0.3))
                et = energy_terms(u, v, ut, vt, pre, co, N)
                if fp["tau"] == 0 and fp["lambda_u"] == 0 and fp["lambda_v"] == 0:
                    assert et["DI"] == 0
                worst = max(worst, abs(et["dEdt"] + et["Dv"] + et["DI"]) / et["scale"])
                rise = max(rise, et["dEdt"] / et["scale"])
    assert worst < 1e-12, worst
    assert rise < 1e-12, rise


def test_convergence_at_a_coefficient_jump(gpu):
    """test/runtests.jl:816-823: the two-layer standing mode converges at about q_u in the energy
    norm for the upwind flux and about 1 for the central flux (q_u = 2, meshes 8 → 16), and the
    interface along y gives the same error as along x."""
    e8 = two_layer_error(W.solve, W.Coefficients, 2, 8, 0.5, "upwind", "x")
    e16 = two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "upwind", "x")
    assert math.log2(e8 / e16) > 1.8
    assert two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "upwind", "y") == pytest.approx(e16, rel=1e-10)
    c8 = two_layer_error(W.solve, W.Coefficients, 2, 8, 0.5, "central", "x")
    c16 = two_layer_error(W.solve, W.Coefficients, 2, 16, 0.5, "central", "x")
    assert math.log2(c8 / c16) > 0.9
