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
  stops (test/runtests.jl:838-848).
"""
import math

import numpy as np
import pytest

import edg_westervelt_gb300 as W

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
