"""The oracle pinned against the reference's stored results and its dense second implementation.

Mirrors test/runtests.jl:156-163 (quadrature), :189-293 and :716-732
(batched RHS = element-by-element reference RHS, max-norm relative < 1e-12),
:207-218 (regression pins, rtol 1e-9) and the stored convergence data
(data/convergence/results.csv, fixtures in tests/golden/).
"""
import json
import os

import numpy as np
import pytest

from conftest import rel_max
from oracle import coefficients as oc
from oracle.precompute import precompute
from oracle.quadrature import gauss_q_cofs, jacobi_p
from oracle.reference_rhs import dense_volume, edg_rhs_reference, reference_pre
from oracle.solver import solve

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_quadrature_and_basis():
    x, w = gauss_q_cofs(5)
    assert abs(np.sum(w) - 2) < 1e-14
    assert abs(np.sum(w * x ** 8) - 2 / 9) < 1e-14
    G = np.array([[np.sum(w * jacobi_p(x, 0, 0, m) * jacobi_p(x, 0, 0, n)) for n in range(5)] for m in range(5)])
    assert np.max(np.abs(G - np.eye(5))) < 1e-13


@pytest.mark.parametrize("case", json.load(open(os.path.join(GOLD, "regression.json")))["cases"],
                         ids=["absorbing_2beta", "absorbing"])
def test_regression_pins(oracle_lib, case):
    e = solve(case["q"], case["N"], case["T"], **case["kw"])
    for k in ("erru", "errv", "errgradu", "errE"):
        assert abs(e[k] / case[k] - 1) < case["rtol"], (k, e[k], case[k])


def test_convergence_data_small_meshes(oracle_lib):
    """Rows of data/convergence/results.csv with N ≤ 6 (computed with mass_solver = :cg)."""
    data = json.load(open(os.path.join(GOLD, "convergence.json")))
    rows = [r for r in data["rows"] if r["N"] <= 6 and r["q"] <= 4]
    assert len(rows) >= 40
    worst = 0.0
    for r in rows:
        e = solve(r["q"], r["N"], data["T"], flux=r["flux"], mixed=r["mixed"], mass_solver="cg")
        for k in ("erru", "errv", "errgradu", "errE"):
            worst = max(worst, abs(e[k] / r[k] - 1))
    assert worst < 1e-9, worst


def _grid(rng, modes, boundaries, qs, Ns, fluxes, extra):
    for mode in modes:
        for boundary in boundaries:
            for q in qs:
                for N in Ns:
                    for flux in fluxes:
                        for mixed in (True, False):
                            yield mode, boundary, q, N, flux, mixed


@pytest.mark.parametrize("mode", ["mms", "initial_value", "source"])
def test_oracle_equals_dense_reference(oracle_lib, mode):
    """test/runtests.jl:189-202, 266-278: every uniform boundary kind, 3 fluxes, both pairings."""
    from oracle.rhs import edg_rhs
    rng = np.random.default_rng(2)
    worst = 0.0
    for boundary in ("absorbing", "dirichlet", "absorbing_2beta", "wall"):
        for q in (1, 3, 4):
            for N in (1, 2, 4):
                for flux in ("upwind", "central", "alternating"):
                    for mixed in (True, False):
                        pre, _ = precompute(q, N, flux=flux, mixed=mixed, mode=mode, boundary=boundary,
                                            sigma=0.3, sigma_dirichlet=0.6, kappa=0.7, phase=(0.4, 0.3))
                        u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                        v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                        a = edg_rhs_reference(u, v, 0.037, N, 1.0 / N, dense_volume(reference_pre(pre)))
                        b = edg_rhs(u, v, 0.037, N, 1.0 / N, pre)
                        worst = max(worst, rel_max(a, b))
    assert worst < 1e-12, worst


def test_oracle_equals_dense_reference_lambda(oracle_lib):
    """test/runtests.jl:281-293: λ_u ≠ λ_v."""
    from oracle.rhs import edg_rhs
    rng = np.random.default_rng(3)
    fp = dict(theta=1.0, tau=0.4, lambda_u=0.7, lambda_v=0.2)
    worst = 0.0
    for boundary in ("absorbing_2beta", "wall"):
        for q in (1, 3):
            for N in (2, 4):
                for mixed in (True, False):
                    for mode in ("mms", "source"):
                        pre, _ = precompute(q, N, flux_params=fp, mixed=mixed, mode=mode, boundary=boundary,
                                            sigma=0.3, kappa=0.7)
                        u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                        v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                        a = edg_rhs_reference(u, v, 0.037, N, 1.0 / N, dense_volume(reference_pre(pre)))
                        worst = max(worst, rel_max(a, edg_rhs(u, v, 0.037, N, 1.0 / N, pre)))
    assert worst < 1e-12, worst


def quadrant_coefficients(xs, ys, c=(1.0, 0.6, 0.8, 0.45), alpha=(0.01, 0.004, 0.02, 0.001),
                          beta=(0.0, 0.03, 0.01, 0.02), smooth=False):
    """Piecewise coefficients on quadrants (test/runtests.jl:46-62)."""
    import math

    def quad(a):
        return lambda x, y: a[int(x >= xs) + 2 * int(y >= ys)]

    cq = quad(c)
    z0 = lambda x, y: 0.0   # noqa: E731
    if smooth:
        return oc.Coefficients(lambda x, y: cq(x, y) * (1 + 0.1 * math.cos(math.pi * x) * math.cos(math.pi * y)),
                               lambda x, y: -0.1 * math.pi * cq(x, y) * math.sin(math.pi * x) * math.cos(math.pi * y),
                               lambda x, y: -0.1 * math.pi * cq(x, y) * math.cos(math.pi * x) * math.sin(math.pi * y),
                               quad(alpha), z0, z0, quad(beta))
    return oc.Coefficients(cq, z0, z0, quad(alpha), z0, z0, quad(beta))


@pytest.mark.parametrize("mode", ["initial_value", "source"])
def test_oracle_equals_dense_reference_piecewise(oracle_lib, mode):
    """test/runtests.jl:716-732: c, α, β jumping across x = ½ and y = ½ (one-sided fluxes)."""
    from oracle.rhs import edg_rhs
    rng = np.random.default_rng(6)
    co = quadrant_coefficients(0.5, 0.5, smooth=True)
    worst = 0.0
    fps = (oc.flux_parameters("upwind"), oc.flux_parameters("central"), oc.flux_parameters("alternating"),
           dict(theta=0.3, tau=0.7, lambda_u=0.4, lambda_v=0.9))
    for q in (1, 3):
        for N in (2, 4):
            for mixed in (True, False):
                for boundary in ("absorbing_2beta", "dirichlet", "wall"):
                    for fp in fps:
                        pre, _ = precompute(q, N, flux_params=fp, mixed=mixed, mode=mode, boundary=boundary,
                                            coefficients=co, sigma=0.3, sigma_dirichlet=0.6, kappa=0.7,
                                            phase=(0.4, 0.3))
                        assert pre["one_sided"]
                        u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                        v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                        a = edg_rhs_reference(u, v, 0.037, N, 1.0 / N, dense_volume(reference_pre(pre)))
                        worst = max(worst, rel_max(a, edg_rhs(u, v, 0.037, N, 1.0 / N, pre)))
    assert worst < 1e-12, worst


def test_oracle_error_messages(oracle_lib):
    """test/runtests.jl:548-577: first failing point / element, reference wording."""
    from oracle.rhs import OracleWorkspace
    N = 8
    co = oc.replace_coefficients(oc.paper_coefficients(), alpha=1e-6, beta=1.0)
    bd = dict(bot="absorbing_2beta", top="absorbing", lft="absorbing", rgt="wall")
    for solver in ("chebyshev", "cg"):
        pre, _ = precompute(3, N, coefficients=co, boundary=bd, mass_solver=solver)
        u = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
        v = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
        v[0, N - 1, 0, 0] = 2.5
        v[3, 0, 0, 0] = 2.5
        with pytest.raises(RuntimeError, match=r"^boundary weight 1 - 2βv_h ≤ 0 at a face point \(absorbing_2beta side\)$"):
            OracleWorkspace(pre).rhs(u, v, 0.0)
        w = np.zeros_like(v)
        w[3, 5, 0, 0] = 2.5
        w[4, 1, 0, 0] = 2.5
        msg = ("mass matrix not positive definite on element 13: 1 - 2βv_h ≤ 0" if solver == "chebyshev"
               else "mass matrix not positive definite on element (5, 2): 1 - 2βv_h ≤ 0")
        with pytest.raises(RuntimeError) as ei:
            OracleWorkspace(pre).rhs(u, w, 0.0)
        assert str(ei.value) == msg
    pre, _ = precompute(3, N, coefficients=co, phase=(0.4, 0.3),
                        boundary=dict(bot="wall", top="wall", lft="absorbing", rgt="absorbing_2beta"))
    z = np.zeros((N, N, pre["qu1"], pre["qu1"]), order="F")
    zv = np.zeros((N, N, pre["qv1"], pre["qv1"]), order="F")
    with pytest.raises(RuntimeError) as ei:
        OracleWorkspace(pre).rhs(z, zv, 0.07)
    assert str(ei.value) == "boundary weight 1 - βg ≤ 0 for the boundary data g (absorbing side)"


# ---- the reference's whole-scheme properties, on the oracle (the same helpers the GPU tests apply
#      to the product: tests/reference_properties.py)

def test_oracle_energy_identity(oracle_lib):
    """test/runtests.jl:734-761 on the oracle: dE/dt = -Σ∫α|∇v_h|² - D_I to 1e-12 with c, α, β
    jumping on x = ½ and y = ½, four walls with κ = 0, q = 1..4, six flux parameter sets."""
    import math

    from oracle.rhs import edg_rhs
    from reference_properties import ENERGY_FLUXES, energy_terms
    co = quadrant_coefficients(0.5, 0.5, beta=(0.0, 0.3, 0.1, 0.2))
    N, worst, rise = 4, 0.0, -math.inf
    for q in (1, 2, 3, 4):
        for mixed in (True, False):
            for fp in ENERGY_FLUXES:
                pre, _ = precompute(q, N, flux_params=fp, mixed=mixed, mode="source", boundary="wall", kappa=0.0,
                                    coefficients=co, source=oc.GaussianSource(amplitude=0.0))
                rng = np.random.default_rng(10 * q + mixed)
                u = np.asfortranarray(rng.standard_normal((N, N, pre["qu1"], pre["qu1"])))
                v = np.asfortranarray(0.05 * rng.standard_normal((N, N, pre["qv1"], pre["qv1"])))
                ut, vt = edg_rhs(u, v, 0.3, N, 1.0 / N, pre)
                et = energy_terms(u, v, ut, vt, pre, co, N)
                if fp["tau"] == 0 and fp["lambda_u"] == 0 and fp["lambda_v"] == 0:
                    assert et["DI"] == 0
                worst = max(worst, abs(et["dEdt"] + et["Dv"] + et["DI"]) / et["scale"])
                rise = max(rise, et["dEdt"] / et["scale"])
    assert worst < 1e-12 and rise < 1e-12, (worst, rise)


def test_oracle_interface_terms_of_the_initial_profile(oracle_lib):
    """test/runtests.jl:760-784 on the oracle (see the GPU test of the same name)."""
    from oracle.rhs import edg_rhs
    from reference_properties import lin_profile, project_u
    from test_host import Step
    z0 = lambda x, y: 0.0   # noqa: E731
    N, h = 8, 1.0 / 8
    for c1, c2, ip in ((1.0, 0.5, lin_profile(0.0, 1.0)), (0.8, 0.8, lin_profile(1.0, 0.0))):
        coef = oc.Coefficients(Step(1, 0.5, c1, c2), z0, z0, Step(1, 0.5, 1e-3 * c1 ** 2, 1e-3 * c2 ** 2), z0, z0, z0)
        for flux in ("upwind", "central", "alternating"):
            for q in (1, 3):
                kw = dict(coefficients=coef, boundary="wall", flux=flux)
                pI, _ = precompute(q, N, mode="initial_value", initial_profile=ip, **kw)
                pS, _ = precompute(q, N, mode="source", source=oc.GaussianSource(amplitude=0.0), **kw)
                assert pI["one_sided"]
                zv = np.zeros((N, N, pI["qv1"], pI["qv1"]), order="F")
                rI = edg_rhs(np.zeros((N, N, pI["qu1"], pI["qu1"]), order="F"), zv, 0.3, N, h, pI)
                rS = edg_rhs(project_u(ip["u0"], pS, N), zv, 0.3, N, h, pS)
                assert np.max(np.abs(rI[1] - rS[1])) <= 1e-11 * np.max(np.abs(rS[1]))
                assert np.max(np.abs(rI[0] - rS[0])) <= 1e-11


def test_oracle_two_layer_convergence(oracle_lib):
    """test/runtests.jl:816-823 on the oracle (see the GPU test of the same name)."""
    import math

    from reference_properties import two_layer_error
    e8 = two_layer_error(solve, oc.Coefficients, 2, 8, 0.5, "upwind", "x")
    e16 = two_layer_error(solve, oc.Coefficients, 2, 16, 0.5, "upwind", "x")
    assert math.log2(e8 / e16) > 1.8
    assert two_layer_error(solve, oc.Coefficients, 2, 16, 0.5, "upwind", "y") == pytest.approx(e16, rel=1e-10)
    c8 = two_layer_error(solve, oc.Coefficients, 2, 8, 0.5, "central", "x")
    c16 = two_layer_error(solve, oc.Coefficients, 2, 16, 0.5, "central", "x")
    assert math.log2(c8 / c16) > 0.9
