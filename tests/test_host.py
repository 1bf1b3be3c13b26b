"""Host side of the product on the CPU: quadrature, precompute, argument checks, the C ABI.

The product's ``precompute`` is compared array by array with the oracle's
restatement of src/solver.jl:341-770; the argument and face-value checks
mirror test/runtests.jl:359-366, 627-698 and 818-830.
"""
import math
import os
import subprocess

import numpy as np
import pytest

import edg_westervelt_gb300 as W
from edg_westervelt_gb300.precompute import precompute as ppre
from oracle import coefficients as oc
from oracle.precompute import precompute as opre
from oracle.quadrature import gauss_q_cofs, grad_jacobi_p, jacobi_p
from test_oracle import quadrant_coefficients

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_quadrature_matches_golub_welsch():
    for q in range(1, 14):
        xa, wa = W.GaussQCofs(q)
        xb, wb = gauss_q_cofs(q)
        assert np.max(np.abs(xa - xb)) < 2e-15 and np.max(np.abs(wa - wb)) < 2e-15, q
    x = np.linspace(-1, 1, 7)
    for n in range(8):
        assert np.max(np.abs(W.JacobiP(x, 0, 0, n) - jacobi_p(x, 0, 0, n))) < 1e-14
        assert np.max(np.abs(W.GradJacobiP(x, 0, 0, n) - grad_jacobi_p(x, 0, 0, n))) < 1e-13
    assert W.JacobiP(1.0, 0, 0, 3) == pytest.approx(math.sqrt(3.5))


def _cmp_pre(q, N, **kw):
    a, ga = opre(q, N, **kw)
    b, gb = ppre(q, N, **kw)
    for k, va in a.items():
        if isinstance(va, np.ndarray):
            vb = np.asarray(b[k])
            assert va.shape == vb.shape, k
            if va.size:
                scale = max(np.max(np.abs(va)), 1e-300)
                # values that are zero up to rounding (e.g. projections at N = 1) get an absolute floor
                assert np.max(np.abs(va - vb)) <= 1e-13 * scale + 1e-15, (k, np.max(np.abs(va - vb)) / scale)
        elif k in ("bc",):
            assert va == b[k]
        elif k != "source":
            assert va == b[k] or (isinstance(va, float) and math.isnan(va) and math.isnan(b[k])), k
    for k in ga:
        assert np.max(np.abs(ga[k] - gb[k])) <= 1e-13 * max(1.0, np.max(np.abs(ga[k]))), k


@pytest.mark.parametrize("q,N,kw", [
    (3, 6, {}),
    (1, 1, {}),
    (2, 3, dict(mixed=False, flux="central", boundary="wall", kappa=0.7)),
    (4, 5, dict(mode="initial_value", phase=(0.4, 0.3), boundary="dirichlet", sigma=0.3)),
    (6, 4, dict(mode="source", mixed=False, coefficients=oc.constant_coefficients(c=1.0, alpha=1e-6, beta=8.0),
                boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"), kappa=0.5)),
    (3, 4, dict(mode="source", coefficients=quadrant_coefficients(0.5, 0.5, smooth=True))),
    (3, 4, dict(mode="initial_value", coefficients=quadrant_coefficients(0.5, 0.5), phase=(0.4, 0.3),
                boundary=dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing"))),
    (5, 3, dict(flux_params=dict(theta=0.3, tau=0.7, lambda_u=0.4, lambda_v=0.9), mass_solver="cg")),
])
def test_precompute_matches_oracle(q, N, kw):
    _cmp_pre(q, N, **kw)


def test_precompute_initial_profile_default_equivalent():
    """test/runtests.jl:627-638: passing Φ explicitly reproduces the default data."""
    pi = math.pi
    prof = dict(u0=lambda x, y: np.cos(2 * pi * x) * np.sin(2 * pi * y),
                u0_x=lambda x, y: -2 * pi * np.sin(2 * pi * x) * np.sin(2 * pi * y),
                u0_y=lambda x, y: 2 * pi * np.cos(2 * pi * x) * np.cos(2 * pi * y),
                u0_xx=lambda x, y: -(2 * pi) ** 2 * np.cos(2 * pi * x) * np.sin(2 * pi * y),
                u0_yy=lambda x, y: -(2 * pi) ** 2 * np.cos(2 * pi * x) * np.sin(2 * pi * y))
    a, _ = ppre(3, 6, mode="initial_value")
    b, _ = ppre(3, 6, mode="initial_value", initial_profile=prof)
    for k in ("PiCdiv", "bcB_sp", "bcL_spx", "hJC", "vJC"):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-12 * max(1.0, np.max(np.abs(a[k]))), k
    with pytest.raises(W.ErrorException, match="initial_profile is only available"):
        ppre(2, 2, initial_profile=prof)


def test_argument_checks():
    """test/runtests.jl:359-366 and the mode / mass_solver checks of src/solver.jl:437-440."""
    for kw in (dict(boundary="dirichlet", sigma=-0.5), dict(boundary="dirichlet", sigma_dirichlet=-0.1),
               dict(boundary="absorbing", sigma=1.5), dict(boundary="wall", kappa=-1.0), dict(boundary="neumann"),
               dict(boundary=dict(bot="wall", top="wall", lft="wall")),
               dict(boundary=dict(bot="wall", top="wall", lft="wall", rgt="foo")), dict(mass_solver="lu"),
               dict(mode="nope")):
        # the reference's error(...) (an ErrorException); a ValueError for Python callers as well
        with pytest.raises(W.ErrorException):
            ppre(2, 2, **kw)
        with pytest.raises(ValueError):
            ppre(2, 2, **kw)
    with pytest.raises(W.ErrorException, match="unknown flux downwind"):
        W.flux_parameters("downwind")
    bc = ppre(2, 2, boundary=dict(bot="absorbing_2beta", top="dirichlet", lft="wall", rgt="absorbing"), sigma=0.3,
              sigma_dirichlet=0.6, kappa=0.7)[0]["bc"]
    assert (bc["bot"]["sigma"], bc["bot"]["kb"], bc["rgt"]["sigma"], bc["rgt"]["kb"]) == (0.3, 2.0, 0.3, 1.0)
    assert (bc["top"]["gamma_abc"], bc["top"]["sigma"], bc["lft"]["kind"], bc["lft"]["kappa"]) == (1.0, 0.6, "wall", 0.7)
    pre, _ = ppre(2, 2, boundary="dirichlet", sigma=0.3)
    assert pre["gamma_abc"] == 1.0 and pre["eta_abc"] == 0.0 and pre["sigma"] == 0.3


class Step:
    """test/runtests.jl:28-32: lo / hi across coordinate `d` = s, `on` on the line, `edge` at 0."""

    def __init__(self, d, s, lo, hi, on=None, edge=None):
        self.d, self.s, self.lo, self.hi = d, s, lo, hi
        self.on = hi if on is None else on
        self.edge = lo if edge is None else edge

    def __call__(self, x, y):
        t = x if self.d == 1 else y
        return self.edge if t == 0 else self.lo if t < self.s else self.on if t == self.s else self.hi


def _step_coef(c, beta=None):
    z0 = lambda x, y: 0.0   # noqa: E731
    return W.Coefficients(c, z0, z0, Step(1, 2.0, 1e-3, 1e-3), z0, z0, beta or Step(1, 2.0, 0.0, 0.0))


def test_face_values_and_jumps():
    """test/runtests.jl:644-698: continuous coefficients keep the point values bit for bit,
    a jump gives each side its own piece, boundary values are seen from inside."""
    pre, _ = ppre(2, 4)
    co = W.paper_coefficients()
    h = 0.25
    z, _ = W.GaussQCofs(3)
    for k in range(4):
        xf = (k * h + (k + 1) * h + h * z) / 2
        for jf in range(5):
            yf = np.full(3, jf * h)
            assert np.array_equal(pre["hc2"][:, jf, k], co.c(xf, yf) ** 2)
            assert np.array_equal(pre["hbf"][:, jf, k], co.beta(xf, yf))
    assert np.array_equal(pre["hc2m"], pre["hc2"]) and np.array_equal(pre["vafm"], pre["vaf"])
    assert not pre["one_sided"]
    for N, kf, cfun in ((4, 2, Step(1, 0.5, 1.0, 2.0)), (4, 2, Step(1, 0.5, 1.0, 2.0, on=1.0)),
                        (4, 2, Step(1, 0.5, 1.0, 2.0, on=7.0)), (10, 3, Step(1, 0.3, 1.0, 2.0)),
                        (10, 3, Step(1, 0.3, 1.0, 2.0, on=1.0))):
        pre, _ = ppre(2, N, mode="source", coefficients=_step_coef(cfun))
        rest = [i for i in range(N + 1) if i != kf]
        assert np.all(pre["vc2m"][:, :, kf] == 1.0) and np.all(pre["vc2"][:, :, kf] == 4.0)
        assert np.array_equal(pre["vc2m"][:, :, rest], pre["vc2"][:, :, rest]) and pre["one_sided"]
    pre, _ = ppre(2, 4, mode="source", coefficients=_step_coef(Step(1, 0.5, 1.0, 2.0, edge=2.0),
                                                                beta=Step(2, 2.0, 0.1, 0.1, edge=5.0)))
    assert np.all(pre["vc2"][:, :, 0] == 1.0) and np.all(pre["vcf"][:, :, 0] == 1.0) and np.all(pre["hbf"][:, 0, :] == 0.1)

    class Spike:
        def __init__(self, g):
            self.g = g

        def __call__(self, x, y):
            return self.g if x == 0.5 else 1.0 if x < 0.25 else 1.5

    for g in (1e8, math.inf, math.nan):
        pre, _ = ppre(2, 8, mode="source", coefficients=_step_coef(Spike(g)))
        assert np.all(pre["vc2m"][:, :, 2] == 1.0) and np.all(pre["vc2"][:, :, 2] == 2.25)
        assert np.all(pre["vc2m"][:, :, 4] == 2.25) and np.all(pre["vc2"][:, :, 4] == 2.25)
        assert np.all(np.isfinite(pre["vc2m"])) and np.all(np.isfinite(pre["vcf"])) and pre["one_sided"]
    # jumps of c or α are refused in :mms mode; β alone is not a jump
    co = quadrant_coefficients(0.5, 0.5, c=(1.0, 1.0, 1.0, 1.0), alpha=(1e-3, 1e-3, 2e-3, 2e-3))
    with pytest.raises(W.ErrorException, match="mode = :mms needs c and α continuous"):
        ppre(2, 6, coefficients=co)
    cb = quadrant_coefficients(0.5, 0.5, c=(1.0, 1.0, 1.0, 1.0), alpha=(1e-3, 1e-3, 1e-3, 1e-3))
    assert not ppre(2, 6, coefficients=cb)[0]["one_sided"]


def test_library_builds_and_exports_every_symbol():
    """libwedg.so builds for sm_103a and exports every entry point of include/wedg.h (no GPU call)."""
    from edg_westervelt_gb300 import _lib, build
    path = build.build()
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = _lib.exported_symbols()
    assert len(declared) >= 14
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    L = _lib.lib()
    assert L.wedg_version().decode().startswith("libwedg")
    assert L.wedg_status_string(3).decode() == "mass matrix not positive definite"


def test_oracle_library_builds():
    from oracle import rhs
    assert os.path.exists(rhs.build())
    assert rhs.max_threads() >= 1


def test_precompute_leaves_many_distinct_inverses_to_the_device():
    """inverses="device" (default): more than 64 distinct element stiffnesses are not inverted
    on the host (the GPU workspace does it); "host" inverts them as the reference does."""
    pre, _ = W.precompute(2, 9, mode="mms")                  # paper coefficients: 81 distinct matrices
    assert pre["Ainv_u"] is None
    pre_h, _ = W.precompute(2, 9, mode="mms", inverses="host")
    assert pre_h["Ainv_u"].shape == (9 * 10 // 2, 81)
    pre_c, _ = W.precompute(2, 9, mode="mms", coefficients=W.constant_coefficients(c=1.0, alpha=1e-4, beta=1.0))
    assert pre_c["Ainv_u"] is not None                        # one shared matrix: inverted on the host
    with pytest.raises(ValueError):
        W.precompute(2, 3, inverses="gpu")


def test_distinct_rows_matches_a_row_sort():
    """The grouping of equal element stiffnesses (precompute) against np.unique(axis=0): all
    rows equal, a few repeated rows, rows whose projection keys coincide although the rows
    differ (the row sort decides then), and the limit above which the device computes the
    inverses."""
    from edg_westervelt_gb300.precompute import _distinct_rows
    rng = np.random.default_rng(8)
    a = np.broadcast_to(rng.standard_normal(9), (50, 9)).copy()
    u, inv = _distinct_rows(a)
    assert u.shape == (1, 9) and np.array_equal(u[inv], a)
    for _ in range(20):
        rows = rng.standard_normal((int(rng.integers(2, 7)), 9))
        a = rows[rng.integers(0, rows.shape[0], 60)]
        u, inv = _distinct_rows(a)
        assert u.shape == np.unique(a, axis=0).shape and np.array_equal(u[inv], a)
    # two different rows with the same key: the key is a · r for a fixed r, so move along a
    # direction orthogonal to r
    r = np.random.default_rng(0).uniform(1.0, 2.0, 9)
    d = np.zeros(9)
    d[0], d[1] = r[1], -r[0]
    x = rng.standard_normal(9)
    a = np.stack([x, x + d, x, x + d])
    u, inv = _distinct_rows(a)
    assert u.shape[0] == 2 and np.array_equal(u[inv], a)
    assert _distinct_rows(rng.standard_normal((100, 4)), limit=64) == (None, None)
    u, inv = _distinct_rows(rng.standard_normal((10, 4)), limit=64)
    assert u.shape[0] == 10
