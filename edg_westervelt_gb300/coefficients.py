"""Coefficients, sources and flux/boundary parameters.

Mirrors src/coefficients.jl and the parameter helpers of src/solver.jl:16-86
of WesterveltEDG.jl. Coefficient functions are callables ``f(x, y)``; they
may accept numpy arrays (evaluated vectorised) or only scalars (evaluated
point by point).
"""
import math
from dataclasses import dataclass

import numpy as np

from .errors import ArgumentErrorException


@dataclass
class Coefficients:
    """Sound speed c, diffusivity alpha, nonlinearity beta and the first
    derivatives of c and alpha as functions (x, y) -> value
    (src/coefficients.jl:28-36). They may jump across mesh lines."""
    c: object
    c_x: object
    c_y: object
    alpha: object
    alpha_x: object
    alpha_y: object
    beta: object


def paper_coefficients():
    """The coefficients of the convergence test (src/coefficients.jl:47-55):
    c = 1 + 0.1 cos(πx) cos(πy), α = 1e-5 + 1e-6 cos(πx) cos(πy),
    β = 1e-4 (1 + 0.1 sin(πx) sin(πy))."""
    pi = math.pi
    return Coefficients(
        lambda x, y: 1 + 0.1 * np.cos(pi * x) * np.cos(pi * y),
        lambda x, y: -0.1 * pi * np.sin(pi * x) * np.cos(pi * y),
        lambda x, y: -0.1 * pi * np.cos(pi * x) * np.sin(pi * y),
        lambda x, y: 1e-5 + 1e-6 * np.cos(pi * x) * np.cos(pi * y),
        lambda x, y: -1e-6 * pi * np.sin(pi * x) * np.cos(pi * y),
        lambda x, y: -1e-6 * pi * np.cos(pi * x) * np.sin(pi * y),
        lambda x, y: 1e-4 * (1 + 0.1 * np.sin(pi * x) * np.sin(pi * y)),
    )


class _Const:
    def __init__(self, val):
        self.val = float(val)

    def __call__(self, x, y):
        return np.full(np.shape(x), self.val) if np.ndim(x) else self.val


def _zero(x, y):
    return np.zeros(np.shape(x)) if np.ndim(x) else 0.0


class _Cells:
    """A function constant on the cells of an m × n grid of (0,1)²: tab[row, column], row from y,
    column from x (the point on a cell boundary belongs to the cell above / right of it)."""

    def __init__(self, tab):
        self.tab = np.ascontiguousarray(tab, dtype=np.float64)
        self.m, self.n = self.tab.shape

    def __call__(self, x, y):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        return self.tab[np.clip(np.floor(self.m * y).astype(int), 0, self.m - 1),
                        np.clip(np.floor(self.n * x).astype(int), 0, self.n - 1)]


def cell_coefficients(c, alpha, beta):
    """Coefficients constant on the cells of an m × n grid of (0,1)²: c, alpha, beta are (m, n)
    arrays indexed [row (y), column (x)] of c, α and β; the derivatives of c and α vanish inside
    the cells. A GPU workspace built from point values looks these tables up on the device."""
    return Coefficients(_Cells(c), _zero, _zero, _Cells(alpha), _zero, _zero, _Cells(beta))


def replace_coefficients(coef, c=None, alpha=None, beta=None):
    """Copy of coef with every coefficient given as a number replaced by that
    constant and its derivatives by zero (src/coefficients.jl:66-76)."""
    return Coefficients(
        coef.c if c is None else _Const(c),
        coef.c_x if c is None else _zero,
        coef.c_y if c is None else _zero,
        coef.alpha if alpha is None else _Const(alpha),
        coef.alpha_x if alpha is None else _zero,
        coef.alpha_y if alpha is None else _zero,
        coef.beta if beta is None else _Const(beta),
    )


def constant_coefficients(*, c, alpha, beta):
    """Constant coefficients (src/coefficients.jl:83-84)."""
    return replace_coefficients(paper_coefficients(), c=c, alpha=alpha, beta=beta)


@dataclass
class GaussianSource:
    """f(t, x) = amplitude exp(-|x - x0|²/r0²) sin(ωt) sin²(πt/Ts) for t ≤ Ts, 0 after
    (src/solver.jl:70-86)."""
    x0: tuple = (0.15, 0.5)
    r0: float = 0.05
    amplitude: float = 1.0
    omega: float = 16 * math.pi
    Ts: float = 1.0


def flux_parameters(flux):
    """(theta, tau, lambda_u, lambda_v) of :upwind, :alternating, :central (src/solver.jl:16-21)."""
    flux = _sym(flux)
    if flux == "upwind":
        return dict(theta=1.0, tau=1.0, lambda_u=1.0, lambda_v=1.0)
    if flux == "alternating":
        return dict(theta=1.0, tau=0.0, lambda_u=0.0, lambda_v=0.0)
    if flux == "central":
        return dict(theta=0.5, tau=0.0, lambda_u=0.0, lambda_v=0.0)
    raise ArgumentErrorException(f"unknown flux {flux} (expected :upwind, :alternating or :central)")


BOUNDARY_KINDS = ("absorbing_2beta", "absorbing", "dirichlet", "wall")
SIDES = ("bot", "top", "lft", "rgt")


def _sym(s):
    """Accept 'upwind' and ':upwind' alike."""
    return s[1:] if isinstance(s, str) and s.startswith(":") else s


def boundary_side(kind, sigma, sigma_dirichlet, kappa):
    """Flux parameters of one side (src/solver.jl:39-45)."""
    kind = _sym(kind)
    if kind == "wall":
        return dict(kind=kind, gamma_abc=0.0, eta_abc=1.0, sigma=0.0, kb=1.0, kappa=kappa)
    g = 1.0 if kind == "dirichlet" else 1.0 / math.sqrt(2.0)
    return dict(kind=kind, gamma_abc=g, eta_abc=math.sqrt(1.0 - g ** 2),
                sigma=sigma_dirichlet if kind == "dirichlet" else sigma,
                kb=2.0 if kind == "absorbing_2beta" else 1.0, kappa=kappa)


def boundary_sides(boundary, sigma, sigma_dirichlet, kappa):
    """Per-side parameters from a kind or a mapping with the keys bot, top, lft, rgt
    (src/solver.jl:50-68), with the reference's argument checks."""
    if isinstance(boundary, str):
        kinds = (_sym(boundary),) * 4
    else:
        if not (len(boundary) == 4 and set(boundary) == set(SIDES)):
            raise ArgumentErrorException("boundary must be a kind or a NamedTuple with the keys bot, top, lft, rgt")
        kinds = tuple(_sym(boundary[s]) for s in SIDES)
    for k in kinds:
        if k not in BOUNDARY_KINDS:
            raise ArgumentErrorException(f"unknown boundary {k} (expected one of {BOUNDARY_KINDS})")
    if any(k in ("absorbing", "absorbing_2beta") for k in kinds) and not (-1.0 <= sigma <= 1.0):
        raise ArgumentErrorException(f"absorbing sides need -1 ≤ sigma ≤ 1 (got {sigma})")
    if "dirichlet" in kinds and not (sigma_dirichlet >= 0.0):
        raise ArgumentErrorException(f"Dirichlet sides need sigma_dirichlet ≥ 0 (got {sigma_dirichlet}; it defaults to sigma)")
    if not kappa >= 0.0:
        raise ArgumentErrorException(f"kappa must be ≥ 0 (got {kappa})")
    return {s: boundary_side(k, sigma, sigma_dirichlet, kappa) for s, k in zip(SIDES, kinds)}
