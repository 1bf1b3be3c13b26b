"""PDE coefficients c, alpha, beta (oracle). Test infrastructure only.

Restates ``src/coefficients.jl`` and ``GaussianSource`` / ``flux_parameters`` /
the boundary-side table of ``src/solver.jl:16-86``. Coefficient functions are
callables ``f(x, y)``; they are evaluated point by point, as the reference
does, so they may be plain Python scalar functions.
"""
import math
from dataclasses import dataclass


@dataclass
class Coefficients:
    c: object
    c_x: object
    c_y: object
    alpha: object
    alpha_x: object
    alpha_y: object
    beta: object


def paper_coefficients():
    """Section 5.1 coefficients (src/coefficients.jl:47-55)."""
    pi = math.pi
    return Coefficients(
        lambda x, y: 1 + 0.1 * math.cos(pi * x) * math.cos(pi * y),
        lambda x, y: -0.1 * pi * math.sin(pi * x) * math.cos(pi * y),
        lambda x, y: -0.1 * pi * math.cos(pi * x) * math.sin(pi * y),
        lambda x, y: 1e-5 + 1e-6 * math.cos(pi * x) * math.cos(pi * y),
        lambda x, y: -1e-6 * pi * math.sin(pi * x) * math.cos(pi * y),
        lambda x, y: -1e-6 * pi * math.cos(pi * x) * math.sin(pi * y),
        lambda x, y: 1e-4 * (1 + 0.1 * math.sin(pi * x) * math.sin(pi * y)),
    )


def _const(val):
    return lambda x, y: val


def _zero(x, y):
    return 0.0


def replace_coefficients(coef, c=None, alpha=None, beta=None):
    """src/coefficients.jl:66-76."""
    return Coefficients(
        coef.c if c is None else _const(float(c)),
        coef.c_x if c is None else _zero,
        coef.c_y if c is None else _zero,
        coef.alpha if alpha is None else _const(float(alpha)),
        coef.alpha_x if alpha is None else _zero,
        coef.alpha_y if alpha is None else _zero,
        coef.beta if beta is None else _const(float(beta)),
    )


def constant_coefficients(c, alpha, beta):
    """src/coefficients.jl:83-84."""
    return replace_coefficients(paper_coefficients(), c=c, alpha=alpha, beta=beta)


@dataclass
class GaussianSource:
    """src/solver.jl:80-86."""
    x0: tuple = (0.15, 0.5)
    r0: float = 0.05
    amplitude: float = 1.0
    omega: float = 16 * math.pi
    Ts: float = 1.0


def flux_parameters(flux):
    """src/solver.jl:16-21."""
    if flux == "upwind":
        return dict(theta=1.0, tau=1.0, lambda_u=1.0, lambda_v=1.0)
    if flux == "alternating":
        return dict(theta=1.0, tau=0.0, lambda_u=0.0, lambda_v=0.0)
    if flux == "central":
        return dict(theta=0.5, tau=0.0, lambda_u=0.0, lambda_v=0.0)
    raise ValueError(f"unknown flux {flux} (expected :upwind, :alternating or :central)")


BOUNDARY_KINDS = ("absorbing_2beta", "absorbing", "dirichlet", "wall")


def boundary_side(kind, sigma, sigma_dirichlet, kappa):
    """Per-side parameters (src/solver.jl:39-45)."""
    if kind == "wall":
        return dict(kind=kind, gamma_abc=0.0, eta_abc=1.0, sigma=0.0, kb=1.0, kappa=kappa)
    g = 1.0 if kind == "dirichlet" else 1.0 / math.sqrt(2.0)
    return dict(kind=kind, gamma_abc=g, eta_abc=math.sqrt(1.0 - g ** 2),
                sigma=sigma_dirichlet if kind == "dirichlet" else sigma,
                kb=2.0 if kind == "absorbing_2beta" else 1.0, kappa=kappa)


def boundary_sides(boundary, sigma, sigma_dirichlet, kappa):
    """src/solver.jl:50-68: a kind for all sides or a dict with bot, top, lft, rgt."""
    names = ("bot", "top", "lft", "rgt")
    if isinstance(boundary, str):
        kinds = (boundary,) * 4
    else:
        if not (len(boundary) == 4 and set(boundary) == set(names)):
            raise ValueError("boundary must be a kind or a NamedTuple with the keys bot, top, lft, rgt")
        kinds = tuple(boundary[s] for s in names)
    for k in kinds:
        if k not in BOUNDARY_KINDS:
            raise ValueError(f"unknown boundary {k} (expected one of {BOUNDARY_KINDS})")
    if any(k in ("absorbing", "absorbing_2beta") for k in kinds) and not (-1.0 <= sigma <= 1.0):
        raise ValueError(f"absorbing sides need -1 ≤ sigma ≤ 1 (got {sigma})")
    if "dirichlet" in kinds and not (sigma_dirichlet >= 0.0):
        raise ValueError(f"Dirichlet sides need sigma_dirichlet ≥ 0 (got {sigma_dirichlet}; it defaults to sigma)")
    if not kappa >= 0.0:
        raise ValueError(f"kappa must be ≥ 0 (got {kappa})")
    return {s: boundary_side(k, sigma, sigma_dirichlet, kappa) for s, k in zip(names, kinds)}
