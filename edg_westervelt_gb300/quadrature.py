"""Orthonormal Jacobi/Legendre polynomials and Gauss-Legendre rules.

Mirrors the exported functions ``JacobiP``, ``GradJacobiP`` and ``GaussQCofs``
of WesterveltEDG.jl (src/quadrature.jl:11-66). The Gauss rule is computed by
Newton's method on the Legendre three-term recurrence (the reference uses the
Golub-Welsch eigenvalue method); both give the nodes and weights to rounding.
"""
import math

import numpy as np

from .errors import ArgumentErrorException


def JacobiP(x, alpha, beta, n):
    """Orthonormal Jacobi polynomial P_n^(alpha,beta) at x (src/quadrature.jl:11-35).

    With alpha = beta = 0 these are the L²(-1,1)-orthonormal Legendre
    polynomials of the modal basis.
    """
    scalar = np.ndim(x) == 0
    xp = np.atleast_1d(np.asarray(x, dtype=np.float64))
    g0 = (2.0 ** (alpha + beta + 1) / (alpha + beta + 1)
          * math.gamma(alpha + 1) * math.gamma(beta + 1) / math.gamma(alpha + beta + 1))
    p_prev = np.full(xp.shape, 1.0 / math.sqrt(g0))
    if n == 0:
        out = p_prev
    else:
        g1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * g0
        p = ((alpha + beta + 2) * xp / 2 + (alpha - beta) / 2) / math.sqrt(g1)
        aold = 2 / (2 + alpha + beta) * math.sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3))
        for i in range(1, n):
            h1 = 2 * i + alpha + beta
            anew = 2 / (h1 + 2) * math.sqrt((i + 1) * (i + 1 + alpha + beta)
                                            * (i + 1 + alpha) * (i + 1 + beta) / (h1 + 1) / (h1 + 3))
            bnew = -(alpha ** 2 - beta ** 2) / h1 / (h1 + 2)
            p_prev, p = p, (1 / anew) * (-aold * p_prev + (xp - bnew) * p)
            aold = anew
        out = p
    return float(out[0]) if scalar else out


def GradJacobiP(x, alpha, beta, n):
    """First derivative of the orthonormal Jacobi polynomial (src/quadrature.jl:44-47)."""
    if n == 0:
        return 0.0 if np.ndim(x) == 0 else np.zeros(np.size(x))
    return math.sqrt(n * (n + alpha + beta + 1)) * JacobiP(x, alpha + 1, beta + 1, n - 1)


def _legendre_and_derivative(n, x):
    """Classical Legendre P_n(x) and P_n'(x) by the three-term recurrence."""
    p0 = np.ones_like(x)
    p1 = x.copy()
    if n == 0:
        return p0, np.zeros_like(x)
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    dp = n * (x * p1 - p0) / (x * x - 1.0)
    return p1, dp


def GaussQCofs(q):
    """Nodes and weights of the q-point Gauss-Legendre rule on [-1, 1], ascending
    (src/quadrature.jl:57-66 computes the same rule by Golub-Welsch)."""
    if q < 1:
        raise ArgumentErrorException("GaussQCofs needs q ≥ 1")
    k = np.arange(1, q + 1, dtype=np.float64)
    x = -np.cos(np.pi * (k - 0.25) / (q + 0.5))      # initial guesses, ascending
    for _ in range(100):
        p, dp = _legendre_and_derivative(q, x)
        dx = p / dp
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    p, dp = _legendre_and_derivative(q, x)
    w = 2.0 / ((1.0 - x * x) * dp * dp)
    # exact symmetry of the rule
    x = 0.5 * (x - x[::-1])
    w = 0.5 * (w + w[::-1])
    return x, w
