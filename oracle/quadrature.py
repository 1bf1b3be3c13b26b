"""Orthonormal Jacobi/Legendre polynomials and Gauss-Legendre rules (oracle).

Test infrastructure only. Restates ``src/quadrature.jl`` of WesterveltEDG.jl.
"""
import math

import numpy as np


def jacobi_p(x, alpha, beta, n):
    """Orthonormal Jacobi polynomial P_n^(alpha,beta) at x (src/quadrature.jl:11-35)."""
    scalar = np.ndim(x) == 0
    xp = np.atleast_1d(np.asarray(x, dtype=np.float64))
    pl = np.zeros((n + 1, xp.size))
    gamma0 = (2.0 ** (alpha + beta + 1) / (alpha + beta + 1)
              * math.gamma(alpha + 1) * math.gamma(beta + 1) / math.gamma(alpha + beta + 1))
    pl[0, :] = 1.0 / math.sqrt(gamma0)
    if n == 0:
        out = pl[0]
    else:
        gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0
        pl[1, :] = ((alpha + beta + 2) * xp / 2 + (alpha - beta) / 2) / math.sqrt(gamma1)
        if n == 1:
            out = pl[1]
        else:
            aold = 2 / (2 + alpha + beta) * math.sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3))
            for i in range(1, n):
                h1 = 2 * i + alpha + beta
                anew = 2 / (h1 + 2) * math.sqrt((i + 1) * (i + 1 + alpha + beta)
                                                * (i + 1 + alpha) * (i + 1 + beta) / (h1 + 1) / (h1 + 3))
                bnew = -(alpha ** 2 - beta ** 2) / h1 / (h1 + 2)
                pl[i + 1, :] = (1 / anew) * (-aold * pl[i - 1, :] + (xp - bnew) * pl[i, :])
                aold = anew
            out = pl[n]
    return float(out[0]) if scalar else out.copy()


def grad_jacobi_p(x, alpha, beta, n):
    """Derivative of the orthonormal Jacobi polynomial (src/quadrature.jl:44-47)."""
    if n == 0:
        return 0.0 if np.ndim(x) == 0 else np.zeros(np.size(x))
    return math.sqrt(n * (n + alpha + beta + 1)) * jacobi_p(x, alpha + 1, beta + 1, n - 1)


def gauss_q_cofs(q):
    """Nodes and weights of the q-point Gauss-Legendre rule, Golub-Welsch (src/quadrature.jl:57-66)."""
    kk = np.arange(1, q, dtype=np.float64) ** 2
    b = np.sqrt(kk / (4 * kk - 1))
    jac = np.diag(b, 1) + np.diag(b, -1)
    vals, vecs = np.linalg.eigh(jac)
    w = 2 * vecs[0, :] ** 2
    idx = np.argsort(vals)
    return vals[idx].copy(), w[idx].copy()
