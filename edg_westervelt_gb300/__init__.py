"""edg_westervelt_gb300: the right-hand side and RK4 hot path of WesterveltEDG.jl on GB300.

A GPU (sm_103a, FP64) drop-in for the reference's ``Workspace``,
``edg_rhs!`` and ``rk4_step!`` behind its public surface. The kernels live in
``csrc/`` and are reached through the C ABI of ``include/wedg.h``
(``_build/libwedg.so``); this package is the host side, with the reference's
names (``edg_rhs_`` / ``rk4_step_`` stand for Julia's ``edg_rhs!`` /
``rk4_step!``) and argument meanings.
"""
from .errors import ArgumentErrorException, DimensionMismatch, ErrorException
from .coefficients import (Coefficients, GaussianSource, cell_coefficients, constant_coefficients, flux_parameters,
                           paper_coefficients, replace_coefficients)
from .precompute import precompute
from .quadrature import GaussQCofs, GradJacobiP, JacobiP
from .solver import difference_norms, misfit, misfit_gradient, misfit_gradients, piecewise_coefficients, solve
from .workspace import (Batch, Workspace, edg_rhs, edg_rhs_, rk4_adjoint_forward_many,
                        rk4_adjoint_reverse_many, rk4_step, rk4_step_)

__all__ = ["solve", "precompute", "edg_rhs", "edg_rhs_", "rk4_step", "rk4_step_", "Workspace", "Batch",
           "difference_norms", "flux_parameters", "GaussianSource", "Coefficients", "paper_coefficients",
           "replace_coefficients", "constant_coefficients", "JacobiP", "GradJacobiP", "GaussQCofs",
           "ErrorException", "DimensionMismatch", "ArgumentErrorException", "misfit", "misfit_gradient", "misfit_gradients",
           "piecewise_coefficients", "cell_coefficients", "rk4_adjoint_forward_many", "rk4_adjoint_reverse_many"]
